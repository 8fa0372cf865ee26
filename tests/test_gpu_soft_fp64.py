"""The device build of the integer-pipe binary64 multiply, add and divide
(soft_fp64.cuh) against the GB300's FP64 hardware, bit for bit, on 8 x 2^26
operand pairs (the host build is checked in test_soft_fp64.py)."""
import os
import subprocess

import pytest

from code_mge_gb300 import build as B

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "code_mge_gb300", "csrc")


def test_soft_fp64_matches_the_fp64_hardware(tmp_path):
    exe = str(tmp_path / "soft_fp64_check")
    subprocess.run([B._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-I", CSRC,
                    "-o", exe, os.path.join(HERE, "soft_fp64_check.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0 " in r.stdout
