"""The integer-pipe binary64 operations the stage kernels use (exact_ops.cuh)
return exactly what the FP64 operations they replace return: x*2, x*0.5,
and max / > of non-negative doubles, on 2^26 bit patterns including zeros,
subnormals, binade edges, inf and NaN."""
import os
import subprocess

import pytest

from code_mge_gb300 import build as B

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_exact_ops_match_fp64(tmp_path):
    exe = str(tmp_path / "exact_ops_check")
    subprocess.run([B._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-o", exe,
                    os.path.join(HERE, "exact_ops_check.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0 " in r.stdout


def test_fast_powers_stay_within_four_ulp_of_pow(tmp_path):
    # x^(5/2) and x^(7/5) of the far-field boundary (fast_pow.cuh) against
    # CUDA's pow at the double exponents 1/(gamma-1) and gamma, gamma = 1.4
    exe = str(tmp_path / "fast_pow_check")
    subprocess.run([B._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-o", exe,
                    os.path.join(HERE, "fast_pow_check.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
