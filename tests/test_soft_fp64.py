"""The integer-pipe binary64 multiply, add and divide (soft_fp64.cuh)
against the host's IEEE-754 arithmetic, bit for bit, on edge values and 8
million random operand pairs (CPU; the GPU builds of the same functions are checked in
test_gpu_soft_fp64.py)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "code_mge_gb300", "csrc")


def test_soft_fp64_matches_the_host(tmp_path):
    exe = tmp_path / "soft_fp64_check"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-I", CSRC,
                           os.path.join(HERE, "soft_fp64_check.cpp"), "-o", str(exe)])
    r = subprocess.run([str(exe), "8000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "mismatches 0" in r.stdout
