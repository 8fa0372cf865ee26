"""The reference's restart text (wsolut.f90:49-92, rsolut.f90:1-41) as the
library writes and reads it: "(5I5)" header of code, low(1:4), upp(1:4) and
"(5f16.7)" values.  Pure host functions: these tests need no GPU."""
import ctypes as C

import numpy as np
import pytest

from code_mge_gb300 import _abi as A


def _fmt(lib, code, ib, jb, kb, w):
    w = np.ascontiguousarray(w, dtype=np.float64)
    pw = w.ctypes.data_as(C.POINTER(C.c_double))
    need = lib.mge_restart_format(code, ib, jb, kb, pw, None, 0)
    buf = C.create_string_buffer(need + 1)
    assert lib.mge_restart_format(code, ib, jb, kb, pw, buf, need + 1) == need
    return buf.raw[:need].decode()


def _parse(lib, text, code, ib, jb, kb):
    w = np.zeros(5 * (ib + 1) * (jb + 1) * (kb + 1))
    raw = text.encode()
    used = lib.mge_restart_parse(raw, len(raw), code, ib, jb, kb, w.ctypes.data_as(C.POINTER(C.c_double)))
    return used, w


def test_layout_follows_the_fortran_formats(gpulib):
    ib, jb, kb = 2, 1, 0
    w = np.zeros(5 * 3 * 2 * 1)
    w[:8] = [1.0, -0.5, 12345678.9, 123456789.0, -1234567.5, 4e-8, -4e-8, float("nan")]
    lines = _fmt(gpulib, 7, ib, jb, kb, w).split("\n")
    assert lines[0] == "    7    0    0    0    1"
    assert lines[1] == "    2    1    0    5"
    assert len(lines) == 2 + 6 + 1 and lines[-1] == ""          # 30 values, 5 per line
    assert all(len(x) == 80 for x in lines[2:-1])
    f = [lines[2][16 * q:16 * q + 16] for q in range(5)] + [lines[3][16 * q:16 * q + 16] for q in range(3)]
    assert f[0] == "       1.0000000"
    assert f[1] == "      -0.5000000"
    assert f[2] == "12345678.9000000"
    assert f[3] == "*" * 16                                      # needs 17 columns
    assert f[4] == "-1234567.5000000"
    assert f[5] == "       0.0000000"
    assert f[6] == "      -0.0000000"
    assert f[7] == "             NaN"


def test_round_trip_keeps_seven_decimals(gpulib):
    rng = np.random.default_rng(3)
    ib, jb, kb = 5, 4, 3
    w = rng.normal(0.0, 3.0, 5 * 6 * 5 * 4) * rng.choice([1e-6, 1.0, 1e3], 5 * 6 * 5 * 4)
    text = _fmt(gpulib, 12, ib, jb, kb, w)
    used, back = _parse(gpulib, text, 12, ib, jb, kb)
    assert used == len(text)
    want = np.array([float("%.7f" % x) for x in w])
    assert np.array_equal(back, want)


def test_two_blocks_parse_in_sequence(gpulib):
    a = np.arange(5 * 2 * 2 * 2, dtype=np.float64) * 0.25
    b = -np.arange(5 * 3 * 2 * 2, dtype=np.float64) * 0.125
    text = _fmt(gpulib, 1, 1, 1, 1, a) + _fmt(gpulib, 2, 2, 1, 1, b)
    used, ra = _parse(gpulib, text, 1, 1, 1, 1)
    assert np.array_equal(ra, a)
    used2, rb = _parse(gpulib, text[used:], 2, 2, 1, 1)
    assert used + used2 == len(text) and np.array_equal(rb, b)


@pytest.mark.parametrize("code,dims", [(8, (2, 1, 0)), (7, (3, 1, 0)), (7, (2, 2, 0)), (7, (2, 1, 1))])
def test_inconsistent_block_is_rejected(gpulib, code, dims):
    # rsolut.f90:27-32 stops when the code or the upper bounds differ
    text = _fmt(gpulib, 7, 2, 1, 0, np.ones(30))
    used, _ = _parse(gpulib, text, code, *dims)
    assert used == A.MGE_EBADCFG


def test_unreadable_field_is_rejected(gpulib):
    w = np.ones(30)
    w[4] = 1e12                                                  # written as asterisks
    text = _fmt(gpulib, 7, 2, 1, 0, w)
    used, _ = _parse(gpulib, text, 7, 2, 1, 0)
    assert used == A.MGE_EBADCFG
