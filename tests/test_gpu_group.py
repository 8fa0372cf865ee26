"""Lockstep group cycles (mge_group_cycle_async / _poll): one launch per
phase over the blocks of many cases of different sizes, or, on the small
levels, one persistent cooperative launch per update of every case.

Each case of a group runs the same phase bodies in the same order as its
own per-phase cycle, so the group's results must equal the cases' own
cycles bit for bit: the same residual every cycle and the same state at the
end of the full-multigrid sequence.  The single cycles are pinned to the
per-phase launch form with global-memory line sweeps (MGE_TUNE_PLAN, and
MGE_COOP_MAX_CELLS=0), the form the group runs.
"""
import ctypes as C
import os

import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import serving as SV

pytestmark = pytest.mark.gpu


def _cases(precision):
    reqs = [SV.Request(0, "ellipsoid", 32, 0.5, 3.0, semi=(1.0, 0.7, 0.5), precision=precision),
            SV.Request(1, "sphere", 40, 0.4, 0.0, precision=precision),
            SV.Request(2, "ellipsoid", 48, 0.7, -2.0, semi=(0.6, 1.2, 0.8), precision=precision)]
    out = []
    for r in reqs:
        c = SV.build_case(r)
        for L in range(c.prm.nlevel - 1):
            c.prm.mcyc[L] = 2
        c.prm.mcyc[c.prm.nlevel - 1] = 3
        out.append(c)
    return out


def _open(cases, monkeypatch):
    from code_mge_gb300.runtime import Cycle
    monkeypatch.setenv("MGE_TUNE_PLAN", "1:0000,2:0000,3:0000")
    monkeypatch.setenv("MGE_COOP_MAX_CELLS", "0")
    try:
        return [Cycle(c) for c in cases]
    finally:
        monkeypatch.delenv("MGE_TUNE_PLAN")
        monkeypatch.delenv("MGE_COOP_MAX_CELLS")


def _fmg_single(lib, cyc, case):
    hist = []
    nl = case.prm.nlevel
    for mlvl in range(1, nl + 1):
        for ncyc in range(1, case.prm.mcyc[mlvl - 1] + 1):
            hist.append(cyc.cycle(mlvl, ncyc=ncyc))
        if mlvl < nl:
            assert lib.mge_prolong_async(cyc.ctx, mlvl) == 0
    return hist


def _fmg_group(lib, cycs, cases):
    n = len(cycs)
    arr = (C.c_void_p * n)(*[c.ctx.value for c in cycs])
    res = (C.c_double * n)()
    rcs = (C.c_int * n)()
    hist = [[] for _ in range(n)]
    nl = cases[0].prm.nlevel
    for mlvl in range(1, nl + 1):
        for ncyc in range(1, cases[0].prm.mcyc[mlvl - 1] + 1):
            assert lib.mge_group_cycle_async(arr, n, mlvl) == 0, lib.mge_last_error(cycs[0].ctx)
            rc = 1
            while rc == 1:
                rc = lib.mge_group_cycle_poll(arr, n, ncyc, res, rcs)
            assert rc == 0 and list(rcs) == [0] * n
            for q in range(n):
                hist[q].append(res[q])
        if mlvl < nl:
            for c in cycs:
                assert lib.mge_prolong_async(c.ctx, mlvl) == 0
    return hist


@pytest.mark.parametrize("coop", ["0", "1000000000"])  # per-phase launches, or one persistent launch per update
@pytest.mark.parametrize("precision", [A.MGE_PREC_FP64, A.MGE_PREC_MIXED])
def test_group_cycles_equal_the_cases_own(gpulib, monkeypatch, precision, coop):
    monkeypatch.setenv("MGE_GROUP_COOP_MAX_CELLS", coop)
    cases = _cases(precision)
    assert len({c.prm.nlevel for c in cases}) == 1
    single = _open(cases, monkeypatch)
    group = _open(cases, monkeypatch)
    hs = [_fmg_single(gpulib, c, k) for c, k in zip(single, cases)]
    hg = _fmg_group(gpulib, group, cases)
    nl = cases[0].prm.nlevel
    for q in range(len(cases)):
        assert hg[q] == hs[q], (q, hg[q], hs[q])
        for L in range(1, nl + 1):
            assert np.array_equal(group[q].field("w", L), single[q].field("w", L)), (q, L)
    # the group cycle is one graph whatever the number of cases
    assert all(h > 0 for h in hg[0])
    for c in single + group:
        c.close()


def test_group_refuses_cases_that_cannot_run_together(gpulib, monkeypatch):
    a, b = _cases(A.MGE_PREC_FP64)[:2]
    b.prm.cfl = a.prm.cfl * 0.5
    cycs = _open([a, b], monkeypatch)
    arr = (C.c_void_p * 2)(*[c.ctx.value for c in cycs])
    assert gpulib.mge_group_cycle_async(arr, 2, 1) == A.MGE_EBADCFG
    assert b"differ" in gpulib.mge_last_error(cycs[0].ctx)
    # nothing is in flight: each case still cycles alone
    assert np.isfinite(cycs[1].cycle(1, ncyc=1))
    for c in cycs:
        c.close()


def test_a_stop_in_one_case_leaves_the_others_of_the_group(gpulib, monkeypatch):
    """A case whose state goes bad stops with the reference's code in its own
    slot of the group's poll; the other cases' cycles are unaffected."""
    cases = _cases(A.MGE_PREC_FP64)
    single = _open(cases, monkeypatch)
    group = _open(cases, monkeypatch)
    L = 1
    for c in single + group:
        c.cycle(L, ncyc=1)
    w = group[1].field("w", L).copy()
    w[0, 4, 4, 4] = -abs(w[0, 4, 4, 4])  # a negative density: timestep.f90:45-48
    group[1].upload(w, L)
    n = len(group)
    arr = (C.c_void_p * n)(*[c.ctx.value for c in group])
    res = (C.c_double * n)()
    rcs = (C.c_int * n)()
    assert gpulib.mge_group_cycle_async(arr, n, L) == 0
    rc = 1
    while rc == 1:
        rc = gpulib.mge_group_cycle_poll(arr, n, 2, res, rcs)
    assert rc == 0
    assert list(rcs) == [0, A.MGE_ENEGPRESS, 0]
    assert b"timestep.f90:45-48" in gpulib.mge_last_error(group[1].ctx)
    for q in (0, 2):
        assert res[q] == single[q].cycle(L, ncyc=2)
        assert np.array_equal(group[q].field("w", L), single[q].field("w", L))
    for c in single + group:
        c.close()
