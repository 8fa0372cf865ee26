"""Cases that stop converging: the GPU and the oracle side by side.

Some ellipsoids of the batched sweep (seed 20261203) never reach a 1e-8
residual drop in FP64, and the 192^3 sphere of the benchmark never reaches a
1e-10 drop.  These tests run them in the plain FP64 form on the GPU and
compare with the oracle over the same cycles: the residual histories agree
and stop falling at the same place, so the stall is the reference
algorithm's, not the GPU path's.
- request 10, a 32^3 ellipsoid at M = 0.72: the residual stops falling after
  a drop of about 55 and then wanders between 2e-2 and 9e-2 of its first
  value; the two histories agree to 1e-12 over 300 cycles;
- request 3, a 48^3 ellipsoid at M = 0.22: the residual levels off near a
  1e6 drop and then wanders between 9e-7 and 5e-6 of its first value; the
  two histories agree to 1e-8 over 700 cycles (their relative difference
  grows as the residual falls, from rounding in the far field's powers and
  the norm's summation order: 2e-12 at a 1e3 drop, 2e-9 on the plateau).
"""
import os

import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import serving as SV

pytestmark = pytest.mark.gpu


def _histories(rid, cycles):
    from code_mge_gb300.runtime import Cycle
    from oracle import oracle as O
    r = [q for q in SV.batched_sweep_requests(64, precision=A.MGE_PREC_FP64, max_cycles=cycles) if q.rid == rid][0]
    case = SV.build_case(r)
    case.prm.conv_drop = 1e30  # run every cycle
    g = Cycle(case)
    hg, ng, _ = g.solve()
    g.close()
    before = O.load().mgeo_get_threads()
    O.set_threads(os.cpu_count() or 1)
    try:
        o = O.OracleCycle(case)
        ho, no, _ = o.solve()
        o.close()
    finally:
        O.set_threads(before)
    assert ng == no == cycles
    return r, hg, ho


def test_transonic_ellipsoid_stalls_in_both():
    r, hg, ho = _histories(10, 300)
    assert r.n == 32 and r.mach > 0.7
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-12
    for h in (hg, ho):
        drop = h[0] / h
        assert drop.max() < 100.0             # never a 1e2 drop
        assert h[-100:].min() / h[0] > 1e-2   # still wandering at the end


def test_low_mach_ellipsoid_levels_off_in_both():
    r, hg, ho = _histories(3, 700)
    assert r.n == 48 and r.mach < 0.3
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-8
    for h in (hg, ho):
        tail = h[-200:] / h[0]
        assert 1e5 < (h[0] / h).max() < 1e7          # a 1e6 drop at best
        assert tail.min() > 5e-7 and tail.max() < 1e-5  # the plateau, not convergence


def test_sphere_192_settles_into_the_same_orbit():
    """The 192^3 sphere (4-level W-cycle, FMG with 50 cycles on each coarse
    level) falls by about 4.6e7 and then cycles: the residual decays smoothly
    to about 8e-11 and jumps back to about 2.6e-9, every 18 to 20 cycles.  The
    oracle's 700 cycles take hours on the host, so they come from a committed
    fixture (tests/golden/make_sphere192_history.py).  Against it the GPU's
    history differs by at most 1e-12 of the first residual in any cycle, jumps
    back at the same cycles and spans the same band."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_sphere192_history as M
    from code_mge_gb300.runtime import Cycle
    ho = np.load(os.path.join(os.path.dirname(M.__file__), "sphere192_fp64_history.npy"))
    g = Cycle(M.case())
    try:
        hg, n, _ = g.solve(max_cycles_total=M.CYCLES, hist_len=M.CYCLES)
    finally:
        g.close()
    assert n == M.CYCLES == len(ho)
    assert np.max(np.abs(hg - ho)) <= 1e-12 * ho[0]
    bursts = [np.flatnonzero(h[1:] / h[:-1] > 5.0) + 1 for h in (hg, ho)]
    assert np.array_equal(bursts[0], bursts[1])
    assert np.sum(bursts[0] >= 500) >= 8
    for h in (hg, ho):
        assert 1e7 < h[0] / h.min() < 1e8          # never the 1e-10 drop
    assert abs(hg[-200:].min() / ho[-200:].min() - 1.0) < 1e-6
    assert abs(hg[-200:].max() / ho[-200:].max() - 1.0) < 1e-6
