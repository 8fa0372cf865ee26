"""GPU parity at the full sizes of the measured workloads.

The per-stage tests of test_gpu_parity.py run on 16^3-32^3 blocks; these
run the same comparisons on the blocks the benchmark times:
- the 192^3 sphere (4-level W-cycle, JST scalar, IRS 0.6), one developed
  W-cycle, then each of the five stages of a finest-level update;
- the 512x512x2 laminar Navier-Stokes cylinder at h = D/96 (Roe MUSCL +
  viscous fluxes, 4 embedded levels), the same;
- the 256x256x2 cylinder slab exactly as the first workload states it
  (M=0.3, JST k2=0.5, k4=1/64, IRS 0.6, 3-level V-cycle, 500 finest cycles):
  the whole residual history and the converged Cd and Cl.

Tolerance: the plain path's per-stage criterion, the infinity norm of the
difference relative to the infinity norm of the oracle field, <= 1e-12
(parity.RTOL).  The oracle runs on every host thread (its OpenMP loops
have independent iterations, so its results do not depend on the count).
"""
import os

import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import cases as K
from parity import RTOL, compare, pair

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _all_threads():
    from oracle import oracle as O
    before = O.load().mgeo_get_threads()
    O.set_threads(os.cpu_count() or 1)
    yield
    O.set_threads(before)


def _stages_from_developed_state(g, o):
    """Upload the same developed state into both, then for each stage count
    run timestep + that many stages and compare."""
    L = g.case.prm.nlevel
    w0 = o.field("w", L)
    errs = {}
    for nstage in range(1, g.case.prm.mstage + 1):
        for c in (g, o):
            c.upload(w0, L)
            c.timestep(L)
            c.euler_partial(L, nstage)
        for f in ("dw", "fw"):
            errs[(nstage, f)] = compare(g, o, f, L)[0]
        for f in ("w", "p"):
            errs[(nstage, f)] = compare(g, o, f, L, phys_only=False)[0]
        if g.spec(L).arrays["nmir"]:
            errs[(nstage, "wsol")] = compare(g, o, "wsol", L)[0]
    return errs


def test_sphere_192_stages():
    case = K.sphere_box(n=192, nlevel=4, extent=10.0, mach=0.5, mgtype=2, mcyc_fine=400, smoo=0.6)
    g, o = pair(case, develop_cycles=1, path="tuned")
    try:
        errs = _stages_from_developed_state(g, o)
        assert max(errs.values()) <= RTOL
    finally:
        g.close()
        o.close()


def test_ns_cylinder_512_stages():
    case = K.cylinder_embedded(n=512, span=2, nlevel=4, h_fine=1.0 / 96.0, mach=0.2, mcyc_fine=200,
                               eqntype=A.MGE_EQN_NS, distype=A.MGE_DIS_ROE2, reynolds=40.0)
    g, o = pair(case, develop_cycles=1, path="tuned")
    try:
        errs = _stages_from_developed_state(g, o)
        assert max(errs.values()) <= RTOL
    finally:
        g.close()
        o.close()


def test_cylinder_256_history_of_500_cycles():
    """Every cycle's residual within 1e-11 of the oracle's, relative; Cd and
    Cl within 1e-9.  The two differ only where the far field's powers and
    the residual norm's summation order round differently; the relative
    difference of the residual grows as the residual falls (3.7 decades in
    these 500 cycles), to about 1e-11 at the end."""
    import numpy as np
    case = K.cylinder_slab(n=256, span=2, nlevel=3, extent=20.0, mach=0.3, mcyc_fine=500, smoo=0.6)
    assert case.prm.mcyc[2] == 500 and case.prm.mgtype == 1
    g, o = pair(case, path="tuned")
    try:
        hg, ng, fg = g.solve()
        ho, no, fo = o.solve()
        assert ng == no == 500
        rel = np.abs(hg - ho) / np.abs(ho)
        assert rel.max() <= 1e-11, (int(rel.argmax()), float(rel.max()))
        assert abs(fg.cd - fo.cd) <= 1e-9 * max(1.0, abs(fo.cd))
        assert abs(fg.cl - fo.cl) <= 1e-9 * max(1.0, abs(fo.cd))
        compare(g, o, "w", 3, rtol=1e-11, phys_only=False)
    finally:
        g.close()
        o.close()
