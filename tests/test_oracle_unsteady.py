"""Unsteady dual time stepping (execmode 1) in the oracle: the BDF source of
euler.f90:249-275, the coarse-level division of :320-331, the update factor of
:387-391, the time-step limit of timestep.f90:85-99 and the time-level shift of
solver.f90:263-276."""
import numpy as np

from code_mge_gb300 import cases as K
from code_mge_gb300.runtime import physical
from oracle.oracle import OracleCycle


def _cycles(case, fine):
    """mcyc of the case (the context copies the parameters when it is made)."""
    L = case.prm.nlevel
    case.prm.mcyc[L - 1] = fine
    for q in range(L - 1):
        case.prm.mcyc[q] = 1
    return case


def _steps(o, nsteps):
    for _ in range(nsteps):
        o.solve()
        o.time_advance()


def test_free_stream_survives_physical_steps():
    case = _cycles(K.free_stream_box(n=(10, 8, 6), nlevel=2, mach=0.5, execmode=1, dtstep=0.5), 3)
    o = OracleCycle(case)
    sp = o.spec(2)
    w0 = physical(o.field("w", 2), sp).copy()
    _steps(o, 3)
    w = physical(o.field("w", 2), sp)
    assert np.max(np.abs(w - w0)) <= 1e-13 * np.max(np.abs(w0))
    assert np.array_equal(o.field("w1", 2), o.field("w", 2))   # after the shift


def test_huge_physical_step_is_the_steady_cycle():
    a = _cycles(K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0), 4)
    b = _cycles(K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, execmode=1, dtstep=1e30), 4)
    oa, ob = OracleCycle(a), OracleCycle(b)
    ob.time_advance()
    ob.time_advance()   # itime 2: the BDF2 source is on, and negligible
    for c in (oa, ob):
        c.solve()
    wa, wb = oa.field("w", 2), ob.field("w", 2)
    assert np.max(np.abs(wa - wb)) <= 1e-13 * np.max(np.abs(wa))


def test_state_moves_in_proportion_to_the_physical_step():
    moved = []
    for dt in (2e-3, 2e-2):
        # one level: with more, every physical step restarts the full
        # multigrid sequence and its prolongation replaces the fine state
        # (solver.f90:119-259 inside the time loop)
        case = _cycles(K.cylinder_slab(n=32, span=2, nlevel=1, extent=4.0, execmode=1, dtstep=dt), 40)
        o = OracleCycle(case)
        sp = o.spec(1)
        # an impulsively started cylinder: step 0 (no source) from free stream,
        # then a BDF1 step; the change over the BDF1 step scales with dt
        _steps(o, 1)
        w1 = physical(o.field("w", 1), sp).copy()
        _steps(o, 1)
        moved.append(np.max(np.abs(physical(o.field("w", 1), sp) - w1)))
    ratio = moved[1] / moved[0]
    assert 3.0 < ratio < 30.0, moved
