"""The reference's stops, reached on the GPU from a bad state injected on the
host, and the context usable again afterwards.

A bad state goes in through mge_upload_state, which (like init_flow.f90
after read_solut) runs depvars, bc_cutcell and bcond on it.  The library
then stops where the reference's sequential run would stop first, with the
same code and location as the oracle on the same state:
- a negative density in a fluid cell: c^2 = gamma*p/rho < 0 in the next
  time step, timestep.f90:45-48 (MGE_ENEGPRESS);
- a NaN energy in a cell of a cut-cell record's cloud: the record's solid
  state is NaN, bc_cutcell.f90:147-156 (MGE_ENAN), already at the upload;
- a NaN energy in a box with no body: depvars' max(.,0) gives p = 0 there,
  so no time step stops; the NaN spreads through the fluxes and the residual
  norm after the finest update is NaN, solver.f90:180 (MGE_ENAN).
The kernels record the first stop in launch order in the context's error
word and the host reads it after the cycle; nothing faults.  A good state
uploaded afterwards runs to the same result as a fresh context given it.
"""
import ctypes as C

import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300.runtime import Cycle, MgeError
from oracle.oracle import OracleCycle
from code_mge_gb300 import cases as K
from parity import small_sphere

pytestmark = pytest.mark.gpu

# (variable, padded index (k, j, i), value, expected code, reference location)
INJECT = {
    "negative_density": (0, (4, 4, 4), -1.0, A.MGE_ENEGPRESS, "timestep.f90:45-48"),
    "nan_in_a_cloud": (4, None, np.nan, A.MGE_ENAN, "bc_cutcell.f90:147-156"),
    "nan_without_a_body": (4, (5, 6, 7), np.nan, A.MGE_ENAN, "solver.f90:180"),
}


def _case(kind="negative_density"):
    if kind == "nan_without_a_body":
        case = K.free_stream_box(n=(12, 10, 8), nlevel=2, mach=0.5)
    else:
        case = small_sphere(nlevel=2, n=16)
    case.prm.mcyc[0] = 1
    case.prm.mcyc[1] = 3
    return case


def _cloud_cell(spec):
    """The first cloud cell of the first cut-cell record, as a padded (k, j, i) index."""
    i, j, k = (int(x) for x in np.asarray(spec.arrays["ijkdex"])[0, 0])
    return (k, j, i)


def _bad_state(w, kind, spec):
    v, at, val, _, _ = INJECT[kind]
    at = at if at is not None else _cloud_cell(spec)
    w = w.copy()
    if kind == "negative_density":
        val = -abs(w[(0,) + at])
    w[(v,) + at] = val
    return w


def _run(c, L, bad):
    """Upload then one cycle; the MgeError of whichever stops first."""
    with pytest.raises(MgeError) as e:
        c.upload(bad, L)
        c.cycle(L, ncyc=2)
    return e.value


@pytest.mark.parametrize("kind", sorted(INJECT))
def test_stop_matches_the_oracle_and_the_context_recovers(gpulib, kind):
    case = _case(kind)
    L = case.prm.nlevel
    g = Cycle(case)
    g.cycle(L, ncyc=1)
    good = [g.field("w", lv) for lv in range(1, L + 1)]
    bad = _bad_state(good[-1], kind, g.spec(L))
    eg = _run(g, L, bad)
    o = OracleCycle(case)
    eo = _run(o, L, bad)
    code, where = INJECT[kind][3], INJECT[kind][4]
    assert eg.code == eo.code == code, (str(eg), str(eo))
    assert where in str(eg) and where in str(eo)
    # good states again on every level (the stopped cycle ran on and spread
    # the bad values to the coarse levels and their records): the same cycle
    # as a fresh context given those states
    for lv in range(1, L + 1):
        g.upload(good[lv - 1], lv)
    r1 = g.cycle(L, ncyc=3)
    f = Cycle(case)
    for lv in range(1, L + 1):
        f.upload(good[lv - 1], lv)
    r2 = f.cycle(L, ncyc=3)
    assert np.isfinite(r1) and r1 == r2
    assert np.array_equal(g.field("w", L), f.field("w", L))
    for c in (g, o, f):
        c.close()


def test_solve_returns_the_stop(gpulib):
    # mge_solve starts on the coarsest level (FMG): the bad state goes there
    case = _case()
    g = Cycle(case)
    g.upload(_bad_state(g.field("w", 1), "negative_density", g.spec(1)), 1)
    with pytest.raises(MgeError) as e:
        g.solve()
    assert e.value.code == A.MGE_ENEGPRESS
    assert "timestep.f90:45-48" in str(e.value)
    g.close()


def test_async_poll_returns_the_stop(gpulib):
    case = _case()
    L = case.prm.nlevel
    lib = gpulib
    g = Cycle(case)
    good = [g.field("w", lv) for lv in range(1, L + 1)]
    g.upload(_bad_state(good[-1], "negative_density", g.spec(L)), L)
    assert lib.mge_cycle_async(g.ctx, L) == A.MGE_OK
    mr = C.c_double()
    rc = 1
    while rc == 1:
        rc = lib.mge_cycle_poll(g.ctx, 1, C.byref(mr))
    assert rc == A.MGE_ENEGPRESS
    assert b"timestep.f90:45-48" in lib.mge_last_error(g.ctx)
    for lv in range(1, L + 1):
        g.upload(good[lv - 1], lv)
    assert lib.mge_cycle_async(g.ctx, L) == A.MGE_OK
    rc = 1
    while rc == 1:
        rc = lib.mge_cycle_poll(g.ctx, 2, C.byref(mr))
    assert rc == A.MGE_OK and np.isfinite(mr.value)
    g.close()
