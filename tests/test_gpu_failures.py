"""The reference's stops, reached on the GPU from a bad state injected on the
host, and the context usable again afterwards.

The reference stops at timestep.f90:45-48 when c^2 = gamma*p/rho is
negative or NaN.  A state with a negative density, or with a NaN, uploaded
through mge_upload_state reaches that test in the first time step of the
next cycle.  The library then returns MGE_ENEGPRESS with the reference's
location from mge_cycle, mge_solve and mge_cycle_poll, as the oracle does
for the same state.  Nothing faults: the kernels set a bit of the context's
error word and the host reads it after the cycle.  A good state uploaded
afterwards runs to the same result as a fresh context given that state.
"""
import ctypes as C

import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300.runtime import Cycle, MgeError
from oracle.oracle import OracleCycle
from parity import small_sphere

pytestmark = pytest.mark.gpu


def _bad_state(w, kind):
    w = w.copy()
    k, j, i = (s // 2 for s in w.shape[1:])
    if kind == "negative_density":
        w[0, k, j, i] = -abs(w[0, k, j, i])
    else:
        w[4, k, j, i] = np.nan
    return w


def _case():
    case = small_sphere(nlevel=2, n=16)
    case.prm.mcyc[0] = 1
    case.prm.mcyc[1] = 3
    return case


@pytest.mark.parametrize("kind", ["negative_density", "nan"])
def test_cycle_stops_as_the_reference_and_recovers(gpulib, kind):
    case = _case()
    L = case.prm.nlevel
    g = Cycle(case)
    g.cycle(L, ncyc=1)
    good = g.field("w", L)
    g.upload(_bad_state(good, kind), L)
    with pytest.raises(MgeError) as e:
        g.cycle(L, ncyc=2)
    assert e.value.code == A.MGE_ENEGPRESS
    assert "timestep.f90:45-48" in str(e.value)
    # the oracle stops at the same place for the same state
    o = OracleCycle(case)
    o.upload(_bad_state(good, kind), L)
    with pytest.raises(MgeError) as eo:
        o.cycle(L, ncyc=2)
    assert eo.value.code == A.MGE_ENEGPRESS
    # a good state again: the same cycle as a fresh context from that state
    g.upload(good, L)
    r1 = g.cycle(L, ncyc=3)
    f = Cycle(case)
    f.upload(good, L)
    r2 = f.cycle(L, ncyc=3)
    assert r1 == r2 and np.isfinite(r1)
    assert np.array_equal(g.field("w", L), f.field("w", L))
    for c in (g, o, f):
        c.close()


def test_solve_returns_the_stop(gpulib):
    # mge_solve starts on the coarsest level (FMG): the bad state goes there
    case = _case()
    g = Cycle(case)
    g.upload(_bad_state(g.field("w", 1), "negative_density"), 1)
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
    good = g.field("w", L)
    g.upload(_bad_state(good, "nan"), L)
    assert lib.mge_cycle_async(g.ctx, L) == A.MGE_OK
    mr = C.c_double()
    rc = 1
    while rc == 1:
        rc = lib.mge_cycle_poll(g.ctx, 1, C.byref(mr))
    assert rc == A.MGE_ENEGPRESS
    assert b"timestep.f90:45-48" in lib.mge_last_error(g.ctx)
    g.upload(good, L)
    assert lib.mge_cycle_async(g.ctx, L) == A.MGE_OK
    rc = 1
    while rc == 1:
        rc = lib.mge_cycle_poll(g.ctx, 2, C.byref(mr))
    assert rc == A.MGE_OK and np.isfinite(mr.value)
    g.close()
