"""Unsteady dual time stepping (execmode 1) on the GPU against the oracle:
per stage with the first-step and BDF2 sources on the finest level (update
factor) and on a coarse level (residual division), the time-level shift, and
a run of physical steps through the captured cycles."""
import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from parity import PATHS, compare, pair, small_cylinder, small_sphere

pytestmark = pytest.mark.gpu


def _history(g, o, itime):
    """Both sides: itime physical-step shifts with an update between, so that
    w, w1 and w2 differ."""
    L = g.case.prm.nlevel
    for q in range(itime):
        for c in (g, o):
            c.time_advance()
            c.timestep(L)
            c.euler(L, itime=q + 1, ncyc=1)


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("itime", [1, 2])
@pytest.mark.parametrize("nstage", [1, 2, 5])
def test_stage_on_the_finest_level(gpulib, itime, nstage, path):
    g, o = pair(small_cylinder(execmode=1, dtstep=0.05), develop_cycles=3, path=path)
    _history(g, o, itime)
    L = g.case.prm.nlevel
    for c in (g, o):
        c.timestep(L)
        c.euler_partial(L, nstage, itime=itime)
    for f in ("dw", "fw", "w", "p", "w1", "w2"):
        compare(g, o, f, L, phys_only=f not in ("w", "p"))
    compare(g, o, "vdtim", L)


@pytest.mark.parametrize("itime", [1, 2])
def test_coarse_level_with_forcing(gpulib, itime):
    g, o = pair(small_sphere(execmode=1, dtstep=0.1), develop_cycles=3)
    _history(g, o, itime)
    L = g.case.prm.nlevel
    for c in (g, o):
        c.timestep(L)
        c.euler(L, itime=itime, ncyc=1, lres=True)
        c.movco(L - 1)
        c.timestep(L - 1)
        c.euler(L - 1, itime=itime, ncyc=1, mgl=L - 1, mlvl=L, lfir=True)
    for f in ("dw", "w", "qf"):
        compare(g, o, f, L - 1)


@pytest.mark.parametrize("mk", [lambda: small_cylinder(execmode=1, dtstep=0.05),
                                lambda: small_sphere(execmode=1, dtstep=0.1, mgtype=2)])
def test_physical_steps(gpulib, mk):
    case = mk()
    L = case.prm.nlevel
    case.prm.mcyc[0] = 2
    case.prm.mcyc[L - 1] = 4
    g, o = pair(case)
    for step in range(3):
        hg, ng, _ = g.solve(use_graph=1)
        ho, no, _ = o.solve()
        assert ng == no
        assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
        compare(g, o, "w", L, rtol=1e-11, phys_only=False)
        assert g.time_advance() == o.time_advance() == step + 1
    compare(g, o, "w2", L, rtol=1e-11, phys_only=False)


def test_bad_unsteady_parameters_are_rejected(gpulib):
    from code_mge_gb300.runtime import Cycle, MgeError
    case = small_cylinder(execmode=1, dtstep=0.0)
    with pytest.raises(MgeError) as e:
        Cycle(case)
    assert e.value.code == A.MGE_EBADCFG
