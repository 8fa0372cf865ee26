"""The moving surface on the GPU against the oracle: mge_move_surface
(movsurf.f90:28-35, called at solver.f90:117 with approxbc on) and the moved
normals and wall velocities in every kernel that reads them
(bc_cutcell.f90:47-50 and the wall fluxes)."""
import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import cases as K
from motion import VEL_FS, move_all
from parity import PATHS, compare, pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("nstage", [1, 5])
@pytest.mark.parametrize("ns", [False, True])
def test_stage_after_a_move(gpulib, path, nstage, ns):
    kw = dict(eqntype=A.MGE_EQN_NS, distype=A.MGE_DIS_ROE2, reynolds=40.0) if ns else {}
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=4, **kw)
    g, o = pair(case, develop_cycles=3, path=path)
    try:
        L = case.prm.nlevel
        for c in (g, o):
            move_all(c, case, theta=0.35, y=0.02, dtheta=0.3, dy=-0.15)
            c.timestep(L)
            c.euler_partial(L, nstage)
        for f in ("dw", "fw", "wsol"):
            compare(g, o, f, L)
        for f in ("w", "p"):
            compare(g, o, f, L, phys_only=False)
        for lv in (1, 2):
            assert np.array_equal(g.surface(lv), o.surface(lv))
    finally:
        g.close()
        o.close()


@pytest.mark.parametrize("graph", [0, 1])
def test_heaving_and_pitching_steps(gpulib, graph):
    """Three physical steps of dual time stepping, the surface moved at the
    start of each: every cycle's residual and the state after each step."""
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=4, execmode=1, dtstep=0.05)
    case.prm.mcyc[0] = 2
    g, o = pair(case)
    try:
        for step in range(3):
            t = step * 0.05
            kin = dict(theta=0.2 * np.sin(4.0 * t), y=0.1 * np.sin(4.0 * t), dtheta=0.8 * np.cos(4.0 * t),
                       dy=0.4 * np.cos(4.0 * t))
            for c in (g, o):
                move_all(c, case, **kin)
            hg, ng, fg = g.solve(use_graph=graph)
            ho, no, fo = o.solve()
            assert ng == no
            assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
            compare(g, o, "w", 2, rtol=1e-11, phys_only=False)
            assert abs(fg.cl - fo.cl) <= 1e-9 * max(1.0, abs(fo.cd))
            assert g.time_advance() == o.time_advance() == step + 1
    finally:
        g.close()
        o.close()


def test_surface_points_and_refusal(gpulib):
    from code_mge_gb300.runtime import Cycle, MgeError
    from motion import rigid
    case = K.cylinder_slab(n=32, span=2, nlevel=1, extent=4.0, mcyc_fine=4)
    sp = case.levels[0][0]
    g = Cycle(case)
    try:
        assert np.array_equal(g.surface(1), sp.arrays["psurf"])
        disp, norv, vel = rigid(sp, theta=0.3, y=0.05)
        g.move_surface(1, disp, norv, vel, VEL_FS)
        assert np.array_equal(g.surface(1), sp.arrays["psurf"] + disp)
        with pytest.raises(MgeError) as e:
            g.move_surface(1, disp, norv, vel, -1.0)
        assert e.value.code == A.MGE_EBADCFG
    finally:
        g.close()
