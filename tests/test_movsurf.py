"""The moving surface in the oracle, on the CPU: movsurf.f90:28-35 (pnew =
psurf + disp, called at solver.f90:117 with approxbc on) and its use in
bc_cutcell.f90:47-50 (the normal norv, the wall velocity vel/vel_fs)."""
import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import cases as K
from motion import VEL_FS, move_all, rigid


def _oracle(case):
    from oracle.oracle import OracleCycle
    return OracleCycle(case)


def test_the_resting_surface_changes_nothing():
    """disp 0, norv = nvec and vel = qb*vel_fs (vel_fs a power of two, so the
    division gives qb back exactly): the same solve, bit for bit."""
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=4, omega=0.4)
    a, b = _oracle(case), _oracle(case)
    try:
        for L, specs in enumerate(case.levels, start=1):
            sp = specs[0]
            qb = sp.arrays["qb"]
            assert np.abs(qb).max() > 0.0
            b.move_surface(L, np.zeros_like(qb), sp.arrays["nvec"], qb * 4.0, 4.0)
        ha, na, fa = a.solve()
        hb, nb, fb = b.solve()
        assert na == nb and np.array_equal(ha, hb) and fa.cd == fb.cd
        assert np.array_equal(a.field("w", 2), b.field("w", 2))
    finally:
        a.close()
        b.close()


def test_moved_points():
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=4)
    o = _oracle(case)
    try:
        for L in (1, 2):
            sp = case.levels[L - 1][0]
            assert np.array_equal(o.surface(L), sp.arrays["psurf"])  # before any move
            disp, norv, vel = rigid(sp, theta=0.3, y=0.05, dtheta=0.2, dy=0.1)
            o.move_surface(L, disp, norv, vel, VEL_FS)
            assert np.array_equal(o.surface(L), sp.arrays["psurf"] + disp)
            # the moved points lie on the turned and shifted circle
            p = o.surface(L)
            assert np.allclose(np.hypot(p[:, 0], p[:, 1] - 0.05), 0.5, atol=1e-12)
    finally:
        o.close()


def test_reflection_uses_the_moved_normal_and_velocity():
    """A uniform state: every cloud interpolates it back, so bc_cutcell's
    reflection (bc_cutcell.f90:139-144) of it about the moved normal n, with
    the wall velocity qb = vel/vel_fs, has the closed form
        m_sol = m - 2 (n . (m - rho qb)) n,  E_sol = p/(gamma-1) + |m_sol|^2/(2 rho)."""
    case = K.cylinder_slab(n=32, span=2, nlevel=1, extent=4.0, mcyc_fine=4)
    sp = case.levels[0][0]
    o = _oracle(case)
    try:
        gamma = case.prm.gamma
        rho, u, v, p = 1.1, 0.3, -0.1, 1.0 / (gamma * 0.09)
        E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
        w = np.zeros((5,) + tuple(sp.dims[::-1]))
        w[0], w[1], w[2], w[3], w[4] = rho, rho * u, rho * v, 0.0, E
        o.upload(w, 1)
        fixed = o.field("wsol", 1)
        disp, norv, vel = rigid(sp, theta=0.4, dtheta=0.3, dy=-0.2)
        o.move_surface(1, disp, 3.0 * norv, vel, VEL_FS)  # the normal need not be unit
        o.upload(w, 1)  # bc_cutcell runs on the upload
        got = o.field("wsol", 1)
        n = norv / np.linalg.norm(norv, axis=1)[:, None]
        qb = vel / VEL_FS
        m = np.array([rho * u, rho * v, 0.0])
        qn = 2.0 * np.sum(n * (m - rho * qb), axis=1)
        msol = m - qn[:, None] * n
        want = np.concatenate([np.full((len(n), 1), rho), msol,
                               (p / (gamma - 1.0) + 0.5 * np.sum(msol * msol, axis=1) / rho)[:, None]], axis=1)
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
        assert np.abs(got - fixed).max() > 1e-3  # the motion changed the reflection
    finally:
        o.close()


def test_bad_motion_is_refused():
    from code_mge_gb300.runtime import MgeError
    case = K.cylinder_slab(n=32, span=2, nlevel=1, extent=4.0, mcyc_fine=4)
    sp = case.levels[0][0]
    o = _oracle(case)
    try:
        disp, norv, vel = rigid(sp, theta=0.1)
        with pytest.raises(MgeError) as e:
            o.move_surface(1, disp, norv, vel, 0.0)
        assert e.value.code == A.MGE_EBADCFG
        with pytest.raises(ValueError):
            o.move_surface(1, disp[:-1], norv, vel, VEL_FS)
        assert o._fn("move_surface")(o.ctx, 2, 1, None, None, None, VEL_FS) == A.MGE_ENOTFOUND
    finally:
        o.close()


def test_heaving_unsteady_steps_run():
    """Dual time stepping with the surface moved at the start of every
    physical step (solver.f90:117): the steps run, and the lift opposes the
    heave velocity (the flow relative to the wall comes from above)."""
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=4, execmode=1, dtstep=0.05)
    o = _oracle(case)
    try:
        cl = []
        for step in range(3):
            t = step * 0.05
            move_all(o, case, theta=0.0, y=0.1 * np.sin(4.0 * t), dy=0.4 * np.cos(4.0 * t))
            h, n, f = o.solve()
            assert n > 0 and np.all(np.isfinite(h))
            cl.append(f.cl)
            o.time_advance()
        assert cl[-1] < 0.0
    finally:
        o.close()


def test_no_slip_wall_takes_the_moved_velocity():
    """Navier-Stokes: bc_cutcell.f90:185 sets the solid state's momentum to
    2 rho qb - m (the normal does not enter) and :201 its energy from psol;
    on a uniform state that is, with qb = vel/vel_fs,
        m_sol = 2 rho qb - m,  E_sol = p/(gamma-1) + |m_sol|^2/(2 rho)."""
    case = K.cylinder_slab(n=32, span=2, nlevel=1, extent=4.0, mcyc_fine=4, eqntype=A.MGE_EQN_NS,
                           distype=A.MGE_DIS_ROE2, reynolds=40.0)
    sp = case.levels[0][0]
    o = _oracle(case)
    try:
        gamma = case.prm.gamma
        rho, u, v, p = 0.9, 0.25, 0.05, 1.0 / (gamma * 0.04)
        w = np.zeros((5,) + tuple(sp.dims[::-1]))
        w[0], w[1], w[2], w[3], w[4] = rho, rho * u, rho * v, 0.0, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
        disp, norv, vel = rigid(sp, theta=0.2, dtheta=0.6, dy=0.3)
        o.move_surface(1, disp, norv, vel, VEL_FS)
        o.upload(w, 1)
        got = o.field("wsol", 1)
        m = np.array([rho * u, rho * v, 0.0])
        msol = 2.0 * rho * (vel / VEL_FS) - m
        want = np.concatenate([np.full((len(msol), 1), rho), msol,
                               (p / (gamma - 1.0) + 0.5 * np.sum(msol * msol, axis=1) / rho)[:, None]], axis=1)
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    finally:
        o.close()
