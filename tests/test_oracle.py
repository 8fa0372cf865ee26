"""CPU oracle: analytic invariants of the restated reference algorithm.

The reference ships no golden vectors for this path, so the oracle's parity
with the reference is unpinned; these invariants pin its behaviour instead.
"""
import numpy as np
import pytest

from code_mge_gb300 import cases as K
from code_mge_gb300.runtime import physical
from oracle.oracle import OracleCycle


def test_free_stream_preserved_exactly():
    case = K.free_stream_box(n=(12, 10, 8), nlevel=2, mach=0.6)
    o = OracleCycle(case)
    o.timestep(2)
    o.euler(2, ncyc=1, lres=True)
    dw = o.field("dw", 2)
    # cells beyond the two-cell stencil reach of the far-field ghosts: exactly zero
    assert np.abs(dw[:, 4:-4, 4:-4, 4:-4]).max() == 0.0
    # next to the boundary the characteristic far-field state differs from the
    # free stream by rounding only
    assert np.abs(physical(dw, o.spec(2))).max() < 1e-14
    o.euler(2, ncyc=1)
    assert o.rtrms(2, 1) < 1e-13


def test_span_independence_of_periodic_slab():
    # without smoothing the two span planes see identical stencils: bit-equal
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=6, smoo=0.0)
    case.prm.mcyc[0] = 2
    o = OracleCycle(case)
    o.solve()
    w = o.field("w", 2)
    assert np.array_equal(w[:, 2], w[:, 3])
    # the two-cell k-lines of psmoo_old round the two planes differently
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=6, smoo=0.6)
    case.prm.mcyc[0] = 2
    o = OracleCycle(case)
    o.solve()
    w = o.field("w", 2)
    np.testing.assert_allclose(w[:, 2], w[:, 3], rtol=1e-12)


def test_symmetry_about_the_flow_axis():
    # smoo = 0: psmoo_old skips blanked cells without re-factoring its pivots
    # (psmoo.f90:174-235), so with smoothing on the solution is not mirror
    # symmetric by construction (see test_psmoo_old_blank_skipping_is_directional)
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=8, mach=0.3, smoo=0.0)
    case.prm.mcyc[0] = 2
    o = OracleCycle(case)
    _, _, f = o.solve()
    w = physical(o.field("w", 2), o.spec(2))
    rho = w[0]
    np.testing.assert_allclose(rho, rho[:, ::-1, :], rtol=1e-12, atol=0)
    np.testing.assert_allclose(w[2], -w[2][:, ::-1, :], rtol=0, atol=1e-12 * np.abs(w[1]).max())
    assert abs(f.cl) < 1e-9


def test_psmoo_old_blank_skipping_is_directional():
    case = K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=8, mach=0.3, smoo=0.6)
    o = OracleCycle(case)
    o.timestep(2)
    o.euler(2, ncyc=1, lres=True)
    d = physical(o.field("dw", 2), o.spec(2))
    assert np.abs(d[0] - d[0][:, ::-1]).max() < 1e-15   # the residual itself is symmetric
    o.timestep(2)
    o.euler_partial(2, 1)
    w = physical(o.field("w", 2), o.spec(2))
    assert np.abs(w[0] - w[0][:, ::-1]).max() > 1e-6    # the smoothed update is not


def _tridiag(n, e):
    T = np.zeros((n, n))
    for q in range(n):
        T[q, q] = 1.0 + 2.0 * e
        if q > 0:
            T[q, q - 1] = -e
        if q < n - 1:
            T[q, q + 1] = -e
    return T


def test_psmoo_old_inverts_the_constant_tridiagonal_operators():
    # no body: every cell is fluid; dw(smoo) = Tz^-1 Ty^-1 Tx^-1 dw(smoo=0)
    rng = np.random.default_rng(7)
    case = K.free_stream_box(n=(10, 8, 6), nlevel=1, mach=0.5, smoo=0.0)
    sp = case.levels[0][0]
    w = None
    outs = {}
    for smoo in (0.0, 0.6):
        case.prm.smoo = smoo
        o = OracleCycle(case)
        if w is None:
            w = o.field("w", 1).copy()
            w[0] *= 1.0 + 0.05 * rng.standard_normal(w[0].shape)
            w[4] *= 1.0 + 0.05 * rng.standard_normal(w[4].shape)
        o.upload(w, 1)
        o.timestep(1)
        o.euler_partial(1, 1)
        outs[smoo] = physical(o.field("dw", 1), sp)
    raw, sm = outs[0.0], outs[0.6]
    nx, ny, nz = sp.n
    Tx, Ty, Tz = _tridiag(nx, 0.6), _tridiag(ny, 0.6), _tridiag(nz, 0.6)
    back = np.einsum("ai,vkji->vkja", Tx, sm)
    back = np.einsum("bj,vkja->vkba", Ty, back)
    back = np.einsum("ck,vkba->vcba", Tz, back)
    np.testing.assert_allclose(back, raw, rtol=0, atol=1e-12 * np.abs(raw).max())


def test_psmoo_inverts_the_variable_tridiagonal_operators():
    # psmoo + progon3 (psmoo.f90:1-95): per-cell eps from the time step,
    # aa = 1+2eps, bb = cc = -eps with the end couplings zeroed; the smoothed
    # residual solves Tx Ty Tz applied in reverse
    rng = np.random.default_rng(11)
    case = K.free_stream_box(n=(9, 7, 5), nlevel=1, mach=0.5, smoo=0.0)
    sp = case.levels[0][0]
    case.prm.irs_variant = 1
    w = None
    outs, eps = {}, None
    for smoo in (0.0, 0.6):
        case.prm.smoo = smoo
        o = OracleCycle(case)
        if w is None:
            w = o.field("w", 1).copy()
            w[0] *= 1.0 + 0.05 * rng.standard_normal(w[0].shape)
            w[1] += 0.2 * rng.standard_normal(w[1].shape)
            w[4] *= 1.0 + 0.05 * rng.standard_normal(w[4].shape)
        o.upload(w, 1)
        o.timestep(1)
        if smoo > 0:
            eps = physical(o.field("eps", 1), sp)
        o.euler_partial(1, 1)
        outs[smoo] = physical(o.field("dw", 1), sp)
    raw, sm = outs[0.0], outs[0.6]
    assert 0.0 < eps.min() and eps.max() <= 0.6 and eps.std() > 0  # variable coefficients
    nx, ny, nz = sp.n

    def apply(e, x, axis):
        # (T x)_q = (1+2e_q) x_q - e_q x_{q+1} - e_q x_{q-1}, no coupling past the ends
        x = np.moveaxis(x, axis, -1)
        e = np.moveaxis(e, axis - 1, -1)
        y = (1.0 + 2.0 * e) * x
        y[..., :-1] -= e[..., :-1] * x[..., 1:]
        y[..., 1:] -= e[..., 1:] * x[..., :-1]
        return np.moveaxis(y, -1, axis)

    back = apply(eps[2], sm, 1)      # undo the k sweep (axis of k in [v, k, j, i])
    back = apply(eps[1], back, 2)    # then j
    back = apply(eps[0], back, 3)    # then i
    np.testing.assert_allclose(back, raw, rtol=0, atol=1e-12 * np.abs(raw).max())


def test_transfers_reproduce_linear_fields():
    case = K.sphere_box(n=16, nlevel=2, extent=2.0, radius=0.01)
    o = OracleCycle(case)
    fine, coarse = o.spec(2), o.spec(1)

    def linear(sp):
        P = sp.dims
        ii = np.arange(P[0]); jj = np.arange(P[1]); kk = np.arange(P[2])
        x = sp.origin[0] + (ii - 1.5) * sp.h[0]
        y = sp.origin[1] + (jj - 1.5) * sp.h[1]
        z = sp.origin[2] + (kk - 1.5) * sp.h[2]
        X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
        f = 2.0 + 0.1 * X - 0.2 * Y + 0.05 * Z
        w = np.stack([f, 0.3 * f, -0.1 * f, 0.2 * f, 5.0 * f]).transpose(0, 3, 2, 1)
        return np.ascontiguousarray(w)

    o.upload(linear(fine), 2)
    o.movco(1)
    wc = physical(o.field("w", 1), coarse)
    np.testing.assert_allclose(wc, physical(linear(coarse), coarse), rtol=1e-13)
    o.upload(linear(coarse), 1)
    o.movfin(2, 1)   # FMG step: w_f = I(w_c)
    wf = physical(o.field("w", 2), fine)
    np.testing.assert_allclose(wf, physical(linear(fine), fine), rtol=1e-13)


def test_negative_pressure_is_reported():
    from code_mge_gb300 import _abi as A
    from code_mge_gb300.runtime import MgeError
    case = K.free_stream_box(n=(8, 8, 8), nlevel=1)
    o = OracleCycle(case)
    w = o.field("w", 1).copy()
    w[0, 5, 5, 5] = -1.0   # negative density: c^2 = gamma p / rho < 0
    o.upload(w, 1)
    with pytest.raises(MgeError) as e:
        o.timestep(1)
    assert e.value.code == A.MGE_ENEGPRESS


def test_w_cycle_converges():
    case = K.sphere_box(n=24, nlevel=3, extent=4.0, mgtype=2, mcyc_fine=40, radius=0.7)
    case.prm.mcyc[0] = 2
    case.prm.mcyc[1] = 4
    o = OracleCycle(case)
    hist, n, f = o.solve()
    assert n == 40
    assert hist[-1] < 0.05 * hist[0]
    assert np.isfinite(f.cd)


def test_viscous_wall_stress_drags_the_body_at_free_stream():
    """At the free-stream start the wall pressure is uniform, so the pressure
    forces of the closed wall cancel; with NS the no-slip wall stress pulls
    the body along the flow (+x), and nothing acts across it."""
    from code_mge_gb300 import _abi as A
    from parity import small_cylinder
    euler = OracleCycle(small_cylinder(mach=0.2)).forces()
    ns = OracleCycle(small_cylinder(mach=0.2, eqntype=A.MGE_EQN_NS, reynolds=40.0)).forces()
    assert abs(euler.force[0]) < 1e-9 and abs(euler.force[1]) < 1e-9
    assert ns.force[0] > 1e3 * abs(euler.force[0]) and ns.force[0] > 0.0
    assert abs(ns.force[1]) <= 1e-12 * ns.force[0]
    assert ns.cd > 0.0


def test_turning_wall_breaks_the_up_down_symmetry():
    """A cylinder at rest in a uniform stream keeps Cl = 0 by symmetry (without
    residual smoothing, whose blank skipping is directional); with the wall
    turning, the records' wall velocity enters the reflected states and the
    wall stress, and a lift appears after a few cycles."""
    from code_mge_gb300 import _abi as A
    from parity import small_cylinder
    out = {}
    for omega in (0.0, 0.8, -0.8):
        case = small_cylinder(mach=0.2, eqntype=A.MGE_EQN_NS, reynolds=40.0, omega=omega, mcyc_fine=6, smoo=0.0)
        case.prm.mcyc[0] = 2
        assert (np.abs(case.levels[-1][0].arrays["qb"]).max() > 0.0) == (omega != 0.0)
        _, _, f = OracleCycle(case).solve()
        out[omega] = f
    assert abs(out[0.0].cl) < 1e-10
    # counter-clockwise turning with the stream along +x: the wall moves with the
    # stream below the body, and the lift points down (the Magnus force)
    assert out[0.8].cl < -1e-3
    assert abs(out[0.8].cl + out[-0.8].cl) <= 1e-10 * abs(out[0.8].cl)


def test_symmetry_planes_preserve_the_free_stream():
    # bc_symm.f90:27-82 mirrors the face-normal momentum; with the flow along
    # x the j and k symmetry planes leave the free stream as it is
    case = K.free_stream_box(n=(12, 10, 8), nlevel=1, mach=0.6, bctype=(-20, -50, -50, -20, -50, -50))
    o = OracleCycle(case)
    o.timestep(1)
    o.euler(1, ncyc=1, lres=True)
    assert np.abs(physical(o.field("dw", 1), o.spec(1))).max() < 1e-14
    o.euler(1, ncyc=1)
    assert o.rtrms(1, 1) < 1e-13


def test_symmetry_and_wall_ghosts_follow_the_reference_formulas():
    """After a stage, the face ghosts (tangential indices physical) of a
    symmetry face and a wall face hold exactly the values of bc_symm.f90:
    57-80 and bc_wall.f90:50-86, including the wall's second pressure ghost
    taken from the first physical cell (bc_wall.f90:59-60)."""
    case = K.sphere_box(n=16, nlevel=1, extent=2.0, radius=0.6, mcyc_fine=3,
                        bctype=(-20, -50, -50, -20, -80, -50))
    o = OracleCycle(case)
    o.solve()
    o.timestep(1)
    o.euler_partial(1, 1)
    w, p = o.field("w", 1), o.field("p", 1)
    nx, ny, nz = o.spec(1).n
    il, jl, kl = nx + 1, ny + 1, nz + 1
    I, Kk = slice(2, il + 1), slice(2, kl + 1)
    # face 2, symmetry at j = 1.5: ghosts 1 and 0 mirror cells 2 and 3, v negated
    for g, q in ((1, 2), (0, 3)):
        want = w[:, Kk, q, I].copy()
        want[2] = -want[2]
        assert np.array_equal(w[:, Kk, g, I], want)
        assert np.array_equal(p[Kk, g, I], p[Kk, q, I])
    # face 5, wall at j = jl + 0.5: all three momenta negated
    for g, q in ((jl + 1, jl), (jl + 2, jl - 1)):
        want = w[:, Kk, q, I].copy()
        want[1:4] = -want[1:4]
        assert np.array_equal(w[:, Kk, g, I], want)
        assert np.array_equal(p[Kk, g, I], p[Kk, jl, I])
    # the flow is not trivial there: the walls' momenta are not zero
    assert np.abs(w[1, Kk, jl, I]).min() > 0.0
