"""Mixed precision: FP32 coarse levels, FP32 time step and residual smoothing
on the finest level, FP64 finest residual, update, norm and forces.  The
multigrid then acts as a defect correction: the converged answer must match
the FP64 plain solve (and hence the FP64 oracle) to the stated tolerance."""
import ctypes as C

import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import cases as K

pytestmark = pytest.mark.gpu

CD_TOL = 1e-6   # |dCd| of the converged mixed solve against the FP64 plain one


def _solve(case, precision, cycles):
    from code_mge_gb300.runtime import Cycle
    case.prm.precision = precision
    case.prm.conv_drop = 1e8       # converge to an 8-decade residual drop (or `cycles`)
    case.prm.mcyc[case.prm.nlevel - 1] = cycles
    g = Cycle(case)
    # mixed: FP32 coarse corrections until a 1e-6 drop, then FP64 to the end
    hist, n, f = g.solve(refine_drop=1e-6 if precision == A.MGE_PREC_MIXED else 0.0)
    w = g.field("w", case.prm.nlevel)
    g.close()
    return hist, f, w


@pytest.mark.parametrize("mk,cycles", [
    (lambda: K.sphere_box(n=24, nlevel=3, extent=4.0, radius=0.7, mgtype=2), 3000),
    (lambda: K.cylinder_slab(n=48, span=2, nlevel=3, extent=6.0, mach=0.3, smoo=0.6), 3000),
])
def test_mixed_converges_to_the_fp64_answer(gpulib, mk, cycles):
    c1, c2 = mk(), mk()
    for c in (c1, c2):
        for L in range(c.prm.nlevel - 1):
            c.prm.mcyc[L] = 5
    h64, f64, w64 = _solve(c1, A.MGE_PREC_FP64, cycles)
    h32, f32, w32 = _solve(c2, A.MGE_PREC_MIXED, cycles)
    # both reach the 8-decade drop; the mixed answer keeps FP64 accuracy
    assert h64[-1] / h64[0] < 1e-8
    assert h32[-1] / h32[0] < 1e-8
    assert abs(f32.cd - f64.cd) <= CD_TOL
    assert abs(f32.cl - f64.cl) <= CD_TOL
    assert np.max(np.abs(w32 - w64)) / np.max(np.abs(w64)) < 1e-6


def test_mixed_levels_precision(gpulib):
    from code_mge_gb300.runtime import Cycle
    case = K.sphere_box(n=16, nlevel=2, extent=3.0, radius=0.7, mgtype=1, precision=A.MGE_PREC_MIXED)
    g = Cycle(case)
    g.solve()
    wc = g.field("w", 1)
    wf = g.field("w", 2)
    # coarse level values are FP32-representable, the finest level is not restricted to them
    assert np.array_equal(wc, wc.astype(np.float32).astype(np.float64))
    assert not np.array_equal(wf, wf.astype(np.float32).astype(np.float64))


def test_precision_switch_round_trip(gpulib):
    from code_mge_gb300.runtime import Cycle
    case = K.sphere_box(n=16, nlevel=2, extent=3.0, radius=0.7, mgtype=1)
    g = Cycle(case)
    g.solve()
    w1 = g.field("w", 1).copy()
    assert gpulib.mge_set_precision(g.ctx, A.MGE_PREC_MIXED) == 0
    assert np.array_equal(g.field("w", 1), w1.astype(np.float32).astype(np.float64))
    assert gpulib.mge_set_precision(g.ctx, A.MGE_PREC_FP64) == 0
    r = g.cycle(2)
    assert np.isfinite(r)


@pytest.mark.parametrize("mk", [
    lambda: K.sphere_box(n=24, nlevel=2, extent=3.0, radius=0.7, mgtype=1, precision=A.MGE_PREC_MIXED),
    lambda: K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0, precision=A.MGE_PREC_MIXED),
])
def test_contracted_residual_is_the_fp64_residual(gpulib, monkeypatch, mk):
    """The mixed form's finest level evaluates the JST residual in its
    contracted FP64 form (fused multiply-adds, central differences of the
    cell fluxes).  On the same state, with the same FP32 time step, its dw,
    fw and updated state agree with the reference form's to FP64 rounding:
    relative to the field's largest value, 1e-10 on dw and fw (the residual
    is a difference of fluxes up to 1e4 times larger) and 1e-10 on w (the
    FP32 line sweeps round the two updates apart by an FP32 ulp of the
    update, itself some 1e-4 of the state); an FP32 residual would differ
    by 1e-7 of the residual."""
    from code_mge_gb300.runtime import Cycle, physical
    from parity import rel_err
    case = mk()
    L = case.prm.nlevel
    dev = Cycle(case)
    for _ in range(4):
        dev.cycle(L, ncyc=1)
    w0 = dev.field("w", L)
    dev.close()
    monkeypatch.setenv("MGE_FAST_RESIDUAL", "0")
    ref = Cycle(case)
    monkeypatch.delenv("MGE_FAST_RESIDUAL")
    fast = Cycle(case)
    sp = ref.spec(L)
    for lres in (True, False):
        for c in (ref, fast):
            c.upload(w0, L)
            c.timestep(L)
            c.euler(L, ncyc=1, lres=lres)
        for f in ("dw", "fw"):
            a, b = physical(fast.field(f, L), sp), physical(ref.field(f, L), sp)
            assert rel_err(a, b) <= 1e-10, (lres, f, rel_err(a, b))
        if lres:  # a different evaluation, not the same bits
            assert not np.array_equal(fast.field("dw", L), ref.field("dw", L))
    assert rel_err(fast.field("w", L), ref.field("w", L)) <= 1e-10
    ref.close()
    fast.close()


def test_warp_scan_sweeps_agree_with_the_line_sweeps(gpulib, monkeypatch):
    """The FP32 i sweep as a warp scan of affine row maps (launch-form digit 2),
    on the mixed form's finest level and in place on its FP32 coarse levels,
    against the sequential line sweeps (digit 0).  Both round in FP32, in a
    different order.  The scan must move the solve by about as much as the
    mixed form's FP32 arithmetic moves it from the FP64 solve of the same
    case: the early cycles amplify any rounding difference alike, so the two
    differences are of one order, and the test allows a factor of 10."""
    from code_mge_gb300.runtime import Cycle
    make = lambda prec: K.sphere_box(n=32, nlevel=3, extent=3.0, radius=0.7, mgtype=2, mcyc_fine=8, precision=prec)
    runs = []
    for digit in "02":
        monkeypatch.setenv("MGE_TUNE_PLAN", ",".join("%d:0%s00" % (L, digit) for L in (1, 2, 3)))
        g = Cycle(make(A.MGE_PREC_MIXED))
        tuned = []
        for L in (1, 2, 3):
            coop = C.c_int()
            irs = (C.c_int * 3)()
            assert gpulib.mge_tuned(g.ctx, L, 1, C.byref(coop), irs) == A.MGE_OK
            tuned.append(irs[0])
        hist, n, fo = g.solve()
        runs.append((tuned, hist, g.field("w", 3), fo.cd))
        g.close()
    monkeypatch.delenv("MGE_TUNE_PLAN")
    g = Cycle(make(A.MGE_PREC_FP64))
    h64, _, f64 = g.solve()
    w64 = g.field("w", 3)
    g.close()
    (t0, h0, w0, cd0), (t2, h2, w2, cd2) = runs
    assert t0 == [0, 0, 0] and t2 == [2, 2, 2]
    assert len(h0) == len(h2) == len(h64) > 0
    assert not np.array_equal(h0, h2)  # the scan ran, and rounds differently
    ratios = (np.max(np.abs(h2 - h0)) / np.max(np.abs(h0 - h64)),
              np.max(np.abs(w2 - w0)) / np.max(np.abs(w0 - w64)),
              abs(cd2 - cd0) / max(abs(cd0 - f64.cd), 1e-7 * abs(cd0)))
    assert max(ratios) < 10.0, ratios
