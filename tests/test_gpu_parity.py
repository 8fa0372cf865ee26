"""GPU parity: the CUDA path against the CPU oracle on identical inputs.

Tolerance: per-stage residual and state, infinity norm of the difference
relative to the infinity norm of the oracle field, <= 1e-12 (parity.RTOL).
"""
import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import cases as K
from parity import PATHS, RTOL, compare, pair, set_path, small_cylinder, small_sphere

pytestmark = pytest.mark.gpu

CASES = {
    "cylinder": lambda: small_cylinder(),
    "sphere": lambda: small_sphere(),
    "cylinder_matrix": lambda: small_cylinder(dissip=A.MGE_DISSIP_MATRIX),
    "sphere_global_dt": lambda: small_sphere(cfl=1.5),
    "ellipsoid_noirs": lambda: K.ellipsoid_box(n=16, nlevel=2, semi=(0.9, 0.6, 0.5), extent=2.5, alpha_deg=5.0,
                                               smoo=0.0, mcyc_fine=4),
    # Navier-Stokes and Roe (this build's definitions, the reference's sources being absent)
    "cylinder_ns": lambda: small_cylinder(eqntype=A.MGE_EQN_NS, reynolds=40.0, mach=0.2),
    "cylinder_roe1": lambda: small_cylinder(distype=A.MGE_DIS_ROE1),
    "sphere_roe2": lambda: small_sphere(distype=A.MGE_DIS_ROE2),
    "cylinder_ns_roe2": lambda: small_cylinder(eqntype=A.MGE_EQN_NS, distype=A.MGE_DIS_ROE2, reynolds=40.0,
                                               mach=0.2),
    # psmoo + progon3 (variable coefficients) in place of psmoo_old
    "sphere_psmoo": lambda: small_sphere(irs_variant=1),
    "cylinder_psmoo": lambda: small_cylinder(irs_variant=1),
    # a turning wall (the records' qb, bc_cutcell.f90:47-55): Euler reflection about the wall
    # velocity, and the no-slip wall moving with it
    "cylinder_rotating": lambda: small_cylinder(omega=0.8),
    "cylinder_ns_rotating": lambda: small_cylinder(eqntype=A.MGE_EQN_NS, reynolds=40.0, mach=0.2, omega=0.8),
    # multiquadric radial-basis clouds in place of the trilinear ones
    "cylinder_rbf": lambda: small_cylinder(cloud="rbf"),
    "sphere_rbf": lambda: small_sphere(cloud="rbf"),
    # symmetry planes (bc_symm.f90:27-82) on four faces of the box, the flow along x between them
    "sphere_symm": lambda: small_sphere(bctype=(-20, -50, -50, -20, -50, -50)),
    # reflecting walls (bc_wall.f90:28-89) on the j faces, symmetry on the k faces
    "sphere_wall": lambda: small_sphere(bctype=(-20, -80, -50, -20, -80, -50)),
}


@pytest.mark.parametrize("name", list(CASES))
def test_init_flow(gpulib, name):
    g, o = pair(CASES[name]())
    for L in range(1, g.case.prm.nlevel + 1):
        compare(g, o, "w", L, phys_only=False)
        compare(g, o, "p", L, phys_only=False)
        if g.spec(L).arrays["nmir"]:
            compare(g, o, "wsol", L)


@pytest.mark.parametrize("name", list(CASES))
def test_timestep(gpulib, name):
    g, o = pair(CASES[name](), develop_cycles=3)
    L = g.case.prm.nlevel
    g.timestep(L)
    o.timestep(L)
    compare(g, o, "vdtim", L)
    compare(g, o, "lam", L)
    if g.case.prm.irs_variant == 1:
        compare(g, o, "eps", L)
    assert abs(g.field("dtim", L) - o.field("dtim", L)) <= RTOL * abs(o.field("dtim", L))


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("nstage", [1, 2, 3, 4, 5])
def test_stage(gpulib, name, nstage, path):
    g, o = pair(CASES[name](), develop_cycles=3, path=path)
    L = g.case.prm.nlevel
    for c in (g, o):
        c.timestep(L)
        c.euler_partial(L, nstage)
    compare(g, o, "dw", L)
    compare(g, o, "fw", L)
    compare(g, o, "w", L, phys_only=False)
    compare(g, o, "p", L, phys_only=False)
    if g.spec(L).arrays["nmir"]:
        compare(g, o, "wsol", L)


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("name", list(CASES))
def test_euler_rtrms_and_residual(gpulib, name, path):
    g, o = pair(CASES[name](), develop_cycles=3, path=path)
    L = g.case.prm.nlevel
    for c in (g, o):
        c.timestep(L)
        c.euler(L, ncyc=1)
    compare(g, o, "w", L, phys_only=False)
    rg, ro = g.rtrms(L, 1), o.rtrms(L, 1)
    assert abs(rg - ro) <= RTOL * abs(ro)
    for c in (g, o):
        c.euler(L, ncyc=1, lres=True)
    compare(g, o, "dw", L)


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("name", ["cylinder", "sphere"])
def test_transfer(gpulib, name, path):
    g, o = pair(CASES[name](), develop_cycles=3, path=path)
    L = g.case.prm.nlevel
    for c in (g, o):
        c.timestep(L)
        c.euler(L, ncyc=1, mgl=L, mlvl=L)
        c.euler(L, ncyc=1, mgl=L, mlvl=L, lres=True)
        c.movco(L - 1)
    for f in ("w", "wr", "p"):
        compare(g, o, f, L - 1, phys_only=(f == "wr"))
    for c in (g, o):
        c.timestep(L - 1)
        c.euler(L - 1, ncyc=1, mgl=L - 1, mlvl=L, lfir=True)
        c.movfin(L, L)
    compare(g, o, "qf", L - 1)
    compare(g, o, "w", L, phys_only=False)
    compare(g, o, "p", L, phys_only=False)


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("name,mgtype", [("cylinder", 1), ("sphere", 2), ("cylinder_ns", 1), ("cylinder_ns_rotating", 1)])
def test_solve(gpulib, name, mgtype, path):
    case = CASES[name]()
    case.prm.mgtype = mgtype
    case.prm.mcyc[0] = 2
    case.prm.mcyc[case.prm.nlevel - 1] = 5
    g, o = pair(case, path=path)
    hg, ng, fg = g.solve(use_graph=1)
    ho, no, fo = o.solve()
    assert ng == no
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
    L = case.prm.nlevel
    compare(g, o, "w", L, rtol=1e-11, phys_only=False)
    assert abs(fg.cd - fo.cd) <= 1e-9 * max(1.0, abs(fo.cd))
    assert abs(fg.cl - fo.cl) <= 1e-9 * max(1.0, abs(fo.cd))


@pytest.mark.parametrize("path", PATHS)
def test_graph_matches_stream(gpulib, path):
    set_path(path)
    case = small_sphere(nlevel=3, n=16, mgtype=2)
    case.prm.mcyc[0] = 1
    case.prm.mcyc[1] = 1
    case.prm.mcyc[2] = 4
    from code_mge_gb300.runtime import Cycle
    a = Cycle(case)
    b = Cycle(case)
    ha, _, _ = a.solve(use_graph=1)
    hb, _, _ = b.solve(use_graph=0)
    assert np.array_equal(ha, hb)
    assert np.array_equal(a.field("w", 3), b.field("w", 3))


EMBEDDED = {
    "jst": dict(mach=0.3),
    # the scheme of the 512x512x2 NS cylinder workload: Roe MUSCL + viscous fluxes
    "ns_roe2": dict(mach=0.2, eqntype=A.MGE_EQN_NS, distype=A.MGE_DIS_ROE2, reynolds=40.0),
}


@pytest.mark.parametrize("scheme", sorted(EMBEDDED))
@pytest.mark.parametrize("path", PATHS)
def test_embedded_levels(gpulib, path, scheme):
    case = K.cylinder_embedded(n=24, span=2, nlevel=3, h_fine=0.1, mcyc_fine=3, **EMBEDDED[scheme])
    case.prm.mcyc[0] = 1
    case.prm.mcyc[1] = 1
    g, o = pair(case, path=path)
    hg, ng, _ = g.solve()
    ho, no, _ = o.solve()
    assert ng == no
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
    compare(g, o, "w", 3, rtol=1e-11, phys_only=False)
    compare(g, o, "w", 2, rtol=1e-11, phys_only=False)


def test_mixed_paths_in_one_hierarchy(gpulib):
    """Coarse levels cooperative, finest per-phase: the split the 192^3 bench uses."""
    import os
    case = small_sphere(nlevel=3, n=32, mgtype=2)
    case.prm.mcyc[0] = 1
    case.prm.mcyc[1] = 1
    case.prm.mcyc[2] = 3
    os.environ["MGE_COOP_MAX_CELLS"] = str(16 ** 3)
    try:
        from code_mge_gb300.runtime import Cycle
        from oracle.oracle import OracleCycle
        g = Cycle(case)
        o = OracleCycle(case)
    finally:
        os.environ.pop("MGE_COOP_MAX_CELLS", None)
    from code_mge_gb300.runtime import load_library
    import ctypes as C
    lib = load_library()
    for L, expect in ((1, 1), (2, 1), (3, 0)):
        coop = C.c_int(-1)
        irs = (C.c_int * 3)()
        assert lib.mge_tuned(g.ctx, L, 1, C.byref(coop), irs) == 0
        assert coop.value == expect
    hg, _, _ = g.solve()
    ho, _, _ = o.solve()
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
    compare(g, o, "w", 3, rtol=1e-11, phys_only=False)


@pytest.mark.parametrize("path", PATHS)
def test_same_level_overlap(gpulib, path):
    """Two fine blocks of one level that share 4 cells around the body
    (bc_overlap.f90:32-90 after every block's update, in movco and in
    movfin): whole solve, both blocks' states, against the oracle."""
    case = K.cylinder_split(n=32, overlap=4, mcyc_fine=4)
    g, o = pair(case, path=path)
    hg, ng, fg = g.solve()
    ho, no, fo = o.solve()
    assert ng == no
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
    for s in (1, 2):
        a, b = g.field("w", 2, serial=s), o.field("w", 2, serial=s)
        assert np.max(np.abs(a - b)) <= 1e-11 * np.max(np.abs(b))
    assert abs(fg.cd - fo.cd) <= 1e-9 * max(1.0, abs(fo.cd))
    # the entry point alone, on the solved states
    assert gpulib.mge_bc_overlap(g.ctx, 2) == 0 and o.lib.mgeo_bc_overlap(o.ctx, 2) == 0
    for s in (1, 2):
        a, b = g.field("w", 2, serial=s), o.field("w", 2, serial=s)
        assert np.max(np.abs(a - b)) <= 1e-11 * np.max(np.abs(b))
