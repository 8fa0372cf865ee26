"""Same-level overlap (bc_overlap.f90:32-90) in the oracle, on CPU.

Blocks of one level that overlap exchange their ghost cells: a ghost cell
of one block whose centre lies in another block's physical cells takes the
trilinear interpolation of that block's state.  The reference's helpers
for it (cell_center, eval_x2cell, shft_cell) are in its absent library; the
build uses the construction of its prolongation.  Pinned here by exactness
on linear fields and by free-stream preservation.
"""
import numpy as np

from code_mge_gb300 import cases as K
from code_mge_gb300.runtime import physical
from oracle.oracle import OracleCycle


def _centres(spec):
    P = spec.dims
    ax = [spec.origin[d] + (np.arange(P[d]) - 1.5) * spec.h[d] for d in range(3)]
    return np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")[::-1]  # x, y, z in [k, j, i] order


def test_ghost_cells_interpolate_linear_fields_exactly():
    case = K.cylinder_split(n=32, overlap=4)
    o = OracleCycle(case)
    a, b = case.levels[1]
    coef = np.array([[1.0, 0.3, -0.2, 0.05], [0.1, 0.7, 0.2, 0.0], [0.0, 0.2, -0.4, 0.0],
                     [0.0, 0.0, 0.0, 0.3], [2.5, -0.1, 0.3, 0.02]])
    for s, spec in enumerate((a, b), start=1):
        x, y, z = _centres(spec)
        w = np.stack([c[0] + c[1] * x + c[2] * y + c[3] * z for c in coef])
        o.upload(w, 2, serial=s)
    assert o.lib.mgeo_bc_overlap(o.ctx, 2) == 0
    for s, spec in enumerate((a, b), start=1):
        x, y, z = _centres(spec)
        want = np.stack([c[0] + c[1] * x + c[2] * y + c[3] * z for c in coef])
        got = o.field("w", 2, serial=s)
        # the ghost layers along x that lie inside the other block
        side = (slice(None), slice(2, -2), slice(2, -2))
        cols = [-2, -1] if s == 1 else [0, 1]
        for q in cols:
            np.testing.assert_allclose(got[side + (q,)], want[side + (q,)], rtol=0, atol=1e-13)


def test_split_level_preserves_the_free_stream():
    case = K.cylinder_split(n=32, overlap=4)
    for row in case.levels:
        for spec in row:
            blank = spec.arrays["blank"]
            blank[:] = 1
            spec.arrays["nmir"] = 0
    o = OracleCycle(case)
    o.solve()
    for s in (1, 2):
        w = physical(o.field("w", 2, serial=s), case.levels[1][s - 1])
        assert np.abs(w[0] - 1.0).max() < 1e-12


def test_wall_faces_of_overlapping_blocks_count_once():
    """At the free stream the pressure is uniform, so the wall force of a
    closed body is zero only if every wall face counts exactly once: the
    faces inside the overlap belong to the block of lower serial."""
    import ctypes as C
    from code_mge_gb300 import _abi as A
    case = K.cylinder_split(n=32, overlap=4)
    o = OracleCycle(case)
    opts = A.MgeSolveOpts()
    opts.ref_area = case.ref_area
    f = A.MgeForces()
    assert o.lib.mgeo_forces_compute(o.ctx, 2, C.byref(opts), C.byref(f)) == 0
    assert max(abs(v) for v in f.force) < 1e-12 * case.prm.p0
