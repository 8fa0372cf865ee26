"""The uniform block metric the library is given, against a restatement of
the reference's init_metric.f90 on the same node grid (CPU only).

init_metric.f90:56-72 places node (i,j,k) at ori + cm*(icel-2); the cell
centre of :80-104 is the mean of its eight nodes; the face vectors of
:111-177 are half the cross products of the face diagonals.  The library
takes the face vectors, the cell volume and the cell centres of
code_mge_gb300/cases.py, and the GPU and the oracle share them, so a sign
or a factor of 1/2 wrong there would pass every parity test; this test
checks them against the reference's own construction instead.
"""
import numpy as np
import pytest

from code_mge_gb300 import cases as K


def _nodes(spec):
    """b%x(1:ib,1:jb,1:kb,:) of init_metric.f90:56-72 with cm = diag(h)."""
    nx, ny, nz = spec.n
    ib, jb, kb = nx + 3, ny + 3, nz + 3
    x = np.zeros((ib + 1, jb + 1, kb + 1, 3))
    for d, (m, o, h) in enumerate(zip((ib, jb, kb), spec.origin, spec.h)):
        idx = np.arange(1, m + 1, dtype=np.float64)
        shape = [1, 1, 1]
        shape[d] = m
        x[1:, 1:, 1:, d] = (h * (idx - 2.0) + o).reshape(shape)
    return x


def _cross_half(x1, x2):
    return 0.5 * np.stack([x1[..., 1] * x2[..., 2] - x1[..., 2] * x2[..., 1],
                           x1[..., 2] * x2[..., 0] - x1[..., 0] * x2[..., 2],
                           x1[..., 0] * x2[..., 1] - x1[..., 1] * x2[..., 0]], axis=-1)


def _face_vectors(x):
    """si, sj, sk of init_metric.f90:111-177 for i, j, k in 1..ie (the
    interior loops; index 0 reads the unset node layer 0)."""
    X = lambda di, dj, dk: x[1 + di:x.shape[0] - 1 + di, 1 + dj:x.shape[1] - 1 + dj, 1 + dk:x.shape[2] - 1 + dk]
    si = _cross_half(X(0, 1, 0) - X(0, 0, 1), X(0, 0, 0) - X(0, 1, 1))
    sj = _cross_half(X(1, 0, 0) - X(0, 0, 1), X(1, 0, 1) - X(0, 0, 0))
    sk = _cross_half(X(1, 1, 0) - X(0, 0, 0), X(1, 0, 0) - X(0, 1, 0))
    return si, sj, sk


SPECS = {
    "cube": lambda: K.sphere_box(n=8, nlevel=1, extent=2.0).levels[0][0],
    "slab": lambda: K.cylinder_slab(n=16, span=2, nlevel=1, extent=4.0).levels[0][0],
    "stretched": lambda: K.BlockSpec(n=(6, 5, 4), h=(0.3, 0.7, 1.9), origin=(-1.0, 0.5, 2.0), bctype=(-20,) * 6),
}


@pytest.mark.parametrize("name", sorted(SPECS))
def test_face_vectors_volume_and_centres(name):
    spec = SPECS[name]()
    x = _nodes(spec)
    si, sj, sk = _face_vectors(x)
    d = K.block_desc(spec) if spec.arrays else None
    hx, hy, hz = spec.h
    want_si = np.array(d.si[:]) if d else np.array((-(hy * hz), 0.0, 0.0))
    want_sj = np.array(d.sj[:]) if d else np.array((0.0, -(hx * hz), 0.0))
    want_sk = np.array(d.sk[:]) if d else np.array((0.0, 0.0, -(hx * hy)))
    # every face of the block has the descriptor's vector, to rounding of the
    # node coordinates' differences
    tol = 1e-12 * max(hx * hy, hy * hz, hx * hz)
    for got, want in ((si, want_si), (sj, want_sj), (sk, want_sk)):
        assert np.abs(got - want).max() <= tol
    # the face vectors point to -x, -y, -z: dw = F(i) - F(i+1) is the net outflow
    assert want_si[0] < 0 and want_sj[1] < 0 and want_sk[2] < 0
    # the closed cell: the six face vectors of a cell sum to zero, and the
    # cell volume is the box the nodes span
    assert np.abs(si[:-1] - si[1:]).max() <= tol
    if d:
        assert abs(d.cellvolume - hx * hy * hz) <= 1e-15 * hx * hy * hz
    # cell centres (init_metric.f90:80-104): the mean of the eight nodes,
    # the positions cases.py blanks cells by (origin + (i - 1.5) h)
    xc = 0.125 * sum(x[1 + a:x.shape[0] - 1 + a, 1 + b:x.shape[1] - 1 + b, 1 + c:x.shape[2] - 1 + c]
                     for a in (0, 1) for b in (0, 1) for c in (0, 1))
    for dd, (o, h) in enumerate(zip(spec.origin, spec.h)):
        idx = np.arange(1, xc.shape[dd] + 1, dtype=np.float64)
        shape = [1, 1, 1]
        shape[dd] = xc.shape[dd]
        ref = (o + (idx - 1.5) * h).reshape(shape)
        assert np.abs(xc[..., dd] - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
