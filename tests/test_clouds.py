"""The records' interpolation clouds: trilinear (default) and multiquadric
radial-basis (rbf).  Both reproduce constants exactly.  On a smooth field
both interpolate the reflected point to within a fraction of the field's
change across a cell; the trilinear cloud, which drops its solid corners and
renormalises, is first order there, and the rbf cloud is closer."""
import numpy as np
import pytest

from code_mge_gb300 import cases as K


def _interp_error(case, field):
    sp = case.levels[-1][0]
    a = sp.arrays
    ox, oy, oz = sp.origin
    hx, hy, hz = sp.h
    errs, sums = [], []
    body = case.body
    for m in range(a["nmir"]):
        pts = a["ijkdex"][m, : a["npoint"][m]]
        w = a["coef"][m, : a["npoint"][m]]
        xc = np.stack([ox + (pts[:, 0] - 1.5) * hx, oy + (pts[:, 1] - 1.5) * hy, oz + (pts[:, 2] - 1.5) * hz], axis=1)
        s = a["scid"][m]
        xs = np.array([[ox + (s[0] - 1.5) * hx, oy + (s[1] - 1.5) * hy, oz + (s[2] - 1.5) * hz]])
        xw, n = body.project(xs)
        xr = xs + 2.0 * np.sum((xw - xs) * n, axis=1)[:, None] * n
        if body.kind == "cylinder":
            xr[:, 2] = xs[:, 2]
        errs.append(abs(np.dot(w, field(xc)) - field(xr)[0]))
        sums.append(np.sum(w))
    return np.array(errs), np.array(sums)


def SMOOTH(x):
    return np.sin(x[:, 0]) + np.cos(1.3 * x[:, 1]) + 0.5 * x[:, 2]


@pytest.mark.parametrize("cloud", ["trilinear", "rbf"])
@pytest.mark.parametrize("make", [lambda c: K.cylinder_slab(n=32, span=2, nlevel=1, extent=2.0, mcyc_fine=1, cloud=c),
                                  lambda c: K.sphere_box(n=16, nlevel=1, extent=1.6, mcyc_fine=1, cloud=c)])
def test_clouds_reproduce_constants_and_interpolate_smooth_fields(make, cloud):
    case = make(cloud)
    h = case.levels[-1][0].h[0]
    errs, sums = _interp_error(case, lambda x: 1.0 + 0.0 * x[:, 0])
    assert len(sums) > 0
    assert np.max(np.abs(sums - 1.0)) < 1e-12
    assert np.max(errs) < 1e-12
    # a smooth field whose change across a cell is about h
    errs, _ = _interp_error(case, SMOOTH)
    assert np.max(errs) < 0.6 * h
    assert np.max(case.levels[-1][0].arrays["npoint"]) <= 8


def test_rbf_clouds_take_the_nearest_fluid_cells():
    case = K.cylinder_slab(n=32, span=2, nlevel=1, extent=2.0, mcyc_fine=1, cloud="rbf")
    a = case.levels[-1][0].arrays
    blank = a["blank"].reshape(case.levels[-1][0].dims[::-1])
    for m in range(a["nmir"]):
        for p in a["ijkdex"][m, : a["npoint"][m]]:
            assert blank[p[2], p[1], p[0]] == 1
    assert np.min(a["npoint"][: a["nmir"]]) >= 4


def test_rbf_clouds_interpolate_closer_than_the_renormalised_trilinear_ones():
    med = {}
    for cloud in ("trilinear", "rbf"):
        case = K.cylinder_slab(n=32, span=2, nlevel=1, extent=2.0, mcyc_fine=1, cloud=cloud)
        errs, _ = _interp_error(case, SMOOTH)
        med[cloud] = np.median(errs)
    assert med["rbf"] < 0.5 * med["trilinear"]
