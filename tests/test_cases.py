"""The synthetic-case preprocessor: blanking and cut-cell record invariants."""
import numpy as np
import pytest

from code_mge_gb300 import cases as K
from code_mge_gb300 import schedule as S


@pytest.mark.parametrize("mk", [
    lambda: K.cylinder_slab(n=32, span=2, nlevel=2, extent=4.0),
    lambda: K.sphere_box(n=24, nlevel=2, extent=3.0, radius=0.8),
    lambda: K.ellipsoid_box(n=24, nlevel=2, semi=(1.2, 0.7, 0.5), extent=3.0),
])
def test_records(mk):
    case = mk()
    for L in case.levels:
        for sp in L:
            a = sp.arrays
            P = sp.dims
            bl = a["blank"].reshape(P[2], P[1], P[0])
            nm = a["nmir"]
            for m in range(nm):
                ci, cj, ck = a["ccid"][m]
                si, sj, sk = a["scid"][m]
                assert bl[ck, cj, ci] == 1 and bl[sk, sj, si] == 0
                d = np.array([si - ci, sj - cj, sk - ck])
                assert np.abs(d).sum() == 1
                ax = int(np.nonzero(d)[0][0])
                assert a["zz"][m] == ax + 1
                assert a["faceid"][m] == ax + 1 + (3 if d[ax] > 0 else 0)
                npnt = a["npoint"][m]
                assert 1 <= npnt <= 8
                assert abs(a["coef"][m, :npnt].sum() - 1.0) < 1e-13
                for q in range(npnt):
                    x, y, z = a["ijkdex"][m, q]
                    assert bl[z, y, x] == 1
                assert abs(np.linalg.norm(a["nvec"][m]) - 1.0) < 1e-12
            # records are ordered by cut cell (Fortran order) then face
            key = [(c[0] + P[0] * (c[1] + P[1] * c[2]), f) for c, f in zip(a["ccid"], a["faceid"])]
            assert key == sorted(key)


def test_blank_ghost_copies():
    case = K.sphere_box(n=16, nlevel=1, extent=1.0, radius=0.9)
    sp = case.levels[0][0]
    P = sp.dims
    bl = sp.arrays["blank"].reshape(P[2], P[1], P[0])
    assert (bl[:, :, 0] == bl[:, :, 2]).all() and (bl[:, :, -1] == bl[:, :, -3]).all()
    assert (bl[0] == bl[2]).all() and (bl[-2] == bl[-3]).all()
    assert (bl == 0).sum() > 0


def test_cycle_visits():
    assert S.cycle_visits(4, 2)[0][1:5] == [4, 6, 3, 1]
    assert S.cycle_visits(4, 2)[1][1:5] == [0, 4, 2, 1]
    assert S.cycle_visits(3, 1)[0][1:4] == [1, 2, 1]
    case = K.sphere_box(n=192, nlevel=4, extent=10.0, mgtype=2)
    assert S.cell_updates_per_cycle(case) == 192 ** 3 + 3 * 96 ** 3 + 6 * 48 ** 3 + 4 * 24 ** 3
    # the NS cylinder workload: 4 embedded levels of 512x512x2 cells, V-cycle
    # (finest and coarsest once, the middle levels twice)
    assert S.cycle_visits(4, 1)[0][1:5] == [1, 2, 2, 1]
    cyl = K.cylinder_embedded(n=512, span=2, nlevel=4, h_fine=1.0 / 96.0, mach=0.2)
    assert cyl.cells_per_level() == [512 * 512 * 2] * 4
    assert S.cell_updates_per_cycle(cyl) == 6 * 512 * 512 * 2
