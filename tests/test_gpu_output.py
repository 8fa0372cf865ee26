"""Solution output on the device path: upload_solut (upload_solut.f90:203-237)
against the oracle's restatement, and the restart text written from the
device state and read back into another context."""
import ctypes as C

import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import cases as K
from parity import RTOL, pair, rel_err, small_cylinder, small_sphere

pytestmark = pytest.mark.gpu


def _solut(cyc, level, p_tot):
    sp = cyc.spec(level)
    n = sp.n[0] * sp.n[1] * sp.n[2]
    out = np.zeros(11 * n)
    nval = C.c_int(0)
    rc = cyc._fn("upload_solut")(cyc.ctx, level, 1, p_tot, out.ctypes.data_as(C.POINTER(C.c_double)), out.size,
                                 C.byref(nval))
    assert rc == 0
    return out[: nval.value * n].reshape(nval.value, n)


@pytest.mark.parametrize("mk,nval", [
    (lambda: small_sphere(), 7),
    (lambda: small_cylinder(eqntype=A.MGE_EQN_NS, reynolds=40.0, mach=0.2), 11),
])
def test_upload_solut_matches_the_oracle(gpulib, mk, nval):
    g, o = pair(mk(), develop_cycles=3)
    L = g.case.prm.nlevel
    prm = g.case.prm
    p_tot = prm.p0 * (1.0 + 0.2 * prm.rm ** 2) ** 3.5
    a, b = _solut(g, L, p_tot), _solut(o, L, p_tot)
    assert a.shape[0] == nval
    for q in range(nval):
        assert rel_err(a[q], b[q]) <= RTOL, q
    # cp and mach of the developed flow are not trivial
    assert np.ptp(a[4]) > 1e-3 and np.ptp(a[5]) > 1e-3


def test_restart_round_trip(gpulib, tmp_path):
    from code_mge_gb300.runtime import Cycle, physical
    case = small_sphere()
    g = Cycle(case)
    g.solve(max_cycles_total=5)
    path = str(tmp_path / "job_restart.dat").encode()
    nb = sum(len(L) for L in case.levels)
    codes = (C.c_int * nb)(*[100 + q for q in range(nb)])
    assert gpulib.mge_write_restart(g.ctx, path, codes, nb) == 0
    h = Cycle(small_sphere())
    assert gpulib.mge_read_restart(h.ctx, path, codes, nb) == 0
    for L in range(1, case.prm.nlevel + 1):
        # the physical cells as written (F16.7); the ghost cells then come
        # from bc_cutcell and bcond, as init_flow.f90:46-66 applies them
        # after read_solut
        want = np.vectorize(lambda x: float("%.7f" % x))(g.field("w", L))
        sp = case.levels[L - 1][0]
        assert np.array_equal(physical(h.field("w", L), sp), physical(want, sp))
    # another block code: the reference stops (rsolut.f90:27-32)
    bad = (C.c_int * nb)(*[200 + q for q in range(nb)])
    assert gpulib.mge_read_restart(h.ctx, path, bad, nb) == A.MGE_EBADCFG
    # another grid: the dimensions differ
    other = Cycle(K.sphere_box(n=12, nlevel=2, extent=3.0, radius=0.7, mgtype=1))
    assert gpulib.mge_read_restart(other.ctx, path, codes, nb) == A.MGE_EBADCFG
    for c in (g, h, other):
        c.close()
