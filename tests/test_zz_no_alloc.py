"""The allocation-free residual norm entry point (mge_residual_norm_noalloc).

Callers that may not call cudaMalloc (a host running inside a stream capture
it does not own, or one held to a fixed device-memory budget) use this entry
point: it computes the residual norm of euler.f90:431-447 from device arrays
the caller passes and keeps its partial sums in a static device array.  Its
reduction has the same fixed partition and order as the cycle's, so its
result is bit-equal to the cycle's rtrms.  This file is named to be collected
last; it passes alone and after the others.
"""
import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import cases as K

pytestmark = pytest.mark.gpu

THREADS = 256          # threads of one partial sum
CELLS_PER_PARTIAL = THREADS * 8
MAX_CELLS = 4096 * CELLS_PER_PARTIAL


def _norm_via_noalloc(gpulib, dw, vd, blank, n, cfl, vt, dtim):
    import torch
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = gpulib.mge_residual_norm_noalloc(dw.data_ptr(), vd.data_ptr(), blank.data_ptr(), n[0], n[1], n[2], cfl, vt,
                                          dtim, out.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == A.MGE_OK
    return out.item()


@pytest.mark.parametrize("cfl", [-2.8, 1.5])  # local (vt = 0) and global (vt = 1) time step
def test_noalloc_norm_matches_the_cycle_twice(gpulib, cfl):
    import torch
    from code_mge_gb300.runtime import Cycle

    case = K.sphere_box(n=24, nlevel=1, extent=3.0, radius=0.7, mcyc_fine=2, cfl=cfl)
    assert case.prm.vt == (0 if cfl < 0 else 1)
    sp = case.levels[0][0]
    cyc = Cycle(case)
    blank = torch.from_numpy(sp.arrays["blank"].astype(np.int32)).cuda()
    for ncyc in (1, 2):  # two calls in a row on the shared static scratch
        cyc.timestep(1)
        cyc.euler(1, ncyc=ncyc)
        ref = cyc.rtrms(1, ncyc)
        dw = torch.from_numpy(np.ascontiguousarray(cyc.field("dw", 1)[0])).cuda()
        vd = torch.from_numpy(np.ascontiguousarray(cyc.field("vdtim", 1))).cuda()
        dtim = float(cyc.field("dtim", 1)) if case.prm.vt else 0.0
        got = _norm_via_noalloc(gpulib, dw, vd, blank, sp.n, case.prm.cfl, case.prm.vt, dtim)
        assert ref > 0.0
        assert got == ref  # the same fixed-order reduction: bit-equal
    cyc.close()


def _fixed_order_norm(dw, vd, blank, n, cfl):
    """numpy restatement of the kernels' fixed-order reduction (vt = 0):
    partial q sums cells [q*per, (q+1)*per) with 256 strided accumulators
    and a halving tree over them; then 32 lanes each add the partials
    l, l+32, ... in turn, and a halving tree over the lanes."""
    nx, ny, nz = n
    tot = nx * ny * nz
    ph = lambda a: a[2:nz + 2, 2:ny + 2, 2:nx + 2].reshape(-1)  # (k, j, i) order: i fastest
    d, v, b = ph(dw), ph(vd), ph(blank)
    rt = np.where(b != 0, d / (cfl * v), 0.0)
    sq = rt * rt
    npart = (tot + CELLS_PER_PARTIAL - 1) // CELLS_PER_PARTIAL
    per = (tot + npart - 1) // npart
    assert per * npart == tot and per % THREADS == 0
    x = sq.reshape(npart, per // THREADS, THREADS)
    acc = np.zeros((npart, THREADS))
    for r in range(x.shape[1]):
        acc = acc + x[:, r, :]
    s = THREADS // 2
    while s > 0:
        acc[:, :s] = acc[:, :s] + acc[:, s:2 * s]
        s //= 2
    lanes = np.zeros(32)
    for q in range(npart):
        lanes[q % 32] = lanes[q % 32] + acc[q, 0]
    s = 16
    while s > 0:
        lanes[:s] = lanes[:s] + lanes[s:2 * s]
        s //= 2
    return float(np.sqrt(lanes[0] / float(tot)))


def test_noalloc_norm_at_the_partial_cap(gpulib):
    """2048 x 2048 x 2 fills all 4096 partial sums of the static array."""
    import torch
    n = (2048, 2048, 2)
    assert n[0] * n[1] * n[2] == MAX_CELLS
    shape = (n[2] + 4, n[1] + 4, n[0] + 4)
    rng = np.random.default_rng(7)
    dw = rng.standard_normal(shape)
    vd = rng.uniform(0.5, 2.0, shape)
    blank = (rng.uniform(size=shape) > 0.1).astype(np.int32)
    want = _fixed_order_norm(dw, vd, blank, n, 2.8)
    tdw, tvd, tb = (torch.from_numpy(a).cuda() for a in (dw, vd, blank))
    for _ in range(2):
        assert _norm_via_noalloc(gpulib, tdw, tvd, tb, n, 2.8, 0, 0.0) == want


def test_noalloc_norm_rejects_oversized_blocks(gpulib):
    import torch
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    b = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc = gpulib.mge_residual_norm_noalloc(d.data_ptr(), d.data_ptr(), b.data_ptr(), 2048, 2048, 3, 2.8, 0, 0.0,
                                          d.data_ptr(), None)
    assert rc == A.MGE_EBADCFG
