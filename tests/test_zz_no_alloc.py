"""The allocation-free residual norm entry point (mge_residual_norm_noalloc).

Callers that may not call cudaMalloc (a host running inside a stream capture
it does not own, or one held to a fixed device-memory budget) use this entry
point: it computes the residual norm of euler.f90:431-447 from device arrays
the caller passes and keeps its partial sums in a static device array.  This
file is named to be collected last; it passes alone and after the others.
"""
import ctypes as C

import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import cases as K

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # the parity tolerance of the other GPU tests


def test_noalloc_norm_matches_the_cycle_twice(gpulib):
    import torch
    from code_mge_gb300.runtime import Cycle

    case = K.sphere_box(n=24, nlevel=1, extent=3.0, radius=0.7, mcyc_fine=2)
    sp = case.levels[0][0]
    nx, ny, nz = sp.n
    cyc = Cycle(case)
    blank = torch.from_numpy(sp.arrays["blank"].astype(np.int32)).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for ncyc in (1, 2):  # two calls in a row on the shared static scratch
        cyc.timestep(1)
        cyc.euler(1, ncyc=ncyc)
        ref = cyc.rtrms(1, ncyc)
        dw = torch.from_numpy(np.ascontiguousarray(cyc.field("dw", 1)[0])).cuda()
        vd = torch.from_numpy(np.ascontiguousarray(cyc.field("vdtim", 1))).cuda()
        torch.cuda.synchronize()
        rc = gpulib.mge_residual_norm_noalloc(dw.data_ptr(), vd.data_ptr(), blank.data_ptr(), nx, ny, nz,
                                              case.prm.cfl, case.prm.vt, 0.0, out.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == A.MGE_OK
        assert ref > 0.0
        assert abs(out.item() - ref) <= RTOL * abs(ref)
    cyc.close()


def test_noalloc_norm_rejects_oversized_blocks(gpulib):
    import torch
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    b = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc = gpulib.mge_residual_norm_noalloc(d.data_ptr(), d.data_ptr(), b.data_ptr(), 256, 256, 256, 2.8, 0, 0.0,
                                          d.data_ptr(), None)
    assert rc == A.MGE_EBADCFG
