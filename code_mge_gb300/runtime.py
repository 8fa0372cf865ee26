"""Python host mirror of the reference's solver interface, over the C-ABI.

``Cycle`` drives one case through the entry points of include/mge_gpu.h with
the names and argument meaning of the reference's Fortran routines
(timestep, euler, movco, movfin, solver).  It takes the loaded library and
its symbol prefix, so the same driver runs the GPU library (prefix ``mge_``)
and, in the tests, the CPU oracle (prefix ``mgeo_``).
"""
import ctypes as C
import os

import numpy as np

from . import _abi as A
from . import cases as K

_LIB = None


class MgeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (A.error_name(code), msg))
        self.code = code


def library_path():
    return os.path.join(A.PACKAGE_DIR, "_build", "libmge_gpu.so")


def load_library():
    """Load the GPU library built in-tree; fail loudly if it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            "libmge_gpu.so not built (%s); run code_mge_gb300.build.build() - there is no CPU fallback" % path)
    lib = C.CDLL(path)
    A.bind(lib, "mge_", A.SIGNATURES)
    A.bind(lib, "mge_", A.PRODUCT_ONLY)
    if lib.mge_abi_version() != A.MGE_ABI_VERSION:
        raise RuntimeError("libmge_gpu.so ABI mismatch: library %d, bindings %d" % (lib.mge_abi_version(),
                                                                                    A.MGE_ABI_VERSION))
    _LIB = lib
    return lib


class Cycle:
    """One case resident in the library (one mge_ctx)."""

    def __init__(self, case: "K.Case", lib=None, prefix="mge_", device=0, init_flow=True, prm=None):
        self.case = case
        self.lib = lib if lib is not None else load_library()
        self.prefix = prefix
        self._descs = case.descs()
        self.prm = prm if prm is not None else case.prm
        ctx = C.c_void_p()
        if prefix == "mge_":
            rc = self._fn("init")(C.byref(self.prm), device, C.byref(ctx))
        else:
            rc = self._fn("init")(C.byref(self.prm), C.byref(ctx))
        if rc != 0:
            raise MgeError(rc, "init failed")
        self.ctx = ctx
        for L, descs in enumerate(self._descs):
            for s, d in enumerate(descs):
                self._chk(self._fn("add_block")(self.ctx, C.byref(d), L + 1, s + 1), "add_block")
        self._chk(self._fn("commit")(self.ctx), "commit")
        if init_flow:
            self.init_flow()

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def _chk(self, rc, what):
        if rc != 0:
            msg = self._fn("last_error")(self.ctx) if getattr(self, "ctx", None) else b""
            raise MgeError(rc, "%s: %s" % (what, (msg or b"").decode(errors="replace")))
        return rc

    # ------------------------------------------------------------ the reference's routines
    def init_flow(self):
        return self._chk(self._fn("init_flow")(self.ctx), "init_flow")

    def timestep(self, level, serial=1):
        return self._chk(self._fn("timestep")(self.ctx, level, serial), "timestep")

    def euler(self, level, serial=1, itime=0, ncyc=1, mgl=None, mlvl=None, lres=False, lfir=False):
        mgl = level if mgl is None else mgl
        mlvl = level if mlvl is None else mlvl
        return self._chk(self._fn("euler")(self.ctx, level, serial, itime, ncyc, mgl, mlvl, int(lres), int(lfir)),
                         "euler")

    def euler_partial(self, level, nstage, serial=1, itime=0, ncyc=1, mgl=None, mlvl=None, lres=False, lfir=False):
        mgl = level if mgl is None else mgl
        mlvl = level if mlvl is None else mlvl
        return self._chk(self._fn("euler_partial")(self.ctx, level, serial, itime, ncyc, mgl, mlvl, int(lres),
                                                   int(lfir), nstage), "euler_partial")

    def movco(self, mgl):
        return self._chk(self._fn("movco")(self.ctx, mgl), "movco")

    def movfin(self, mgl, mlvl):
        return self._chk(self._fn("movfin")(self.ctx, mgl, mlvl), "movfin")

    def rtrms(self, level, ncyc, serial=1):
        out = C.c_double()
        self._chk(self._fn("get_rtrms")(self.ctx, level, serial, ncyc, C.byref(out)), "get_rtrms")
        return out.value

    def solve(self, max_cycles_total=0, hist_len=100000, use_graph=1, refine_drop=0.0):
        hist = np.zeros(hist_len, dtype=np.float64)
        nd = C.c_int(0)
        fo = A.MgeForces()
        o = A.MgeSolveOpts()
        o.max_cycles_total = max_cycles_total
        o.ref_area = self.case.ref_area
        o.moment_center[:] = (0.0, 0.0, 0.0)
        o.use_graph = use_graph
        o.refine_drop = refine_drop
        self._chk(self._fn("solve")(self.ctx, C.byref(o), hist.ctypes.data_as(C.POINTER(C.c_double)), hist_len,
                                    C.byref(nd), C.byref(fo)), "solve")
        return hist[: min(nd.value, hist_len)].copy(), nd.value, fo

    def time_advance(self):
        """End of a physical time step of the unsteady mode (solver.f90:263-276):
        w2 = w1, w1 = w; returns the new step counter."""
        it = C.c_int(0)
        self._chk(self._fn("time_advance")(self.ctx, C.byref(it)), "time_advance")
        return it.value

    def move_surface(self, level, disp, norv, vel, vel_fs, serial=1):
        """movsurf.f90:28-35 for one block: per record pnew = psurf + disp, the
        wall normal norv and the wall velocity vel/vel_fs ([nmir, 3] arrays in
        record order)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (disp, norv, vel)]
        nm = self.spec(level, serial).arrays["nmir"]
        for a in arrs:
            if a.shape != (nm, 3):
                raise ValueError("move_surface: arrays must be [%d, 3]" % nm)
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        return self._chk(self._fn("move_surface")(self.ctx, level, serial, ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]),
                                                  float(vel_fs)), "move_surface")

    def surface(self, level, serial=1):
        """The records' moved points pnew, [nmir, 3]."""
        nm = self.spec(level, serial).arrays["nmir"]
        out = np.zeros((max(nm, 1), 3))
        self._chk(self._fn("get_surface")(self.ctx, level, serial, out.ctypes.data_as(C.POINTER(C.c_double))),
                  "get_surface")
        return out[:nm]

    def forces(self, level=None):
        level = self.case.prm.nlevel if level is None else level
        o = A.MgeSolveOpts()
        o.ref_area = self.case.ref_area
        fo = A.MgeForces()
        self._chk(self._fn("forces_compute")(self.ctx, level, C.byref(o), C.byref(fo)), "forces_compute")
        return fo

    # ------------------------------------------------------------ data movement
    def spec(self, level, serial=1):
        return self.case.levels[level - 1][serial - 1]

    def field(self, name, level, serial=1):
        sp = self.spec(level, serial)
        P = sp.dims
        N = P[0] * P[1] * P[2]
        nvar = 5 if name in ("w", "dw", "fw", "wn", "ws", "wr", "qf", "w1", "w2") else (3 if name == "eps" else 1)
        if name in ("wsol", "psol"):
            nm = sp.arrays["nmir"]
            n = 5 * nm if name == "wsol" else nm
            out = np.zeros(max(n, 1), dtype=np.float64)
            self._chk(self._fn("download_field")(self.ctx, level, serial, name.encode(),
                                                 out.ctypes.data_as(C.POINTER(C.c_double)), out.size), "download")
            return out[:n].reshape((nm, 5)) if name == "wsol" else out[:n]
        if name == "dtim":
            out = np.zeros(1, dtype=np.float64)
            self._chk(self._fn("download_field")(self.ctx, level, serial, b"dtim",
                                                 out.ctypes.data_as(C.POINTER(C.c_double)), 1), "download")
            return float(out[0])
        out = np.zeros(nvar * N, dtype=np.float64)
        self._chk(self._fn("download_field")(self.ctx, level, serial, name.encode(),
                                             out.ctypes.data_as(C.POINTER(C.c_double)), out.size), "download")
        shp = (nvar, P[2], P[1], P[0]) if nvar > 1 else (P[2], P[1], P[0])
        return out.reshape(shp)

    def upload(self, w, level, serial=1):
        w = np.ascontiguousarray(w, dtype=np.float64)
        self._chk(self._fn("upload_state")(self.ctx, level, serial, w.ctypes.data_as(C.POINTER(C.c_double))),
                  "upload_state")

    def close(self):
        if getattr(self, "ctx", None):
            self._fn("destroy")(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def physical(a, spec):
    """View of the physical cells (2..il etc.) of a field in [.., k, j, i] order."""
    nx, ny, nz = spec.n
    return a[..., 2:nz + 2, 2:ny + 2, 2:nx + 2]


def _cycle(self, mlvl=None, ncyc=2):
    """One multigrid cycle at FMG level mlvl (mge_cycle / mgeo_cycle); returns max_res."""
    mlvl = self.case.prm.nlevel if mlvl is None else mlvl
    out = C.c_double()
    self._chk(self._fn("cycle")(self.ctx, mlvl, ncyc, C.byref(out)), "cycle")
    return out.value


Cycle.cycle = _cycle
