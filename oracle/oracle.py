"""ctypes binding of the CPU oracle (test infrastructure only).

Tests, __graft_entry__.smoke() and the CPU legs of bench.py use it as the
checker; the GPU product never imports it.  ``OracleCycle`` is the product's
``Cycle`` driver bound to the oracle's mgeo_ entry points, so one test drives
both with the same call sequence.
"""
import ctypes as C
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from code_mge_gb300 import _abi as A  # noqa: E402
from code_mge_gb300.runtime import Cycle  # noqa: E402

from . import build as _build  # noqa: E402

_LIB = None


def load(build_if_missing=True):
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.OUT
    if build_if_missing:
        _build.build()
    lib = C.CDLL(path)
    A.bind(lib, "mgeo_", A.SIGNATURES)
    A.bind(lib, "mgeo_", [A.ORACLE_INIT])
    lib.mgeo_set_threads.argtypes = [C.c_int]
    lib.mgeo_set_threads.restype = None
    lib.mgeo_get_threads.restype = C.c_int
    lib.mgeo_cycle.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.mgeo_cycle.restype = C.c_int
    _LIB = lib
    return lib


def set_threads(n):
    load().mgeo_set_threads(int(n))


class OracleCycle(Cycle):
    def __init__(self, case, init_flow=True, prm=None):
        super().__init__(case, lib=load(), prefix="mgeo_", init_flow=init_flow, prm=prm)
