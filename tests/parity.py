"""Shared helpers of the parity tests: drive the GPU library and the oracle
with the same call sequence and compare fields with a stated tolerance."""
import numpy as np

from code_mge_gb300 import cases as K
from code_mge_gb300.runtime import Cycle, physical
from oracle.oracle import OracleCycle

# Per-stage residual and state tolerance of the plain FP64 path: the
# infinity-norm difference relative to the infinity norm of the oracle field.
RTOL = 1e-12


def rel_err(a, b, region=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.max(np.abs(a - b)) if a.size else 0.0
    s = np.max(np.abs(b)) if b.size else 0.0
    return d / s if s > 0 else d


def exact_fraction(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.mean(a == b)) if a.size else 1.0


PATHS = ("coop", "phases", "tuned")


def set_path(path):
    """Small blocks run euler as one cooperative launch; 'phases' forces one
    launch per phase (the path of large blocks)."""
    import os
    if path == "phases":
        os.environ["MGE_COOP_MAX_CELLS"] = "0"
    elif path == "coop":
        os.environ["MGE_COOP_MAX_CELLS"] = str(10 ** 9)
    else:  # "tuned": the autotuner chooses
        os.environ.pop("MGE_COOP_MAX_CELLS", None)


def pair(case, develop_cycles=0, path="coop"):
    """(gpu, oracle) Cycles on the same case; optionally develop the flow on the
    oracle for a few cycles and load that state into both."""
    set_path(path)
    o = OracleCycle(case)
    g = Cycle(case)
    if develop_cycles:
        # the context copies its parameters when it is made: set the cycle
        # counts on a copy first
        prm = type(case.prm).from_buffer_copy(case.prm)
        prm.mcyc[case.prm.nlevel - 1] = develop_cycles
        for L in range(case.prm.nlevel - 1):
            prm.mcyc[L] = 1
        dev = OracleCycle(case, prm=prm)
        dev.solve()
        for L in range(1, case.prm.nlevel + 1):
            w = dev.field("w", L)
            o.upload(w, L)
            g.upload(w, L)
        dev.close()
    return g, o


def compare(g, o, name, level, rtol=RTOL, phys_only=True):
    a = g.field(name, level)
    b = o.field(name, level)
    if phys_only and name not in ("wsol", "psol", "dtim"):
        sp = g.spec(level)
        a, b = physical(a, sp), physical(b, sp)
    e = rel_err(a, b)
    assert e <= rtol, "%s level %d: rel err %.3e > %.1e (exact %.4f)" % (name, level, e, rtol, exact_fraction(a, b))
    return e, exact_fraction(a, b)


def small_cylinder(**kw):
    a = dict(n=32, span=2, nlevel=2, extent=4.0, mcyc_fine=4, mach=0.3)
    a.update(kw)
    return K.cylinder_slab(**a)


def small_sphere(**kw):
    a = dict(n=16, nlevel=2, extent=2.0, mcyc_fine=4, radius=0.6)
    a.update(kw)
    return K.sphere_box(**a)
