"""Continuous-batching solve service and batched sweep over the C-ABI.

Requests (geometry, grid size, Mach, angle, residual-drop tolerance) arrive
over time.  Each admitted request becomes one resident case (one mge_ctx: its
whole multigrid hierarchy stays in HBM until it converges).  Admission is
gated by free device memory.  Every in-flight case advances by asynchronous
multigrid cycles: its own (mge_cycle_async / mge_cycle_poll, on its own
stream), or, with ``group=True``, group cycles that advance all the cases at
the same FMG level and precision form together, one launch per phase over all
of them (mge_group_cycle_async / _poll).  A request that arrives while others
run is admitted as soon as memory frees up; its case can be built on host
threads ahead of its admission (``builders``).  A case follows the
reference's full-multigrid schedule (solver.f90:119-259): mcyc cycles per
coarse FMG level, then cycles on the finest level until its residual has
dropped by the requested factor.

The scheduler is independent of the GPU: ``FakeBackend`` drives it in the
CPU tests; ``GpuBackend`` runs it on libmge_gpu.
"""
import ctypes as C
import heapq
import math
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A
from . import cases as K


# --------------------------------------------------------------------- requests
@dataclass
class Request:
    rid: int
    geometry: str          # "sphere", "ellipsoid", "cylinder"
    n: int                 # finest cells per axis (slab: n x n x 2)
    mach: float
    alpha_deg: float = 0.0
    tol: float = 1e-8      # converged when residual <= tol * first residual of the finest level
    precision: int = A.MGE_PREC_MIXED
    arrival: float = 0.0
    semi: tuple = (1.0, 0.7, 0.5)
    max_cycles: int = 2000
    refine_drop: float = 1e-6  # mixed form: switch to FP64 at this residual drop ...
    refine_stall: int = 40     # ... or once the residual has not improved by 5 % for this many cycles
    # retire (not converged) once the residual, in FP64 (the plain form, or the
    # mixed form after its switch), has not improved by 5 % for this many
    # cycles: a case caught in a limit cycle; 0 runs it to max_cycles
    retire_stall: int = 0
    # results
    t_admit: float = None
    t_done: float = None
    cycles: int = 0
    residual: float = None
    drop: float = None
    cd: float = None
    cl: float = None
    converged: bool = False  # retired on the residual drop (not on max_cycles)
    stalled: bool = False    # retired by retire_stall
    refined_at: int = None   # finest cycle of the switch to FP64 (mixed form)
    error: str = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def build_case(r: Request):
    """The synthetic case of a request (3 levels, W-cycle, JST, 5-stage RK)."""
    nlevel = 3 if r.n >= 32 else 2
    if r.geometry == "sphere":
        c = K.sphere_box(n=r.n, nlevel=nlevel, extent=6.0, mach=r.mach, mgtype=2, alpha_deg=r.alpha_deg,
                         precision=r.precision)
    elif r.geometry == "ellipsoid":
        c = K.ellipsoid_box(n=r.n, semi=r.semi, nlevel=nlevel, extent=4.0 * max(r.semi), mach=r.mach,
                            alpha_deg=r.alpha_deg, mgtype=2, precision=r.precision)
    elif r.geometry == "cylinder":
        c = K.cylinder_slab(n=r.n, span=2, nlevel=nlevel, extent=8.0, mach=r.mach, alpha_deg=r.alpha_deg,
                            precision=r.precision)
    else:
        raise ValueError(r.geometry)
    for L in range(nlevel - 1):
        c.prm.mcyc[L] = 10
    c.prm.mcyc[nlevel - 1] = r.max_cycles
    return c


def case_bytes(case):
    """Device bytes a case holds (fields, records, stage scratch)."""
    fine = max(s.dims[0] * s.dims[1] * s.dims[2] for L in case.levels for s in L)
    mixed = case.prm.precision == A.MGE_PREC_MIXED
    tot = 64 * 8 * fine
    for li, L in enumerate(case.levels):
        esz = 4 if (mixed and li + 1 < len(case.levels)) else 8
        for s in L:
            n = s.dims[0] * s.dims[1] * s.dims[2]
            tot += n * (38 * esz + 3 + 4) + s.arrays["nmir"] * 512
    return int(tot * 1.05) + (8 << 20)


# --------------------------------------------------------------------- backends
class GpuBackend:
    """One mge_ctx per case, advanced with asynchronous cycles."""

    def __init__(self, device=0, coop_ctas=32):
        from .runtime import load_library
        self.lib = load_library()
        self.device = device
        self.coop_ctas = coop_ctas

    def free_memory(self):
        f, t = C.c_size_t(), C.c_size_t()
        if self.lib.mge_device_mem(self.device, C.byref(f), C.byref(t)) != 0:
            raise RuntimeError("mge_device_mem failed")
        return f.value

    def open(self, case):
        from .runtime import Cycle
        cyc = Cycle(case, lib=self.lib, device=self.device)
        if self.coop_ctas:
            self.lib.mge_set_coop_ctas(cyc.ctx, self.coop_ctas)
        return cyc

    def launch(self, h, mlvl):
        return self.lib.mge_cycle_async(h.ctx, mlvl)

    def poll(self, h, ncyc):
        out = C.c_double()
        rc = self.lib.mge_cycle_poll(h.ctx, ncyc, C.byref(out))
        return rc, out.value

    def prolong(self, h, mlvl):
        return self.lib.mge_prolong_async(h.ctx, mlvl)

    def launch_group(self, hs, mlvl):
        """One lockstep cycle of several cases (mge_group_cycle_async);
        returns a group token, or None when the cases cannot run together."""
        arr = (C.c_void_p * len(hs))(*[h.ctx.value for h in hs])
        if self.lib.mge_group_cycle_async(arr, len(hs), mlvl) != 0:
            return None
        return {"arr": arr, "n": len(hs), "res": (C.c_double * len(hs))(), "rcs": (C.c_int * len(hs))()}

    def poll_group(self, g):
        """1 while running; else (0, residuals, stop codes)."""
        rc = self.lib.mge_group_cycle_poll(g["arr"], g["n"], -1, g["res"], g["rcs"])
        if rc == 1:
            return 1, None, None
        if rc != 0:
            return rc, [float("nan")] * g["n"], [rc] * g["n"]
        return 0, list(g["res"]), list(g["rcs"])

    def refine(self, h):
        return self.lib.mge_set_precision(h.ctx, A.MGE_PREC_REFINED)

    def finish(self, h):
        f = h.forces()
        return f.cd, f.cl

    def close(self, h):
        h.close()


class FakeBackend:
    """Deterministic stand-in used by the CPU tests: each case's residual falls
    geometrically per cycle; a cycle completes after `latency` polls."""

    def __init__(self, free_bytes=1 << 34, rate=0.7, latency=2, floor32=0.0, floor64=0.0):
        self.free = free_bytes
        self.rate = rate
        self.latency = latency
        self.launched = 0
        self.floor32 = floor32     # mixed form: the residual stalls here until refined
        self.floor64 = floor64     # the residual in FP64 stalls here (a limit cycle)

    def free_memory(self):
        return self.free

    def open(self, case):
        self.free -= case_bytes(case)
        return {"case": case, "res": 1.0, "busy": 0, "bytes": case_bytes(case)}

    def launch(self, h, mlvl):
        h["busy"] = self.latency
        self.launched += 1
        return 0

    def poll(self, h, ncyc):
        h["busy"] -= 1
        if h["busy"] > 0:
            return 1, 0.0
        nxt = h["res"] * self.rate
        if h["case"].prm.precision == A.MGE_PREC_MIXED and not h.get("refined"):
            nxt = max(nxt, self.floor32)
        else:
            nxt = max(nxt, self.floor64)
        h["res"] = nxt
        return 0, h["res"]

    def prolong(self, h, mlvl):
        return 0

    def launch_group(self, hs, mlvl):
        self.groups = getattr(self, "groups", 0) + 1
        for h in hs:
            self.launch(h, mlvl)
        return {"hs": hs, "out": {}}

    def poll_group(self, g):
        for q, h in enumerate(g["hs"]):
            if q not in g["out"]:
                rc, res = self.poll(h, 0)
                if rc != 1:
                    g["out"][q] = (rc, res)
        if len(g["out"]) < len(g["hs"]):
            return 1, None, None
        return 0, [g["out"][q][1] for q in range(len(g["hs"]))], [g["out"][q][0] for q in range(len(g["hs"]))]

    def refine(self, h):
        h["refined"] = True
        return 0

    def finish(self, h):
        return 0.5 + 0.01 * h["case"].prm.rm, 0.0

    def close(self, h):
        self.free += h["bytes"]


# --------------------------------------------------------------------- scheduler
@dataclass
class _Slot:
    req: Request
    case: object
    handle: object
    nlevel: int
    mlvl: int = 1
    ncyc: int = 0
    ini: float = None
    inflight: bool = False
    cycles_fine: int = 0
    refined: bool = False
    best: float = None         # best finest-level residual so far, and the cycle it came at
    best_at: int = 0
    grouped: bool = False      # its cycle in flight is part of a group cycle


class Server:
    """Continuous batching: admit while memory allows, keep every admitted case
    cycling, retire cases as they converge."""

    def __init__(self, backend, reserve_bytes=2 << 30, max_active=64, clock=time.perf_counter, group=False,
                 builders=0, lookahead=4, max_cells=0):
        self.be = backend
        # max_cells > 0: admit while the cases in flight hold at most this many
        # finest-level cells (one case is always admitted), so that under
        # overload the admitted cases fill the GPU and finish, instead of every
        # arrived case sharing it and none finishing
        self.max_cells = max_cells
        # builders > 0: the cases of the next `lookahead` arrived requests are
        # built on host threads while the GPU works, instead of in the
        # scheduler pass that admits them
        self.builder = ThreadPoolExecutor(max_workers=builders) if builders else None
        self.lookahead = lookahead
        self.pending = {}
        self.reserve = reserve_bytes
        self.max_active = max_active
        self.clock = clock
        # group: the cycles of cases at the same FMG level and precision form
        # launch together (one launch per phase over all of them)
        self.group = group
        self.inflight_groups = []  # (token, [slots])
        self.group_cycles = 0
        self.queue = []           # (arrival, rid, request) min-heap
        self.active = []
        self.done = []
        self.peak_active = 0
        self.cases = {}

    def submit(self, r: Request):
        heapq.heappush(self.queue, (r.arrival, r.rid, r))

    def _case_of(self, r):
        """The request's case, once built (None while a host thread builds it)."""
        if r.rid in self.cases:
            return self.cases[r.rid]
        if self.builder is None:
            self.cases[r.rid] = build_case(r)
            return self.cases[r.rid]
        f = self.pending.get(r.rid)
        if f is None:
            f = self.pending[r.rid] = self.builder.submit(build_case, r)
        if not f.done():
            return None
        del self.pending[r.rid]
        self.cases[r.rid] = f.result()
        return self.cases[r.rid]

    def _admit(self, now):
        if self.builder is not None:
            for _, _, r in heapq.nsmallest(self.lookahead, self.queue):
                if r.arrival <= now and r.rid not in self.cases and r.rid not in self.pending:
                    self.pending[r.rid] = self.builder.submit(build_case, r)
        while self.queue and self.queue[0][0] <= now and len(self.active) < self.max_active:
            r = self.queue[0][2]
            case = self._case_of(r)
            if case is None:
                return  # still being built (FIFO: no overtaking)
            need = case_bytes(case)
            if self.active and self.be.free_memory() - need < self.reserve:
                return  # wait for memory to free up (FIFO: no overtaking)
            if (self.active and self.max_cells > 0 and
                    sum(s.case.finest_cells for s in self.active) + case.finest_cells > self.max_cells):
                return  # the GPU is full of work: wait for a case to finish
            heapq.heappop(self.queue)
            try:
                h = self.be.open(case)
            except Exception as e:  # admission failed (out of memory): retry later unless nothing is running
                if not self.active:
                    r.error = str(e)
                    r.t_done = now
                    self.done.append(r)
                    continue
                heapq.heappush(self.queue, (r.arrival, r.rid, r))
                return
            r.t_admit = self.clock()
            self.cases.pop(r.rid, None)
            self.active.append(_Slot(r, case, h, case.prm.nlevel))
            self.peak_active = max(self.peak_active, len(self.active))

    def _prepare(self, s: _Slot):
        """The FMG step to the next finer level when due, and the next cycle's count."""
        prm = s.case.prm
        if s.mlvl < s.nlevel and s.ncyc >= prm.mcyc[s.mlvl - 1]:
            self.be.prolong(s.handle, s.mlvl)        # FMG step to the next finer level
            s.mlvl += 1
            s.ncyc = 0
        s.ncyc += 1

    def _advance(self, s: _Slot):
        """Launch the next cycle of a slot (or finish it); returns False when retired."""
        self._prepare(s)
        rc = self.be.launch(s.handle, s.mlvl)
        if rc != 0:
            self._retire(s, "cycle launch failed (%d)" % rc)
            return False
        s.inflight = True
        return True

    def _retire(self, s: _Slot, err=None):
        r = s.req
        if err is None:
            try:
                r.cd, r.cl = self.be.finish(s.handle)
            except Exception as e:
                err = str(e)
        r.error = err
        r.cycles = s.cycles_fine
        r.t_done = self.clock()
        self.be.close(s.handle)
        self.active.remove(s)
        self.done.append(r)

    def step(self):
        """One scheduler pass; returns True while work remains."""
        now = self.clock()
        self._admit(now)
        progressed = False
        for tok, members in list(self.inflight_groups):
            rc, res, rcs = self.be.poll_group(tok)
            if rc == 1:
                continue
            self.inflight_groups.remove((tok, members))
            progressed = True
            for q, s in enumerate(members):
                s.grouped = False
                self._complete(s, rcs[q], res[q])
        for s in list(self.active):
            if not s.inflight or s.grouped:
                continue
            rc, res = self.be.poll(s.handle, s.ncyc)
            if rc == 1:
                continue
            progressed = True
            self._complete(s, rc, res)
        ready = [s for s in self.active if not s.inflight]
        if ready:
            progressed = True
            self._launch(ready)
        return bool(self.active or self.queue), progressed

    def _launch(self, ready):
        if not self.group:
            for s in ready:
                self._advance(s)
            return
        for s in ready:
            self._prepare(s)
        groups = {}
        for s in ready:
            key = (s.mlvl, s.nlevel, s.req.precision, s.refined)
            groups.setdefault(key, []).append(s)
        for key, members in groups.items():
            tok = self.be.launch_group([s.handle for s in members], key[0]) if len(members) > 1 else None
            if tok is None:  # one case, or cases that cannot run together: their own cycles
                for s in members:
                    rc = self.be.launch(s.handle, s.mlvl)
                    if rc != 0:
                        self._retire(s, "cycle launch failed (%d)" % rc)
                    else:
                        s.inflight = True
                continue
            self.group_cycles += 1
            for s in members:
                s.inflight = True
                s.grouped = True
            self.inflight_groups.append((tok, members))

    def _complete(self, s, rc, res):
        """A slot's cycle has finished: residual bookkeeping, precision
        switch, retirement; the slot is left ready for its next cycle."""
        s.inflight = False
        if rc != 0:
            self._retire(s, "cycle failed (%s)" % A.error_name(rc))
            return
        if s.mlvl == s.nlevel:
            s.cycles_fine += 1
            if s.ncyc == 1:
                s.ini = res
            s.req.residual = res
            s.req.drop = res / s.ini if s.ini else None
            if s.best is None or res < 0.95 * s.best:
                s.best, s.best_at = res, s.cycles_fine
            # FP32 coarse corrections stall near eps32 * |tau|: switch to
            # FP64 at the set drop, or as soon as the residual stops falling
            stalled = s.req.refine_stall > 0 and s.cycles_fine - s.best_at >= s.req.refine_stall
            if (s.req.precision == A.MGE_PREC_MIXED and not s.refined and s.ini
                    and ((s.req.refine_drop > 0.0 and res <= s.req.refine_drop * s.ini) or stalled)):
                if self.be.refine(s.handle) != 0:
                    self._retire(s, "precision refinement failed")
                    return
                s.refined = True
                s.req.refined_at = s.cycles_fine
                s.best, s.best_at = res, s.cycles_fine  # the FP64 stall window starts here
                if s.req.tol >= s.req.refine_drop:
                    return  # the drop counts only once an FP64 cycle confirms it
            conv = bool(s.ini) and res <= s.req.tol * s.ini
            fp64 = s.req.precision == A.MGE_PREC_FP64 or s.refined
            stall_out = s.req.retire_stall > 0 and fp64 and s.cycles_fine - s.best_at >= s.req.retire_stall
            if conv or stall_out or s.cycles_fine >= s.req.max_cycles or res != res:
                s.req.converged = conv
                s.req.stalled = stall_out and not conv
                self._retire(s)

    def run(self, idle_sleep=50e-6, deadline=None):
        while True:
            more, progressed = self.step()
            if not more:
                break
            if deadline is not None and self.clock() > deadline:
                break
            if not progressed:
                time.sleep(idle_sleep)
        return self.done


def poisson_requests(rate, duration, seed=20261204, sizes=(64, 256), mach=(0.1, 0.8), tol=1e-8,
                     precision=A.MGE_PREC_MIXED, max_cycles=2000, retire_stall=0):
    """Poisson arrivals (rate per second) over `duration` seconds; geometry
    uniform over sphere / ellipsoid / cylinder slab, n a multiple of 8 in
    [sizes], Mach uniform in [mach]."""
    rng = np.random.default_rng(seed)
    t, out, rid = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        g = ["sphere", "ellipsoid", "cylinder"][int(rng.integers(0, 3))]
        n = int(8 * rng.integers(sizes[0] // 8, sizes[1] // 8 + 1))
        out.append(Request(rid, g, n, float(rng.uniform(*mach)), float(rng.uniform(-5.0, 10.0)) if g != "sphere" else 0.0,
                           tol=tol, precision=precision, arrival=t,
                           semi=tuple(float(x) for x in rng.uniform(0.5, 2.0, 3)), max_cycles=max_cycles,
                           retire_stall=retire_stall))
        rid += 1
    return out


def batched_sweep_requests(count=64, seed=20261203, sizes=(32, 48, 64, 96, 128), precision=A.MGE_PREC_MIXED,
                           tol=1e-8, max_cycles=2000, retire_stall=0):
    """The batched sweep: `count` ellipsoid cases with seeded sizes, semi-axes,
    Mach and angle of attack, all present at t = 0."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(count):
        n = int(rng.choice(sizes))
        semi = tuple(float(x) for x in rng.uniform(0.5, 2.0, 3))
        out.append(Request(q, "ellipsoid", n, float(rng.uniform(0.2, 0.8)), float(rng.uniform(-5.0, 10.0)),
                           tol=tol, precision=precision, arrival=0.0, semi=semi, max_cycles=max_cycles,
                           retire_stall=retire_stall))
    return out


def summarize(done, t_wall):
    ok = [r for r in done if r.error is None]
    conv = [r for r in ok if r.converged]
    lat = np.array([r.latency for r in ok]) if ok else np.zeros(0)
    return {
        "requests": len(done),
        "completed": len(ok),
        "converged": len(conv),
        "stalled": sum(1 for r in ok if r.stalled),
        "failed": len(done) - len(ok),
        "solves_per_s": len(conv) / t_wall if t_wall > 0 else None,
        "p50_s": float(np.percentile(lat, 50)) if lat.size else None,
        "p99_s": float(np.percentile(lat, 99)) if lat.size else None,
        "wall_s": t_wall,
    }
