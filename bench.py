"""Benchmark of the GB300 multigrid Runge-Kutta cycle.

Workload (default): 3-D inviscid flow past a D=1 sphere cut into a 192^3
uniform Cartesian box [-10,10]^3, M=0.5, alpha=0, JST central flux with
scalar dissipation (k2=0.5, k4=1/64), 5-stage Jameson RK (cstp 1/4,1/6,3/8,
1/2,1; cdis 1,0,0.56,0,0.44), CFL 2.8 local time step, implicit residual
smoothing eps=0.6, 4-level W-cycle (192^3/96^3/48^3/24^3).  Synthetic:
the geometry is generated analytically (there is no dataset).

A step is one multigrid W-cycle at the finest FMG level.  The metric counts
cell-updates: one physical cell advanced by one full RK update (all five
stages); per W-cycle that is 192^3 + 3*96^3 + 6*48^3 + 4*24^3 =
10,450,944 cell-updates (residual-only evaluations are not counted).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                    [--precision fp64|mixed]

--gpus N > 1 runs one independent replica per GPU (the path does not shard
across GPUs within one case); value is the whole-job aggregate.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from code_mge_gb300 import _abi as A  # noqa: E402
from code_mge_gb300 import cases as K  # noqa: E402
from code_mge_gb300 import replicas as R  # noqa: E402
from code_mge_gb300 import schedule as S  # noqa: E402

METRIC = "MG-cycle cell-updates/s (mixed vs FP64 plain); solves/s & p50/p99 latency"
UNIT = "cell-updates/s"

# Algorithmic HBM bytes per cell-update of one full euler update (FP64,
# 5-variable fields of 40 B): smoothing stages 11 fields, non-smoothing
# stages 4 fields, 17 B of scalars per stage, 56 B for the time step.
BYTES_PER_CELL_UPDATE_IRS = (11 + 4 + 11 + 4 + 11) * 40 + 5 * 17 + 56   # 1,781
# The roofline kernel is k_face on a stage with dissipation (stage 1), one
# thread per cell of [2..ie]^3.  Compulsory bytes per cell: it reads the
# per-cell fluxes F (15), sensors (3), the differences w(q)-w(q-1) (15) and
# lambda (1), and writes the convective and dissipative face fluxes (15 + 15):
# 64 doubles.
FACE_DOUBLES_DISSIP = 64
# The Roe + viscous face pass (MUSCL states from w and p, viscous stresses
# from the cell-centred u, v, w, T) on such a stage reads w (5), p (1) and
# the 4 viscous variables once per cell and writes the convective, upwind
# and viscous face fluxes (15 + 15 + 15): 55 doubles.
FACE_DOUBLES_ROE_NS = 55
# From one ncu capture of that launch on the 128^3 sphere (2,146,689 cells):
# DRAM read + write 1,115.3 MB = 519.6 B per cell, and 118.2 FP64
# instructions (DADD + DMUL, no DFMA under --fmad=false) per cell.  Traffic
# scales with the cells a launch covers.
FACE_DRAM_BYTES_PER_CELL = 519.6
FACE_FP64_PER_CELL = 118.2
# The three passes of the residual on a stage with dissipation (stage 1),
# plain FP64, from ncu captures of each pass on the 128^3 sphere (one launch
# of stage 1, --set full):
#   cells     which cells one thread each: "prep" [1..ie]^3, "face" [2..ie]^3, "phys" [2..il]^3
#   alg       compulsory HBM bytes per cell
#   dram      measured DRAM read + write bytes per cell
#   fp64      binary64 operations per cell (DADD + DMUL + DFMA), as ncu counted
#             them when every one ran on the FP64 pipe; the kernels now run
#             part of the products on the integer pipes (soft_fp64.cuh), so
#             the rate of these operations can pass the FP64 pipe's peak
# prep reads w, p (6 doubles) and writes H, F, dlt, fp (34); face reads F, fp,
# dlt, lambda (34) and writes efs, dfs (30); combine reads efs, dfs, vdtim
# (31 doubles), blank (1 B), cutmap (4 B) and writes fw, dw (10 doubles).
KERNEL_MODEL = {
    "prep": {"cells": "prep", "alg": 40 * 8, "dram": 320.6, "fp64": 120.1},
    "face": {"cells": "face", "alg": FACE_DOUBLES_DISSIP * 8, "dram": FACE_DRAM_BYTES_PER_CELL,
             "fp64": FACE_FP64_PER_CELL},
    "combine": {"cells": "phys", "alg": 41 * 8 + 5, "dram": 338.6, "fp64": 75.0},
}
# The mixed form's finest-level passes (the contracted FP64 residual), per
# physical cell and averaged over the launches of one update, from the ncu
# capture of every kernel of one 128^3 update (FP64 instruction and DRAM byte
# counters):
# its prep pass (5 launches), dissipation face pass (3) and combine pass (5).
# alg: prep reads w, p and writes H, F (stages 2, 4) or H, F, dlt, fp
# (stages 1, 3, 5): 32.8 doubles on average; the face pass reads dlt, fp,
# lambda and writes dfs: 34 doubles; combine reads F, dfs, fw, vdtim, blank,
# cutmap and writes fw, dw: 41 doubles + 5 B.
MIXED_MODEL = {
    "prep": {"alg": 32.8 * 8, "dram": 1349.9 / 5, "fp64": 325.3 / 5, "launches": 5},
    "face": {"alg": 34 * 8, "dram": 819.6 / 3, "fp64": 244.9 / 3, "launches": 3},
    "combine": {"alg": 41 * 8 + 5, "dram": 1776.2 / 5, "fp64": 329.0 / 5, "launches": 5},
}
FP64_LANES_PER_SM_CYCLE = 2      # GB300: 2 FP64 thread-operations per SM per cycle
# binary64 operations of every kernel of one finest-level update of the 128^3
# sphere (ncu's FP64 instruction count with every product on the FP64 pipe),
# per cell-update, by precision form
FP64_PER_CELL_UPDATE = {"fp64": 1793.9, "mixed": 1003.4}
GB300_SMS = 152
LAUNCHES_PER_UPDATE = {"timestep": 1, "prep": 5, "face": 5, "rec": 5, "combine": 5, "irs_i": 3, "irs_j": 3,
                       "irs_k_update": 3, "cutcell": 5, "bcond": 5, "rtrms": 1}


WORKLOADS = {
    "sphere192": "sphere D=1 in 192^3 box [-10,10]^3, M=0.5, JST scalar, 5-stage RK, CFL 2.8, IRS 0.6, "
                 "4-level W-cycle; step = 1 W-cycle",
    "cylinder512ns": "laminar NS cylinder D=1, Re=40, M=0.2, 512x512x2 finest grid at h=D/96 with 3 coarser "
                     "embedded levels (each doubling h and extent), Roe MUSCL + viscous fluxes, adiabatic no-slip "
                     "cut-cell wall, 5-stage RK, CFL 2.8, IRS 0.6, 4-level V-cycle; step = 1 V-cycle",
}


GEOMETRY = {"sphere192": "sphere", "cylinder512ns": "cylinder"}


def workload_case(precision="fp64", n=192, name="sphere192"):
    prec = A.MGE_PREC_MIXED if precision == "mixed" else A.MGE_PREC_FP64
    if name == "cylinder512ns":
        return K.cylinder_embedded(n=512, span=2, nlevel=4, h_fine=1.0 / 96.0, mach=0.2, mcyc_fine=200,
                                   eqntype=A.MGE_EQN_NS, distype=A.MGE_DIS_ROE2, reynolds=40.0, precision=prec)
    return K.sphere_box(n=n, nlevel=4, extent=10.0, mach=0.5, mgtype=2, mcyc_fine=400, smoo=0.6,
                        precision=prec)


def jst_euler(case):
    return (case.prm.eqntype == A.MGE_EQN_EULER and case.prm.distype == A.MGE_DIS_CENTRAL
            and case.prm.dissip == A.MGE_DISSIP_SCALAR)


def kernel_roofline(case, kind, stage_ms, peak, pkind, fp64_peak):
    """The roofline line of one pass on stage 1 (dissipation on) of the
    finest-level update, from its CUDA-event time and KERNEL_MODEL; the
    passes without a model get the whole update's line only."""
    nx, ny, nz = case.levels[-1][0].n
    cells = {"prep": (nx + 2) * (ny + 2) * (nz + 2), "face": (nx + 1) * (ny + 1) * (nz + 1), "phys": nx * ny * nz}
    if case.prm.precision != A.MGE_PREC_FP64 and jst_euler(case) and kind in MIXED_MODEL:
        # the mixed form: the pass's average launch over one update
        m = MIXED_MODEL[kind]
        runs = [x for x in stage_ms[kind] if x > 0.01]
        t = sum(runs) / len(runs) if runs else 0.0
        n = cells["phys"]
        alg = m["alg"] * n
        ach = alg / (t * 1e-3) / 1e9 if t > 0 else 0.0
        fp = m["fp64"] * n / (t * 1e-3) if t > 0 else 0.0
        name = {"prep": "k_prep (contracted form)", "face": "k_face_diss", "combine": "k_combine (contracted form)"}
        roof = {"bound": "hbm", "kernel": name[kind] + ", average launch of an update", "achieved": ach,
                "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": m["dram"] * n,
                "algorithmic_bytes_per_launch": alg, "launch_ms": t, "peak_kind": pkind,
                "note": "per physical cell; the FP64 issue rate bounds this pass: see fp64_roofline"}
        fp64 = {"kernel": roof["kernel"], "achieved": fp / 1e12, "peak": fp64_peak / 1e12, "unit": "T FP64 op/s",
                "frac": fp / fp64_peak, "fp64_per_cell": m["fp64"],
                "peak_basis": "the FP64 pipe: 2 FP64 thread-ops per SM per cycle x 152 SMs x median SM clock",
                "ops_basis": "binary64 operations per cell as ncu counted them with every product on the FP64 pipe; part of the products now run on the integer pipes, so frac can pass 1"}
        return roof, fp64
    m = KERNEL_MODEL.get(kind)
    if m is None or kind not in stage_ms or not jst_euler(case) or case.prm.precision != A.MGE_PREC_FP64:
        # the Roe + viscous and the mixed passes: their byte models only
        t = stage_ms["face"][0]
        nf = cells["face"]
        dbl = FACE_DOUBLES_DISSIP if jst_euler(case) else FACE_DOUBLES_ROE_NS
        if case.prm.precision != A.MGE_PREC_FP64 and jst_euler(case):
            dbl = 34  # the contracted form's dissipation faces: dlt, fp, lambda in, dfs out
        alg = 8.0 * dbl * nf
        ach = alg / (t * 1e-3) / 1e9 if t > 0 else 0.0
        return ({"bound": "hbm", "kernel": "face pass (stage 1)", "achieved": ach, "peak": peak, "unit": "GB/s",
                 "frac": ach / peak, "traffic": None, "algorithmic_bytes_per_launch": alg, "launch_ms": t,
                 "peak_kind": pkind, "note": "dominant pass: %s; no DRAM capture of this form's pass" % kind}, None)
    t = stage_ms[kind][0]
    n = cells[m["cells"]]
    alg = m["alg"] * n
    ach = alg / (t * 1e-3) / 1e9 if t > 0 else 0.0
    fp = m["fp64"] * n / (t * 1e-3) if t > 0 else 0.0
    roof = {"bound": "hbm", "kernel": "k_%s (stage 1, dissipation on)" % kind, "achieved": ach, "peak": peak,
            "unit": "GB/s", "frac": ach / peak, "traffic": m["dram"] * n, "algorithmic_bytes_per_launch": alg,
            "launch_ms": t, "peak_kind": pkind,
            "note": "the FP64 issue rate, not HBM, bounds this pass: see fp64_roofline; traffic scales the ncu "
                    "capture's DRAM bytes per cell (128^3 sphere) to this launch's cells"}
    fp64 = {"kernel": "k_%s (stage 1)" % kind, "achieved": fp / 1e12, "peak": fp64_peak / 1e12,
            "unit": "T FP64 op/s", "frac": fp / fp64_peak, "fp64_per_cell": m["fp64"],
            "peak_basis": "the FP64 pipe: 2 FP64 thread-ops per SM per cycle x 152 SMs x median SM clock",
            "ops_basis": "binary64 operations per cell as ncu counted them with every product on the FP64 pipe; part of the products now run on the integer pipes, so frac can pass 1"}
    return roof, fp64


def l2_note(lib, cyc, sp):
    field_mb = 5 * 8 * sp.dims[0] * sp.dims[1] * sp.dims[2] / 1e6
    dev_mb = lib.mge_device_bytes(cyc.ctx) / 1e6
    if field_mb > 129.0:
        return "finest 5-variable fields of %.0f MB each exceed the 129 MB L2 (no flush needed)" % field_mb
    return ("finest 5-variable fields of %.0f MB fit in the 129 MB L2, but one step streams the context's "
            "%.0f MB of device fields (a stage's scratch alone is 64 fields of the finest block), so each step's "
            "own traffic turns L2 over; no separate flush" % (field_mb, dev_mb))


def run_profile(args):
    """Short run for the ncu captures: set up the workload, one warm cycle,
    then one timed update of the finest level through the per-kernel path."""
    import torch
    from code_mge_gb300.runtime import Cycle, load_library
    lib = load_library()
    if args.workload in WORKLOADS and not args.workload.startswith("sphere"):
        case = workload_case(args.precision, name=args.workload)
    else:
        case = workload_case(args.precision, n=int(args.workload[len("sphere"):]))
    cyc = Cycle(case)
    cyc.cycle(case.prm.nlevel, ncyc=1)
    ms = np.zeros(len(A.KERNEL_KINDS))
    torch.cuda.nvtx.range_push("profiled")  # one finest-level update, kernel by kernel
    lib.mge_kernel_times(cyc.ctx, case.prm.nlevel, 1, ms.ctypes.data_as(C.POINTER(C.c_double)), len(ms))
    torch.cuda.nvtx.range_pop()
    print(json.dumps({"profile_run": args.workload, "kernel_ms": dict(zip(A.KERNEL_KINDS, ms.tolist()))}))
    cyc.close()
    return 0


def launch_plan(lib, cyc, nlevel):
    """The launch forms the autotuner chose, as MGE_TUNE_PLAN takes them:
    level:CIJK (C cooperative euler, I/J/K line-sweep form per direction)."""
    out = []
    for L in range(1, nlevel + 1):
        coop = C.c_int(0)
        irs = (C.c_int * 3)()
        lib.mge_tuned(cyc.ctx, L, 1, C.byref(coop), irs)
        out.append("%d:%d%d%d%d" % (L, coop.value, irs[0], irs[1], irs[2]))
    return ",".join(out)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return d, "measured"
        except Exception:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def hbm_peak_gbs():
    d, kind = peaks()
    for k in ("hbm_gbs", "hbm_GBs", "hbm_copy_gbs"):
        if k in d:
            v = d[k]
            if isinstance(v, dict):
                v = v.get("burst", v.get("value", next(iter(v.values()))))
            return float(v), kind
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for q, nm in enumerate(names):
                    if r[5 + q].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def time_cpu_oracle(case, threads, cycles=1):
    """Oracle (the reference's algorithm restated in C++) on the same case."""
    from oracle.oracle import OracleCycle, set_threads
    set_threads(threads)
    o = OracleCycle(case)
    t0 = time.perf_counter()
    for q in range(cycles):
        o.cycle(ncyc=q + 1)
    dt = time.perf_counter() - t0
    o.close()
    return dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    wl = args.workload if args.workload in WORKLOADS else "sphere192"
    case = workload_case("fp64", name=wl)
    cu = S.cell_updates_per_cycle(case)
    from oracle.oracle import OracleCycle, set_threads
    set_threads(threads)
    o = OracleCycle(case)
    for q in range(args.warmup):
        o.cycle(ncyc=q + 1)
    t0 = time.perf_counter()
    for q in range(args.steps):
        o.cycle(ncyc=args.warmup + q + 1)
    dt = time.perf_counter() - t0
    v = args.steps * cu / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic %s geometry)" % GEOMETRY[wl],
        "config": {"workload": WORKLOADS[wl], "cells_finest": case.finest_cells,
                   "cell_updates_per_step": cu},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d cycles of the same case, OpenMP over %d host threads" % (args.steps, threads)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (Fortran mgsol/pmgsol) cannot be built or run here; the timed CPU implementation is "
                "the line-by-line C++ restatement of its algorithm",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local
    from code_mge_gb300.runtime import Cycle, load_library
    lib = load_library()
    wl = args.workload if args.workload in WORKLOADS else "sphere192"
    case = workload_case(args.precision, name=wl)
    cu = S.cell_updates_per_cycle(case)
    L = case.prm.nlevel
    cyc = Cycle(case, device=dev)
    plan = launch_plan(lib, cyc, L)
    if args.plan_out and rank == 0:
        with open(args.plan_out, "w") as fh:
            fh.write(plan + "\n")
    for q in range(args.warmup):
        cyc.cycle(L, ncyc=q + 1)

    def barrier():
        torch.cuda.synchronize(dev)
        R.barrier()
        torch.cuda.synchronize(dev)

    sampler = ClockSampler(dev)
    barrier()
    sampler.start()
    dev_ms = 0.0
    n_launch0 = lib.mge_launch_count(cyc.ctx)
    t0 = time.perf_counter()
    res = []
    torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed steps
    for q in range(args.steps):
        res.append(cyc.cycle(L, ncyc=args.warmup + q + 1))
        dev_ms += lib.mge_last_cycle_ms(cyc.ctx)
    torch.cuda.nvtx.range_pop()
    barrier()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    n_launch = lib.mge_launch_count(cyc.ctx) - n_launch0
    # replicas: every rank ran the same cycles; units of all ranks over the
    # slowest rank's device time
    dev_s = R.max_over_ranks(dev_ms / 1e3)
    value = R.whole_job_rate(args.steps * cu, dev_ms / 1e3)

    # end to end through the C-ABI with host buffers: H2D of the finest state
    # from pinned memory, one cycle, D2H of the cycle's residual
    sp = case.levels[L - 1][0]
    w_host = torch.empty(5 * sp.dims[0] * sp.dims[1] * sp.dims[2], dtype=torch.float64, pin_memory=True)
    w_np = w_host.numpy()
    w_np[:] = cyc.field("w", L).ravel()
    wptr = w_np.ctypes.data_as(C.POINTER(C.c_double))
    barrier()
    t0 = time.perf_counter()
    for q in range(args.steps):
        rc = lib.mge_upload_state(cyc.ctx, L, 1, wptr)
        if rc:
            raise RuntimeError("upload failed %d" % rc)
        cyc.cycle(L, ncyc=2)
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e = R.whole_job_rate(args.steps * cu, e2e_s)
    # the drop-in ends a solve with mge_download_state of the state (once per
    # solve, not per cycle): timed on its own
    t0 = time.perf_counter()
    rc = lib.mge_download_state(cyc.ctx, L, 1, wptr, None)
    dl_ms = 1e3 * (time.perf_counter() - t0) if rc == 0 else None

    # per-kernel device times (CUDA events on the library stream), finest
    # level; the prep, face and combine passes also per stage
    nk = len(A.KERNEL_KINDS)
    ms_ = case.prm.mstage
    ms = np.zeros(nk + 3 * ms_)
    lib.mge_kernel_times(cyc.ctx, L, 2, ms.ctypes.data_as(C.POINTER(C.c_double)), len(ms))
    kt = {k: float(ms[q]) for q, k in enumerate(A.KERNEL_KINDS)}
    stage_ms = {"face": [float(x) for x in ms[nk:nk + ms_]], "prep": [float(x) for x in ms[nk + ms_:nk + 2 * ms_]],
                "combine": [float(x) for x in ms[nk + 2 * ms_:nk + 3 * ms_]]}
    share = {k: kt[k] * LAUNCHES_PER_UPDATE[k] for k in kt}
    tot = sum(share.values()) or 1.0
    dom = max(share, key=share.get)
    peak, pkind = hbm_peak_gbs()
    ncell = case.finest_cells
    clk = (clocks.get("sm_mhz") or 2070.0) * 1e6
    fp64_peak = FP64_LANES_PER_SM_CYCLE * GB300_SMS * clk
    roof, fp64_roof = kernel_roofline(case, dom, stage_ms, peak, pkind, fp64_peak)
    upd_ms = sum(kt[k] * LAUNCHES_PER_UPDATE[k] for k in kt)
    whole_update_gbs = BYTES_PER_CELL_UPDATE_IRS * ncell / (upd_ms * 1e-3) / 1e9 if upd_ms > 0 else 0.0
    fp64_upd = FP64_PER_CELL_UPDATE.get(args.precision) if jst_euler(case) else None
    whole_update_fp64 = (fp64_upd * ncell / (upd_ms * 1e-3) / fp64_peak) if (fp64_upd and upd_ms > 0) else None

    # solution output of the finest level (upload_solut.f90:203-237) through
    # the C-ABI: device kernel, device-to-host copy of the 7 variables
    prm = case.prm
    p_tot = prm.p0 * (1.0 + 0.2 * prm.rm ** 2) ** 3.5
    sol = np.zeros(7 * ncell)
    nval = C.c_int(0)
    t0 = time.perf_counter()
    rc = lib.mge_upload_solut(cyc.ctx, L, 1, p_tot, sol.ctypes.data_as(C.POINTER(C.c_double)), sol.size,
                              C.byref(nval))
    solut_ms = 1e3 * (time.perf_counter() - t0) if rc == 0 else None

    l2 = l2_note(lib, cyc, sp)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        dt = time_cpu_oracle(case, threads=1, cycles=1)
        cpu = {"value": cu / dt, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "1 cycle of the same case on 1 host thread (%.1f s)" % dt}
    cyc.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f64-fine/f32-coarse",
            "data": "synthetic (analytic %s geometry, free-stream start)" % GEOMETRY[wl],
            "config": {"workload": WORKLOADS[wl], "cells_finest": ncell,
                       "cell_updates_per_step": cu, "precision": args.precision,
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "launch_plan": plan,
                       "l2": l2},
            "wall_ms_per_step": 1e3 * wall / args.steps,
            "residual_last": res[-1] if res else None,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(w_np.nbytes), "d2h_bytes_per_step": 8,
                    "note": "per step: the finest state uploaded from pinned host memory (mge_upload_state, which "
                            "also runs depvars, bc_cutcell and bcond), one cycle, its residual read back; a solve "
                            "downloads the state once at its end, timed in download_state"},
            "gpu_launches": None,
            "roofline": roof,
            "fp64_roofline": fp64_roof,
            "stage_ms": stage_ms,
            "upload_solut": {"ms": solut_ms, "cells": ncell, "d2h_bytes": int(sol.nbytes), "nval": nval.value},
            "download_state": {"ms": dl_ms, "d2h_bytes": int(w_np.nbytes)},
            "whole_update": {"ms": upd_ms, "hbm_achieved_gbs": whole_update_gbs, "hbm_frac": whole_update_gbs / peak,
                             "bytes_per_cell_update": BYTES_PER_CELL_UPDATE_IRS,
                             "fp64_frac": whole_update_fp64, "fp64_per_cell_update": fp64_upd,
                             "fp64_basis": "binary64 operations of every kernel of one finest-level update (128^3 "
                                           "sphere; ncu's FP64 instruction count with every product on the FP64 "
                                           "pipe), per cell-update, over the summed kernel time, against the FP64 "
                                           "pipe's peak; part of the products run on the integer pipes"},
            "kernel_ms": kt, "kernel_share": {k: share[k] / tot for k in share}, "dominant_kernel": dom,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        line["gpu_launches"] = int(n_launch)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_converge(args):
    """One workload solved in FP64 and in the mixed form to a residual drop:
    cycles, wall time, the final drop, Cl and Cd (pressure on the wall
    records, plus the wall's viscous stress with NS) and their differences,
    and for the cylinder the length of the closed wake on y = 0.  The FP64 solve is the reference the mixed one is
    measured against; the FP64 path itself matches the oracle to 1e-9 in Cd
    on the cases the GPU tests solve."""
    from code_mge_gb300.runtime import Cycle, load_library
    load_library()
    wl = args.workload if args.workload in WORKLOADS else "sphere192"
    out = {}
    for prec in ("fp64", "mixed"):
        case = workload_case(prec, name=wl)
        L = case.prm.nlevel
        case.prm.conv_drop = 1.0 / args.tol
        case.prm.mcyc[L - 1] = args.max_cycles
        cyc = Cycle(case)
        t0 = time.perf_counter()
        hist, n, fo = cyc.solve(max_cycles_total=args.max_cycles,
                                refine_drop=args.refine_drop if prec == "mixed" else 0.0)
        wall = time.perf_counter() - t0
        r = {"cycles": int(n), "wall_s": wall, "drop": float(hist[0] / hist[-1]) if len(hist) else None,
             "converged": bool(len(hist) and hist[0] / hist[-1] > 1.0 / args.tol), "cd": fo.cd, "cl": fo.cl,
             "residual_last": float(hist[-1]) if len(hist) else None,
             "residual_every_50": [float(x) for x in hist[::50]]}
        if GEOMETRY[wl] == "cylinder":
            levels = [(cyc.field("w", lv), cyc.spec(lv)) for lv in range(L, 0, -1)]
            r["recirculation_length"] = K.recirculation_length(levels, radius=0.5)
        cyc.close()
        out[prec] = r
    f, m = out["fp64"], out["mixed"]
    line = {"pattern": "converge", "metric": "time to a %.0e residual drop, FP64 plain vs mixed" % args.tol,
            "unit": "s", "value": m["wall_s"], "fp64_s": f["wall_s"],
            "speedup": f["wall_s"] / m["wall_s"] if m["wall_s"] > 0 else None,
            "abs_dcd": abs(m["cd"] - f["cd"]), "abs_dcl": abs(m["cl"] - f["cl"]),
            "fp64": f, "mixed": m,
            "config": {"workload": WORKLOADS[wl], "tol_drop": args.tol, "max_cycles_finest": args.max_cycles,
                       "refine_drop": args.refine_drop,
                       "forces": "pressure on the wall records, plus the no-slip wall stress with NS; "
                                 "Cd over q_inf x reference area"}}
    if "recirculation_length" in f:
        a, b = f["recirculation_length"], m["recirculation_length"]
        line["abs_d_recirculation_length"] = abs(a - b) if a is not None and b is not None else None
    print(json.dumps(line), flush=True)
    return 0


def run_pattern(args):
    """The batched sweep and the serving loop (one JSON line each)."""
    from code_mge_gb300 import serving as SV
    from code_mge_gb300.runtime import load_library
    load_library()
    if args.pattern == "batched":
        sizes = tuple(int(x) for x in args.sizes.split(","))
        reqs = SV.batched_sweep_requests(args.cases, sizes=sizes, precision=A.MGE_PREC_MIXED, tol=args.tol,
                                         max_cycles=args.max_cycles, retire_stall=args.retire_stall)
        srv = SV.Server(SV.GpuBackend(coop_ctas=args.coop_ctas), max_active=args.cases, group=not args.no_group)
        t0 = time.perf_counter()
        for r in reqs:
            r.arrival = t0
            srv.submit(r)
        done = srv.run()
        tb = time.perf_counter() - t0
        batched = SV.summarize(done, tb)
        # the FP64 plain path on the same cases, one at a time
        plain, t0 = [], time.perf_counter()
        for r in SV.batched_sweep_requests(args.cases, sizes=sizes, precision=A.MGE_PREC_FP64, tol=args.tol,
                                           max_cycles=args.max_cycles, retire_stall=args.retire_stall):
            if args.no_serial:
                break
            r.arrival = t0
            one = SV.Server(SV.GpuBackend(coop_ctas=0), max_active=1)
            one.submit(r)
            plain += one.run()
        tp = time.perf_counter() - t0
        if args.no_serial:  # the mixed sweep alone
            line = {"pattern": "batched sweep", "metric": "converged solves/s", "unit": "solves/s",
                    "value": batched["solves_per_s"], "baseline_fp64_serial": None, "cases": args.cases,
                    "batched": batched, "group_cycles": srv.group_cycles, "peak_active": srv.peak_active,
                    "per_case": [{"rid": r.rid, "n": r.n, "cycles": r.cycles, "converged": r.converged,
                                  "cd": r.cd} for r in sorted(done, key=lambda r: r.rid)]}
            print(json.dumps(line), flush=True)
            return 0
        serial = SV.summarize(plain, tp)
        mix = {r.rid: r for r in done}
        both = [r for r in plain if r.error is None and mix[r.rid].error is None
                and r.converged and mix[r.rid].converged]
        dcd = [abs(mix[r.rid].cd - r.cd) for r in both]
        per_case = [{"rid": r.rid, "n": r.n, "mach": round(r.mach, 4), "alpha_deg": round(r.alpha_deg, 3),
                     "semi": [round(x, 3) for x in r.semi],
                     "fp64": {"cycles": r.cycles, "converged": r.converged, "stalled": r.stalled, "cd": r.cd,
                              "error": r.error},
                     "mixed": {"cycles": mix[r.rid].cycles, "fp64_from_cycle": mix[r.rid].refined_at,
                               "converged": mix[r.rid].converged, "stalled": mix[r.rid].stalled,
                               "cd": mix[r.rid].cd, "error": mix[r.rid].error},
                     "abs_dcd": (abs(mix[r.rid].cd - r.cd) if r.cd is not None and mix[r.rid].cd is not None
                                 else None)} for r in plain]
        line = {"pattern": "batched sweep", "metric": "converged solves/s", "unit": "solves/s",
                "value": batched["solves_per_s"], "baseline_fp64_serial": serial["solves_per_s"],
                "speedup": batched["solves_per_s"] / serial["solves_per_s"] if serial["solves_per_s"] else None,
                "max_abs_dcd_vs_fp64": max(dcd) if dcd else None, "dcd_cases": len(dcd), "cases": args.cases,
                "per_case": per_case,
                "config": {"sizes": sizes, "tol_drop": args.tol, "levels": 3, "cycle": "W",
                           "precision": "FP32 coarse / FP64 fine", "seed": 20261203,
                           "max_cycles": args.max_cycles, "retire_stall": args.retire_stall},
                "batched": batched, "fp64_serial": serial, "peak_active": srv.peak_active,
                "group_cycles": srv.group_cycles,
                "launch_form": "group cycles (one launch per phase over the cases at the same FMG level and "
                               "precision form)" if not args.no_group else "one graph per case on its own stream"}
        print(json.dumps(line), flush=True)
        return 0
    # serving loop: the mixed form with continuous batching, then the serial
    # FP64 plain path (one case at a time, FIFO) on the same seeded stream
    # over the same window (arrivals plus a bounded drain)
    lo, hi = [int(x) for x in args.sizes.split(",")][:2] if "," in args.sizes else (64, 256)

    def cells(r):
        return r.n * r.n * 2 if r.geometry == "cylinder" else r.n ** 3

    def serve(precision, max_active):
        reqs = SV.poisson_requests(args.rate, args.duration, sizes=(lo, hi), tol=args.tol,
                                   max_cycles=args.max_cycles, precision=precision, retire_stall=args.retire_stall)
        srv = SV.Server(SV.GpuBackend(coop_ctas=args.coop_ctas if max_active > 1 else 0), max_active=max_active,
                        group=max_active > 1 and not args.no_group, builders=2,
                        max_cells=args.max_cells if max_active > 1 else 0)
        t_start = time.perf_counter()
        for r in reqs:
            r.arrival += t_start
            srv.submit(r)
        done = srv.run(deadline=t_start + args.duration + args.drain)
        wall = time.perf_counter() - t_start
        # the cases still running at the deadline are not completions
        for sl in list(srv.active):
            srv.be.close(sl.handle)
        st = SV.summarize(done, wall)
        ok = [r for r in done if r.error is None]
        st.update({"errors": [[r.rid, r.error] for r in done if r.error is not None][:8],
                   "submitted": len(reqs), "finished": len(done), "unfinished": len(reqs) - len(done),
                   "in_flight_at_deadline": len(srv.active), "never_admitted": len(srv.queue),
                   "peak_active": srv.peak_active,
                   "finest_cell_cycles_per_s": sum(r.cycles * cells(r) for r in ok) / wall if wall > 0 else None,
                   "mean_finest_cells": float(np.mean([cells(r) for r in reqs])) if reqs else None})
        return st

    mixed = serve(A.MGE_PREC_MIXED, 64)
    serial = serve(A.MGE_PREC_FP64, 1)
    offered = args.rate
    line = {"pattern": "serving", "metric": "solves/s & p50/p99 time-to-converged", "unit": "solves/s",
            "value": mixed["solves_per_s"], "p50_s": mixed["p50_s"], "p99_s": mixed["p99_s"],
            "submitted": mixed["submitted"], "completed": mixed["converged"], "unfinished": mixed["unfinished"],
            "peak_active": mixed["peak_active"], "offered_req_per_s": offered,
            # requests finished (converged, retired as stalled or at max_cycles) per second
            "service_req_per_s": mixed["finished"] / mixed["wall_s"] if mixed["wall_s"] else None,
            "overload": (offered * mixed["wall_s"] / mixed["finished"]) if mixed["finished"] else None,
            "mixed_continuous_batching": mixed, "fp64_serial": serial,
            "speedup_solves_per_s": (mixed["solves_per_s"] / serial["solves_per_s"]) if serial["solves_per_s"]
            else None,
            "config": {"arrivals": "Poisson %.1f req/s for %.0f s (seed 20261204)" % (args.rate, args.duration),
                       "drain_s": args.drain, "sizes": [lo, hi], "tol_drop": args.tol,
                       "max_cycles": args.max_cycles, "retire_stall": args.retire_stall,
                       "admission": "FIFO, by free memory and at most %d finest cells in flight" % args.max_cells,
                       "precision": "FP32 coarse / FP64 fine (contracted residual), refined to FP64 coarse",
                       "baseline": "FP64 plain, one case at a time in arrival order, same stream and window"}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--pattern", default=None, choices=["batched", "serving", "converge"])
    ap.add_argument("--refine-drop", type=float, default=1e-5,
                    help="mixed form: switch to FP64 once the residual has dropped by this factor")
    ap.add_argument("--cases", type=int, default=64)
    ap.add_argument("--sizes", default="32,48,64,96,128")
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--max-cycles", type=int, default=2000)
    ap.add_argument("--retire-stall", type=int, default=0,
                    help="batched sweep: retire a case whose FP64 residual has not improved by 5%% for this many "
                         "cycles (both forms; 0 runs it to --max-cycles)")
    ap.add_argument("--rate", type=float, default=4.0)
    ap.add_argument("--duration", type=float, default=300.0)
    ap.add_argument("--drain", type=float, default=120.0)
    ap.add_argument("--coop-ctas", type=int, default=32)
    ap.add_argument("--no-serial", action="store_true", help="batched: skip the FP64 one-at-a-time baseline")
    ap.add_argument("--max-cells", type=int, default=8000000,
                    help="serving: admit while the cases in flight hold at most this many finest cells")
    ap.add_argument("--no-group", action="store_true",
                    help="batched/serving: each case its own cycles (no group launches)")
    ap.add_argument("--workload", default="sphere192", choices=["sphere192", "cylinder512ns", "sphere128", "sphere96"])
    ap.add_argument("--profile", action="store_true", help="short run for ncu captures")
    ap.add_argument("--plan-out", default=None, help="write the tuned launch plan (MGE_TUNE_PLAN form) here")
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.pattern == "converge":
        return run_converge(args)
    if args.pattern:
        return run_pattern(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
