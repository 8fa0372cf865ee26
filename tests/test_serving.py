"""Serving scheduler and batched sweep: host logic on CPU with a fake
backend, continuous batching and alone-vs-mix equality on the GPU."""
import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import serving as S


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 0.001
        return self.t


def test_scheduler_completes_all_requests_in_fifo_admission():
    be = S.FakeBackend(rate=0.5, latency=2)
    srv = S.Server(be, reserve_bytes=0, clock=FakeClock())
    reqs = [S.Request(q, ["sphere", "ellipsoid", "cylinder"][q % 3], 16, 0.3 + 0.05 * q, tol=1e-3,
                      arrival=0.0005 * q, max_cycles=100) for q in range(9)]
    for r in reqs:
        srv.submit(r)
    done = srv.run(idle_sleep=0)
    assert len(done) == 9 and all(r.error is None for r in done)
    # each request converged: the fake residual halves per cycle, so a 1e-3 drop
    # from the first finest-level residual takes 10 more cycles (11 in all)
    assert all(r.cycles == 11 for r in done)
    assert srv.peak_active > 1   # requests overlapped
    assert all(r.converged for r in done)
    st = S.summarize(done, 1.0)
    assert st["completed"] == 9 and st["converged"] == 9 and st["p99_s"] >= st["p50_s"]


def test_group_mode_gives_every_request_the_same_cycles():
    """Cases at the same FMG level and precision form advance in group
    cycles; each request's cycle count, refinement point and outcome are
    those of the one-case-at-a-time scheduling."""
    def run(group):
        be = S.FakeBackend(rate=0.6, latency=2, floor32=1e-5)
        srv = S.Server(be, reserve_bytes=0, clock=FakeClock(), group=group)
        reqs = [S.Request(q, ["sphere", "ellipsoid"][q % 2], 16, 0.3 + 0.05 * q, tol=1e-8, arrival=0.0,
                          max_cycles=200, precision=A.MGE_PREC_MIXED if q % 3 else A.MGE_PREC_FP64,
                          refine_drop=1e-6, refine_stall=0) for q in range(8)]
        for r in reqs:
            srv.submit(r)
        done = sorted(srv.run(idle_sleep=0), key=lambda r: r.rid)
        return done, srv, be
    alone, _, _ = run(False)
    grouped, srv, be = run(True)
    assert [(r.cycles, r.converged, r.refined_at) for r in grouped] == \
        [(r.cycles, r.converged, r.refined_at) for r in alone]
    assert srv.group_cycles > 0 and be.groups == srv.group_cycles


def test_admission_is_bounded_by_work_in_flight():
    """max_cells: cases are admitted while those in flight hold at most that
    many finest cells (one is always admitted), FIFO."""
    reqs = [S.Request(q, "sphere", 16, 0.4, tol=1e-2, arrival=0.0, max_cycles=50) for q in range(6)]
    one = S.build_case(reqs[0]).finest_cells
    be = S.FakeBackend(rate=0.5, latency=1)
    srv = S.Server(be, reserve_bytes=0, clock=FakeClock(), max_cells=2 * one + 1)
    for r in reqs:
        srv.submit(r)
    done = srv.run(idle_sleep=0)
    assert len(done) == 6 and all(r.converged for r in done)
    assert srv.peak_active == 2
    assert [r.rid for r in sorted(done, key=lambda r: r.t_admit)] == list(range(6))


def test_admission_is_gated_by_free_memory():
    reqs = [S.Request(q, "sphere", 16, 0.4, tol=1e-2, arrival=0.0, max_cycles=50) for q in range(6)]
    one = S.case_bytes(S.build_case(reqs[0]))
    be = S.FakeBackend(free_bytes=int(2.5 * one), rate=0.5, latency=1)
    srv = S.Server(be, reserve_bytes=0, clock=FakeClock())
    for r in reqs:
        srv.submit(r)
    done = srv.run(idle_sleep=0)
    assert len(done) == 6
    assert srv.peak_active == 2      # only two cases fit at once
    assert be.free == int(2.5 * one)  # every case released its memory


def test_mixed_case_refines_when_its_residual_stalls():
    # the fake's mixed residual stops at 1e-4 until the case switches to FP64
    be = S.FakeBackend(rate=0.5, latency=1, floor32=1e-4)
    srv = S.Server(be, reserve_bytes=0, clock=FakeClock())
    r = S.Request(0, "sphere", 16, 0.5, tol=1e-8, max_cycles=500, refine_drop=1e-9, refine_stall=20)
    srv.submit(r)
    (d,) = srv.run(idle_sleep=0)
    assert d.converged and d.refined_at is not None
    # the coarse FMG cycles already halve the fake residual 10 times: the
    # floor is reached in the 4th finest cycle, the stall is seen 20 later
    assert d.refined_at == 24
    assert d.cycles < 80


def test_case_caught_in_a_limit_cycle_is_retired_when_asked():
    # the fake's FP64 residual stops at 1e-6, above the 1e-8 tolerance
    for precision in (A.MGE_PREC_FP64, A.MGE_PREC_MIXED):
        done = {}
        for retire in (0, 30):
            be = S.FakeBackend(rate=0.5, latency=1, floor32=1e-4, floor64=1e-6)
            srv = S.Server(be, reserve_bytes=0, clock=FakeClock())
            srv.submit(S.Request(0, "sphere", 16, 0.5, tol=1e-8, max_cycles=400, precision=precision,
                                 refine_stall=20, retire_stall=retire))
            (done[retire],) = srv.run(idle_sleep=0)
        assert not done[0].converged and not done[0].stalled and done[0].cycles == 400
        d = done[30]
        assert not d.converged and d.stalled and d.error is None
        # the window opens at the switch to FP64 (mixed) or at the last 5 % gain
        assert d.cycles < 100
        assert d.cycles - (d.refined_at or 0) >= 30


def test_poisson_and_sweep_generators_are_seeded():
    a = S.poisson_requests(4.0, 10.0)
    b = S.poisson_requests(4.0, 10.0)
    assert [(r.geometry, r.n, r.mach) for r in a] == [(r.geometry, r.n, r.mach) for r in b]
    assert all(64 <= r.n <= 256 and r.n % 8 == 0 for r in a)
    sw = S.batched_sweep_requests(64)
    assert len(sw) == 64 and {r.n for r in sw} <= {32, 48, 64, 96, 128}
    assert all(0.2 <= r.mach <= 0.8 and -5.0 <= r.alpha_deg <= 10.0 for r in sw)


@pytest.mark.gpu
@pytest.mark.parametrize("group", [False, True])
def test_results_are_the_same_alone_and_in_the_mix(gpulib, monkeypatch, group):
    """Each result is bit-identical alone and in a mix of four, with the
    mix's cases on their own cycles or in group cycles (the launch forms
    pinned to the per-phase form with global-memory sweeps, the form a group
    cycle runs)."""
    if group:
        monkeypatch.setenv("MGE_AUTOTUNE", "0")
        monkeypatch.setenv("MGE_COOP_MAX_CELLS", "0")
    mk = lambda: [S.Request(0, "sphere", 16, 0.5, tol=1e-4, max_cycles=200),
                  S.Request(1, "ellipsoid", 24, 0.3, alpha_deg=4.0, tol=1e-4, max_cycles=200),
                  S.Request(2, "cylinder", 32, 0.4, tol=1e-4, max_cycles=200),
                  S.Request(3, "sphere", 24, 0.7, tol=1e-4, max_cycles=200)]
    alone = {}
    for r in mk():
        srv = S.Server(S.GpuBackend(), reserve_bytes=1 << 30)
        srv.submit(r)
        (d,) = srv.run()
        assert d.error is None
        alone[d.rid] = d
    srv = S.Server(S.GpuBackend(), reserve_bytes=1 << 30, group=group)
    for r in mk():
        srv.submit(r)
    mix = {d.rid: d for d in srv.run()}
    assert srv.peak_active == 4
    assert (srv.group_cycles > 0) == group
    for rid, a in alone.items():
        m = mix[rid]
        assert m.error is None and m.cycles == a.cycles
        # each case computes on its own resident state: identical in the mix
        assert m.cd == a.cd and m.residual == a.residual
