"""Replica bookkeeping for runs on several GPUs of one node.

One multigrid case does not shard in this library: every block of a level is
updated by the GPU that holds the case, and the block-to-block exchange the
reference's MPI driver performs (srcmp/solver_mp.f90, bc_overlap between
ranks) is not part of the cycle built here.  With N GPUs each rank therefore
runs its own replica (its own case, or its own share of a request stream) and
no collective touches the data path.  The only cross-rank steps are host-side:
a barrier around the timed region, the maximum of the ranks' elapsed times,
and sums of counters.

The helpers take the process group's backend into account: NCCL reduces CUDA
tensors, gloo CPU tensors, so the same code runs under torchrun on GPUs and in
the CPU tests.
"""
import torch


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def _device():
    dist = _dist()
    if dist is not None and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def world():
    dist = _dist()
    return (dist.get_rank(), dist.get_world_size()) if dist is not None else (0, 1)


def max_over_ranks(x):
    """Maximum of a float over all ranks (the value itself without a group)."""
    dist = _dist()
    if dist is None:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x):
    """Sum of a number over all ranks."""
    dist = _dist()
    if dist is None:
        return x
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier():
    dist = _dist()
    if dist is not None:
        dist.barrier()


def whole_job_rate(units_per_rank, seconds):
    """Units all ranks processed per second of the slowest rank.

    Every rank passes its own unit count and elapsed time; all ranks get the
    same answer."""
    total = sum_over_ranks(units_per_rank)
    slowest = max_over_ranks(seconds)
    return total / slowest if slowest > 0 else 0.0


def shard(items, rank=None, nranks=None):
    """Round-robin share of a list for one rank: item q goes to rank q % N.

    Round-robin rather than contiguous ranges, so that a size-sorted or
    time-ordered stream spreads its large cases and its arrivals evenly."""
    if rank is None or nranks is None:
        rank, nranks = world()
    return [it for q, it in enumerate(items) if q % nranks == rank]
