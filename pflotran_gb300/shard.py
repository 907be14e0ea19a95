"""Multi-GPU sharding of the reaction step.

Cells are independent within a reaction step (RTReact's loop,
src/pflotran/reactive_transport.F90:1697-1724, reads no neighbour), so N
GPUs take contiguous cell ranges and exchange nothing on the data path.  The
only collective is the reduction of the per-rank Newton statistics, the
counterpart of RTReact's OS_STATISTICS MPI_Allreduce
(reactive_transport.F90:1767-1775): sum of cells and iterations, max
iterations, sum of non-converged cells.
"""
from __future__ import annotations


def shard_bounds(ncells: int, rank: int, world: int):
    """[lo, hi) of the contiguous range of cells rank `rank` owns."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(ncells, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def reduce_stats(ncells: int, sum_iterations: int, max_iterations: int, nonconverged: int, group=None):
    """All-reduce of the per-rank statistics (torch.distributed, any backend)."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    s = torch.tensor([ncells, sum_iterations, nonconverged], dtype=torch.int64, device=dev)
    m = torch.tensor([max_iterations], dtype=torch.int64, device=dev)
    dist.all_reduce(s, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(m, op=dist.ReduceOp.MAX, group=group)
    return int(s[0]), int(s[1]), int(m[0]), int(s[2])
