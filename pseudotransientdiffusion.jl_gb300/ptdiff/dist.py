"""Multi-process helpers (one process per GPU, launched by torchrun).

The PT solve of one grid does not shard without the reference's halo
exchange (ImplicitGlobalGrid + MPI, which this build drops), so multi-GPU runs
are replicas of the whole workload, and the batched solver shards its
independent instances across ranks with no data-path collective.  The only
collectives are the max/sum reductions of timings and byte counts.
"""
from __future__ import annotations


def shard_instances(n: int, rank: int, world: int):
    """Indices of the instances rank `rank` owns: a contiguous block, sizes
    differing by at most one, covering 0..n-1 exactly once over all ranks."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return list(range(start, stop))


def shard_by_cells(sizes, world: int):
    """Greedy balance of instances with `sizes` cells over `world` ranks
    (largest first to the least-loaded rank).  Returns a list per rank."""
    order = sorted(range(len(sizes)), key=lambda i: -sizes[i])
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: load[k])
        out[r].append(i)
        load[r] += sizes[i]
    return [sorted(v) for v in out]


def _reduce(v: float, op: str, pg=None) -> float:
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return float(v)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM, group=pg)
    return float(t.item())


def reduce_max(v: float, pg=None) -> float:
    return _reduce(v, "max", pg)


def reduce_sum(v: float, pg=None) -> float:
    return _reduce(v, "sum", pg)
