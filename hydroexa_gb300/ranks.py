"""Cross-rank reductions of the level loop, one process per GPU.

The reference reduces each level's CFL bound over its MPI ranks with
``ParallelDescriptor::ReduceRealMin`` (include/solvers/BaseSolver.H:133)
before projecting the bounds to level 0; each rank holds some of the level's
boxes.  Here the ranks are ``torch.distributed`` processes (NCCL between GPUs,
gloo on CPU).  Without an initialised process group every reduction is the
identity, as ReduceRealMin is on one process.  Independent units of work
(ensemble members, replicas) are split by ``shard`` and need no collective.
"""
from __future__ import annotations

import torch


def _group():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist
    return None


def rank_and_world() -> tuple[int, int]:
    d = _group()
    if d is None:
        return 0, 1
    return d.get_rank(), d.get_world_size()


def _reduce(values, op_name: str) -> list[float]:
    vals = [float(v) for v in values]
    d = _group()
    if d is None or d.get_world_size() == 1 or not vals:
        return vals
    dev = torch.device("cuda", torch.cuda.current_device()) if d.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor(vals, dtype=torch.float64, device=dev)
    d.all_reduce(t, op=getattr(d.ReduceOp, op_name))
    return [float(x) for x in t.cpu()]


def reduce_real_min(values) -> list[float]:
    """Element-wise minimum over the ranks (ParallelDescriptor::ReduceRealMin)."""
    return _reduce(values, "MIN")


def reduce_real_max(values) -> list[float]:
    """Element-wise maximum over the ranks (the bench's slowest-rank time)."""
    return _reduce(values, "MAX")


def shard(n: int, rank: int, world: int) -> range:
    """Contiguous block of the n units rank owns: the blocks of the world's
    ranks are disjoint, cover 0..n-1 and differ in length by at most one."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("bad shard arguments")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return range(lo, lo + q + (1 if rank < r else 0))


__all__ = ["rank_and_world", "reduce_real_min", "reduce_real_max", "shard"]
