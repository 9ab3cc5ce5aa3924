"""The N > 1 host path on CPU: two gloo ranks.

The reference reduces the per-level CFL bounds over its ranks before the
level-0 projection (include/solvers/BaseSolver.H:120-165); the bench takes the
slowest rank's time; independent units (members, replicas) are split without a
collective.  Each rank here holds different per-level bounds; both must arrive
at the same dt list, the one a single process holding all boxes computes."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from hydroexa_gb300 import ranks
from hydroexa_gb300.solver import BaseSolver

LEVEL_DT = {0: [0.030, 0.011, 0.0041], 1: [0.020, 0.013, 0.0035]}  # per rank: levels 0..2 (after the cfl factor)
RATIO = [(2, 2), (2, 2)]


class _Boxes(BaseSolver):
    """compute_dt_level of this rank's boxes (no device work)."""

    def __init__(self, rank):
        super().__init__()
        self.rank = rank

    def compute_dt_level(self, U, terrain, geom, lev, cfl):
        return LEVEL_DT[self.rank][lev]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert ranks.rank_and_world() == (rank, world)
        dt = []
        _Boxes(rank).compute_dt(dt, None, None, None, RATIO, 2, 0.45)
        mx = ranks.reduce_real_max([10.0 + rank, -float(rank)])
        mine = ranks.shard(11, rank, world)
        got = [None] * world
        dist.all_gather_object(got, (mine.start, mine.stop))
        out.put((rank, dt, mx, got))
    finally:
        dist.destroy_process_group()


def test_two_ranks_agree_on_dt_and_timing():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        r, dt, mx, got = q.get(timeout=120)
        res[r] = (dt, mx, got)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # one process holding all boxes: per-level minimum, then the projection to level 0
    mins = [min(LEVEL_DT[0][k], LEVEL_DT[1][k]) for k in range(3)]
    d0 = min(mins[0], mins[1] * 2.0, mins[2] * 4.0)
    expect = [d0, d0 / 2.0, d0 / 4.0]
    for r in range(world):
        dt, mx, got = res[r]
        assert dt == expect
        assert mx == [11.0, 0.0]
        spans = sorted(got)
        assert spans[0][0] == 0 and spans[-1][1] == 11
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))


def test_single_process_is_the_identity():
    assert ranks.rank_and_world() == (0, 1)
    assert ranks.reduce_real_min([3.0, 1.0]) == [3.0, 1.0]
    dt = []
    _Boxes(0).compute_dt(dt, None, None, None, RATIO, 2, 0.45)
    d0 = min(0.030, 0.011 * 2, 0.0041 * 4)
    assert dt == [d0, d0 / 2, d0 / 4]


@pytest.mark.parametrize("n,world", [(0, 3), (5, 1), (7, 3), (256, 8)])
def test_shard_partitions(n, world):
    seen = []
    for r in range(world):
        seen.extend(ranks.shard(n, r, world))
    assert seen == list(range(n))
    sizes = [len(ranks.shard(n, r, world)) for r in range(world)]
    assert max(sizes) - min(sizes) <= 1
