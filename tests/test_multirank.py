"""CPU tests of the multi-rank path with two `gloo` ranks: the work-item split
covers the triangle exactly once across ranks (checked through the Python
restatement of the pair kernel's scheduler), and the max-over-ranks timing
reduction bench.py uses returns the slowest rank."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, tile, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from seismic_gb300.shard import couple_range, max_over_ranks
    from test_host import _scheduler_pairs_range
    nb = (n + tile - 1) // tile
    total = nb * (nb + 1) // 2 * (tile * tile // 2)
    b, e = couple_range(total, world, rank)
    mine = _scheduler_pairs_range(n, tile, b, e)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    slowest = max_over_ranks(1.5 + rank)
    if rank == 0:
        out_q.put((gathered, slowest))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("n,tile", [(37, 4), (64, 8)])
def test_two_ranks_cover_triangle_once(n, tile):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, tile, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered, slowest = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    allpairs = [pr for part in gathered for pr in part]
    assert len(allpairs) == len(set(allpairs)) == n * (n + 1) // 2
    assert set(gathered[0]).isdisjoint(gathered[1])
    assert slowest == 2.5


def test_couple_range_balanced():
    from seismic_gb300.shard import couple_range
    ranges = [couple_range(103, 4, r) for r in range(4)]
    assert ranges[0][0] == 0 and ranges[-1][1] == 103
    assert all(ranges[k][1] == ranges[k + 1][0] for k in range(3))
    assert max(e - b for b, e in ranges) - min(e - b for b, e in ranges) <= 1
