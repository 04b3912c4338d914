"""The multi-rank path of bench.py on CPU: two `gloo` ranks.

bench.py runs one process per GPU under torchrun.  Each rank renders its
own scenes (the batched form shards scenes, no collective on the data path),
ranks meet at a barrier around the timed region, and every rank takes the
slowest rank's step time.  These tests exercise that logic with gloo ranks
on the host: the process group set-up, the max over ranks, and disjoint scene
shards whose trees differ.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    r, w = bench.dist_setup(world, backend="gloo")
    assert (r, w) == (rank, world)
    dist.barrier()
    # a rank-dependent step time: every rank must report the slowest one
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, w, torch.device("cpu"))
    idx = bench.shard(rank, 3)
    gathered = [None] * world
    dist.all_gather_object(gathered, idx)
    out.put((rank, ms, gathered))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_max_and_shards():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, gathered in res:
        assert ms == 15.0  # the slower rank's time on both ranks
        assert gathered == [[0, 1, 2], [3, 4, 5]]


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1, None) == 12.5
    assert bench.shard(0, 4) == [0, 1, 2, 3]


def test_shards_render_different_scenes():
    """Scene i of rank r is generated from index r * n + i: the ranks' batches
    differ, so the aggregate is over distinct work."""
    sys.path.insert(0, ROOT)
    R = pytest.importorskip("resvg_gb300")
    import bench
    a = [R.Tree.generate(3, seed=bench.SEED, index=i, scale=0.05) for i in bench.shard(0, 2)]
    b = [R.Tree.generate(3, seed=bench.SEED, index=i, scale=0.05) for i in bench.shard(1, 2)]
    sa = [tuple(t.size) + (t.view().contents.path_count,) for t in a]
    sb = [tuple(t.size) + (t.view().contents.path_count,) for t in b]
    assert sa != sb
