"""The multi-rank path of bench.py on CPU: two `gloo` ranks.

bench.py runs one process per GPU under torchrun.  The batched workload is
one batch split over the ranks by estimated cost (greedy LPT on side^2 x
paths, resvg_gb300.batch.lpt_partition), with no collective on the data path;
ranks meet at a barrier around the timed region, and every rank takes the
slowest rank's step time.  These tests exercise that logic with gloo ranks on
the host: the process group set-up, the max over ranks, and a split that
covers every scene exactly once with balanced cost.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N_SCENES = 4096


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
    idx = bench.batch_shard(rank, world, N_SCENES)
    gathered = [None] * world
    dist.all_gather_object(gathered, idx)
    out.put((rank, ms, gathered))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_max_and_cost_split():
    import torch.multiprocessing as mp
    from resvg_gb300 import batch as B
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    costs = B.config3_costs(2026, N_SCENES)
    for rank, ms, gathered in res:
        assert ms == 15.0  # the slower rank's time on both ranks
        # both ranks computed the same split; it covers every scene once
        flat = sorted(i for part in gathered for i in part)
        assert flat == list(range(N_SCENES))
        assert not set(gathered[0]) & set(gathered[1])
        loads = [sum(costs[i] for i in part) for part in gathered]
        # LPT bound against the lower bound max(total / ranks, largest scene)
        assert B.lpt_bound_ok(costs, gathered)
        # and in practice the two halves of this batch are within 1% of each other
        assert max(loads) / min(loads) < 1.01, loads
    assert res[0][2] == res[1][2]


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1, None) == 12.5
    assert bench.batch_shard(0, 1, 4) == [0, 1, 2, 3]


def test_lpt_partition_properties():
    from resvg_gb300 import batch as B
    costs = [100.0, 1.0, 50.0, 49.0, 30.0, 20.0, 10.0, 1.0]
    parts = B.lpt_partition(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    assert B.lpt_bound_ok(costs, parts)
    # one huge scene: it alone sets the bound and sits in a part of its own
    parts = B.lpt_partition([1000.0] + [1.0] * 10, 4)
    assert [0] in parts
    assert B.lpt_partition([], 2) == [[], []]


def test_cost_estimate_matches_generated_scenes():
    """The partition's cost model reads each scene's side and path count from
    the generator's first draws without building the tree."""
    R = pytest.importorskip("resvg_gb300")
    from resvg_gb300 import batch as B
    for i in range(40):
        side, paths = B.config3_shape(2026, i)
        t = R.Tree.generate(3, seed=2026, index=i)
        assert t.size == (side, side)
        # the tree holds one more path (the clip polygon) when the scene has a clip and a blur
        assert t.view().contents.path_count in (paths, paths + 1)
