"""Host-side helpers of the batched form: tuning candidates, the cost model
and the split of one batch over several GPUs.

resvg renders one tree per call (crates/resvg/src/lib.rs:34-43); a batch of
independent trees therefore shards by scene with no exchange between GPUs.
`lpt_partition` splits one batch over ranks by estimated cost (greedy
longest-processing-time first), so every rank gets about the same raster work
and the job's time is not set by one rank holding the largest scenes.
"""
from __future__ import annotations

import heapq

import numpy as np

# (band rows, pixels per thread) the autotuner searches; band rows 0 = chosen
# per stream from its width.
TUNING_CANDIDATES = [(0, 8), (0, 16), (1, 4), (2, 4), (4, 4), (2, 8), (4, 8), (8, 8), (4, 16), (8, 16)]

# Buckets of the tuning table: stream width (canvas side) and draws (fills and
# strokes), upper bounds; the band heights tried per bucket.
WIDTH_BUCKETS = (128, 256, 512, 1024, 32767)
DRAW_BUCKETS = (64, 256, 1024, 1 << 30)
BAND_CANDIDATES = (1, 2, 4, 8)


def scene_draws(tree) -> int:
    """Draws the flattener makes for a tree: one per fill and one per stroke."""
    v = tree.view().contents
    n = 0
    for i in range(v.path_count):
        p = v.paths[i]
        n += (p.fill_paint >= 0) + (p.stroke_paint >= 0)
    return n


def bucket_of(width: float, draws: int):
    wb = next((b for b in WIDTH_BUCKETS if width <= b), WIDTH_BUCKETS[-1])
    db = next(b for b in DRAW_BUCKETS if draws <= b)
    return wb, db


def _time_scene(R, torch, trees, widths, heights, ptrs, stream, reps):
    sc = R.Scene(trees, [(1, 0, 0, 1, 0, 0)] * len(trees), widths, heights, ptrs)
    for _ in range(2):  # sizing, then graph capture
        sc.render(stream.cuda_stream)
    sc.check()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        sc.render(stream.cuda_stream)
    e1.record(stream)
    sc.check()
    return e0.elapsed_time(e1) / reps


def autotune_table(trees, widths, heights, device_ptrs, reps: int = 2, min_share: float = 0.05,
                   min_gain: float = 0.01):
    """The batched form's autotuner; every timing renders the whole sample as
    one prepared batch, so each choice is judged where it runs.

    1. (band rows, pixels per thread) over TUNING_CANDIDATES, one value for
       every stream: the best pair is the starting point.
    2. Scenes are grouped by (canvas-width bucket, draw-count bucket); for
       every bucket holding at least `min_share` of the sample's estimated
       cost (side^2 x draws), heaviest first, the other band heights are tried
       for that bucket alone and kept when the batch gets faster by more than
       `min_gain`.
    Installs the table and the pixels per thread, and returns (table, pixels
    per thread, {"global": {candidate: ms}, bucket: {band rows: ms}})."""
    import torch
    import resvg_gb300 as R
    stream = torch.cuda.Stream()
    saved = R.get_tuning()
    args = (trees, widths, heights, device_ptrs, stream, reps)
    timings = {"global": {}}
    try:
        R.set_tuning_table([])
        for b, px in TUNING_CANDIDATES:
            R.set_tuning(b, px)
            timings["global"][(b, px)] = _time_scene(R, torch, *args)
        (b0, px0), best = min(timings["global"].items(), key=lambda kv: kv[1])
        cost = {}
        for i, t in enumerate(trees):
            d = scene_draws(t)
            key = bucket_of(widths[i], d)
            cost[key] = cost.get(key, 0.0) + scene_cost(widths[i], heights[i], d)
        total = sum(cost.values()) or 1.0
        # a table entry for every bucket, starting from the global band height
        # (band rows 0 keeps the per-stream rule of that candidate)
        table = {(wb, db): b0 for wb in WIDTH_BUCKETS for db in DRAW_BUCKETS}

        def install():
            R.set_tuning_table([(wb, db, table[(wb, db)]) for wb in WIDTH_BUCKETS for db in DRAW_BUCKETS])
        R.set_tuning(0, px0)
        install()
        for key in sorted(cost, key=cost.get, reverse=True):
            if cost[key] / total < min_share:
                break
            res = {table[key]: best}
            for b in BAND_CANDIDATES:
                if b == table[key]:
                    continue
                keep = table[key]
                table[key] = b
                install()
                res[b] = _time_scene(R, torch, *args)
                if res[b] < best * (1.0 - min_gain):
                    best = res[b]
                else:
                    table[key] = keep
            install()
            timings[key] = res
        entries = [(wb, db, table[(wb, db)]) for wb in WIDTH_BUCKETS for db in DRAW_BUCKETS]
    except Exception:
        R.set_tuning(*saved)
        raise
    return entries, px0, timings


def scene_cost(width: float, height: float, paths: int) -> float:
    """Estimated raster cost of a scene: output pixels times path count (each
    path's coverage and shading touch on the order of a fixed fraction of the
    canvas for the synthetic workloads)."""
    return float(width) * float(height) * max(1, int(paths))


def lpt_partition(costs, parts: int):
    """Greedy LPT: scenes in decreasing cost, each to the currently lightest
    part.  Returns `parts` lists of scene indices (each in increasing index
    order).  The heaviest part is at most 4/3 of the optimum, and at most
    total/parts + max(costs) in any case."""
    parts = max(1, int(parts))
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, p) for p in range(parts)]
    out = [[] for _ in range(parts)]
    for i in order:
        load, p = heapq.heappop(heap)
        out[p].append(i)
        heapq.heappush(heap, (load + float(costs[i]), p))
    return [sorted(o) for o in out]


_M64 = (1 << 64) - 1


def _splitmix_next(state):
    state = (state + 0x9E3779B97F4A7C15) & _M64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return state, z ^ (z >> 31)


def config3_shape(seed: int, index: int):
    """(side, path count) of scene `index` of the seeded batched workload,
    from the generator's first two draws (resvg_gb300/csrc/host/gen.cpp,
    gen_config3) without building the tree.  An estimate for partitioning:
    float rounding of log/exp may differ from the C library's in the last
    place."""
    f32 = np.float32
    s = ((seed * 1000003 + index * 7919 + 3) & _M64)
    s = (s * 0x9E3779B97F4A7C15 + 0x632BE59BD9B4E019) & _M64

    def uf(a, b):
        nonlocal s
        s, z = _splitmix_next(s)
        u = f32(z >> 40) * f32(1.0 / 16777216.0)
        return f32(f32(a) + f32(f32(f32(b) - f32(a)) * u))

    side = float(np.round(np.exp(uf(np.log(f32(64)), np.log(f32(1024))))))
    paths = int(round(float(np.exp(uf(np.log(f32(10)), np.log(f32(2000)))))))
    return side, paths


def config3_costs(seed: int, count: int):
    """Estimated cost of every scene of a `count`-scene batched workload."""
    out = []
    for i in range(count):
        side, paths = config3_shape(seed, i)
        out.append(scene_cost(side, side, paths))
    return out


def lpt_bound_ok(costs, parts_lists) -> bool:
    """True when the heaviest part respects the LPT guarantee against the
    lower bound max(total / parts, largest cost)."""
    loads = [sum(float(costs[i]) for i in p) for p in parts_lists]
    m = len(parts_lists)
    lower = max(sum(float(c) for c in costs) / m, max((float(c) for c in costs), default=0.0))
    return max(loads, default=0.0) <= (4.0 / 3.0) * lower * (1 + 1e-9)
