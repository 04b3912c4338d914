"""The code paths bench.py times, checked against the oracle at full size.

bench.py measures:
  * a prepared scene (rgpu_scene_prepare / rgpu_scene_render) replayed from a
    captured CUDA graph, for the full 512^2, 1024^2 and 2048^2 workloads;
  * one prepared submission of many batched-workload scenes, graph-replayed,
    under the tuning the autotuner picked;
  * rgpu_render_batch (the end-to-end line) and the plain per-scene call
    rgpu_render_device (the comparison arm).
Each of these is compared here with the oracle on the same trees, including
the full 1024^2 scene (2000 gradient fills, 500 strokes, 20 nested clips, 10
luminance masks) and the largest scenes of the 4096-scene batch.

Tolerance: 0, bit-exact, with the differing-pixel count in the message.
These workloads run tiny-skia's lowp pipeline (solid colours, linear and
simple radial gradients, source-over, the integer clip and mask passes), the
integer box blur, and the IIR blur with the reference's f64 operations in the
reference's order.  The 2048^2 filter chain converts to linearRGB and back and
runs the colour matrix and arithmetic composite in f32; the floating-point
tolerance of the filter path is 1/255 there, and this test asserts the
tighter bound the device reaches.
"""
import os

import numpy as np
import pytest

import resvg_gb300 as R
from resvg_gb300.batch import TUNING_CANDIDATES
from tests.helpers import diff_stats

pytestmark = pytest.mark.gpu

SEED = 2026  # the benchmark's seed
IDENT = (1, 0, 0, 1, 0, 0)
THREADS = max(1, len(os.sched_getaffinity(0)))
# The four costliest scenes (side^2 x paths) of the 4096-scene batch, then a
# run of ordinary ones (indices 0..27 hold small, medium and large canvases and
# three scenes with a clip and a blur).
BATCH_LARGEST = [3587, 97, 1847, 3656]
BATCH_INDICES = BATCH_LARGEST + list(range(28))


def _torch():
    import torch
    return torch


def _oracle_many(oracle_mod, trees):
    sizes = [tuple(int(v) for v in t.size) for t in trees]
    return oracle_mod.render_many([t.view() for t in trees], [IDENT] * len(trees), sizes, THREADS)


@pytest.fixture(scope="module")
def batch_case(gpu, oracle_mod):
    trees = [R.Tree.generate(3, seed=SEED, index=i) for i in BATCH_INDICES]
    # heaviest first so the slowest oracle renders start first
    order = sorted(range(len(trees)), key=lambda k: -trees[k].size[0] * trees[k].size[1] *
                   trees[k].view().contents.path_count)
    refs = [None] * len(trees)
    outs = _oracle_many(oracle_mod, [trees[k] for k in order])
    for k, o in zip(order, outs):
        refs[k] = o
    return trees, refs


class _DeviceBatch:
    """One device buffer holding every scene's pixmap, as bench.py lays it out."""

    def __init__(self, trees):
        torch = _torch()
        self.sizes = [tuple(int(v) for v in t.size) for t in trees]
        self.offs, total = [], 0
        for w, h in self.sizes:
            self.offs.append(total)
            total += ((w * h * 4 + 255) // 256) * 256
        self.buf = torch.zeros(total, dtype=torch.uint8, device="cuda")
        self.ptrs = [self.buf.data_ptr() + o for o in self.offs]
        self.ws = [w for w, _ in self.sizes]
        self.hs = [h for _, h in self.sizes]

    def image(self, i):
        w, h = self.sizes[i]
        o = self.offs[i]
        return self.buf[o:o + w * h * 4].cpu().numpy().reshape(h, w, 4)


def _compare_all(db, refs, what):
    bad = []
    for i, ref in enumerate(refs):
        n, mx = diff_stats(db.image(i), ref)
        if n:
            bad.append((BATCH_INDICES[i], db.sizes[i], n, mx))
    assert not bad, "%s: scenes differing from the oracle (index, size, px, max): %s" % (what, bad)


@pytest.mark.parametrize("config,max_delta", [(0, 0), (1, 0), (2, 1)])
def test_prepared_scene_graph_replay_full_size(gpu, oracle_mod, config, max_delta):
    torch = _torch()
    tree = R.Tree.generate(config, seed=SEED, index=0, scale=1.0)
    w, h = (int(v) for v in tree.size)
    ref = oracle_mod.render(tree.view(), IDENT, w, h)
    surface = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    scene = R.Scene([tree], [IDENT], [w], [h], [surface.data_ptr()])
    # render 1 sizes the buffers un-captured, render 2 captures the graph,
    # render 3 replays it: each from a cleared surface
    for k in range(3):
        surface.zero_()
        torch.cuda.synchronize()
        scene.render(stream.cuda_stream)
        scene.check()
        n, mx = diff_stats(surface.cpu().numpy(), ref)
        assert mx <= max_delta and (max_delta or n == 0), \
            "config %d render %d: %d px differ from the oracle (max %d)" % (config, k + 1, n, mx)


def test_batch_prepared_graph_replay(batch_case):
    torch = _torch()
    trees, refs = batch_case
    db = _DeviceBatch(trees)
    scene = R.Scene(trees, [IDENT] * len(trees), db.ws, db.hs, db.ptrs)
    stream = torch.cuda.Stream()
    for k in range(3):
        db.buf.zero_()
        torch.cuda.synchronize()
        scene.render(stream.cuda_stream)
        scene.check()
        _compare_all(db, refs, "prepared batch, render %d" % (k + 1))


def test_render_batch_one_submission(batch_case):
    torch = _torch()
    trees, refs = batch_case
    db = _DeviceBatch(trees)
    stream = torch.cuda.Stream()
    R.render_batch(trees, [IDENT] * len(trees), db.ws, db.hs, db.ptrs, stream.cuda_stream)
    torch.cuda.synchronize()
    _compare_all(db, refs, "rgpu_render_batch")


@pytest.mark.parametrize("chunks", [2, 5, 32])
def test_render_batch_pipelined_chunks(batch_case, chunks):
    """rgpu_render_batch with the host/device pipeline forced to `chunks`
    chunks (two slots alternating, the host flattening a chunk while the
    device renders the previous one): every scene equals the oracle."""
    torch = _torch()
    trees, refs = batch_case
    db = _DeviceBatch(trees)
    stream = torch.cuda.Stream()
    R.set_batch_chunks(chunks)
    try:
        R.render_batch(trees, [IDENT] * len(trees), db.ws, db.hs, db.ptrs, stream.cuda_stream)
        torch.cuda.synchronize()
    finally:
        R.set_batch_chunks(0)
    _compare_all(db, refs, "rgpu_render_batch in %d chunks" % chunks)


def test_plain_per_scene_device_calls(batch_case):
    torch = _torch()
    trees, refs = batch_case
    db = _DeviceBatch(trees)
    stream = torch.cuda.Stream()
    for i, t in enumerate(trees):
        R.render_device(t, IDENT, db.ws[i], db.hs[i], db.ptrs[i], db.ws[i] * 4, stream.cuda_stream)
    torch.cuda.synchronize()
    _compare_all(db, refs, "rgpu_render_device per scene")


@pytest.fixture(scope="module")
def tuning_case(gpu, oracle_mod):
    """A mixed set for the tuning sweep: the full 512^2 scene, a 1024^2 scene
    with clips and masks at a tenth of the paths, and batched-workload scenes
    of several sizes including two with a clip and a blur."""
    trees = [R.Tree.generate(0, seed=SEED, index=0, scale=1.0), R.Tree.generate(1, seed=SEED, index=0, scale=0.1)]
    trees += [R.Tree.generate(3, seed=SEED, index=i) for i in (1, 2, 4, 6, 9, 11, 17, 22)]
    refs = _oracle_many(oracle_mod, trees)
    return trees, refs


@pytest.mark.parametrize("tuning", TUNING_CANDIDATES, ids=["b%d_px%d" % t for t in TUNING_CANDIDATES])
def test_every_tuning_candidate(tuning_case, tuning):
    torch = _torch()
    trees, refs = tuning_case
    saved = R.get_tuning()
    R.set_tuning(*tuning)
    try:
        db = _DeviceBatch(trees)
        scene = R.Scene(trees, [IDENT] * len(trees), db.ws, db.hs, db.ptrs)
        stream = torch.cuda.Stream()
        for k in range(3):  # un-captured, captured, replayed
            db.buf.zero_()
            torch.cuda.synchronize()
            scene.render(stream.cuda_stream)
            scene.check()
        bad = []
        for i, ref in enumerate(refs):
            n, mx = diff_stats(db.image(i), ref)
            if n:
                bad.append((i, db.sizes[i], n, mx))
        assert not bad, "tuning %s: scenes differing (slot, size, px, max): %s" % (tuning, bad)
    finally:
        R.set_tuning(*saved)


def test_autotuned_tuning_renders_exactly(tuning_case):
    torch = _torch()
    trees, refs = tuning_case
    saved = R.get_tuning()
    try:
        db = _DeviceBatch(trees)
        best, ms = R.autotune(trees, [IDENT] * len(trees), db.ws, db.hs, db.ptrs, TUNING_CANDIDATES, reps=1)
        assert tuple(best) in [tuple(t) for t in TUNING_CANDIDATES] and ms > 0
        assert R.get_tuning() == tuple(best)
        db.buf.zero_()
        torch.cuda.synchronize()
        R.render_batch(trees, [IDENT] * len(trees), db.ws, db.hs, db.ptrs)
        torch.cuda.synchronize()
        for i, ref in enumerate(refs):
            assert diff_stats(db.image(i), ref) == (0, 0), "autotuned %s: slot %d differs" % (best, i)
    finally:
        R.set_tuning(*saved)


def test_tuning_table_autotuner_renders_exactly(tuning_case):
    """The bench's autotuner: a global (band rows, pixels per thread) choice,
    then band rows refined per (width, draws) bucket; the batch it tunes
    renders bit-exactly under the resulting table."""
    import torch
    from resvg_gb300 import batch as BT
    trees, refs = tuning_case
    saved = R.get_tuning()
    try:
        db = _DeviceBatch(trees)
        table, px, timings = BT.autotune_table(trees, db.ws, db.hs, db.ptrs, reps=1)
        assert table and px in {p for _, p in TUNING_CANDIDATES}
        assert R.get_tuning_table() == [tuple(e) for e in table]
        assert all(b in (0,) + BT.BAND_CANDIDATES for _, _, b in table)
        assert timings["global"] and R.get_tuning() == (0, px)
        scene = R.Scene(trees, [IDENT] * len(trees), db.ws, db.hs, db.ptrs)
        for _ in range(3):
            db.buf.zero_()
            torch.cuda.synchronize()
            scene.render()
            scene.check()
        for i, ref in enumerate(refs):
            assert diff_stats(db.image(i), ref) == (0, 0), "table %s px %d: slot %d differs" % (table, px, i)
    finally:
        R.set_tuning_table([])
        R.set_tuning(*saved)
