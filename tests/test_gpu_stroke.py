"""Device-side stroking (kernels/stroke.cu) against the host stroker.

Both run the same stroker source (host/stroke_core.h, tiny-skia-path's
Path::stroke), so the device outlines must equal the host's bit for bit; the
host stroker is in turn pinned by resvg's stroke golden images.  Renders with
device-built outlines are also compared with renders whose outlines the host
built, and with the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A_MOVE, A_LINE, A_QUAD, A_CUBIC, A_CLOSE = 0, 1, 2, 3, 4


@pytest.fixture(scope="module")
def R():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import resvg_gb300 as R
    R.init(0)
    yield R
    R.set_stroke_mode(True)


def _same(a, b):
    (va, pa), (vb, pb) = a, b
    return np.array_equal(va, vb) and pa.shape == pb.shape and np.array_equal(pa.view(np.uint32), pb.view(np.uint32))


def _random_paths(rng, n):
    out = []
    for i in range(n):
        verbs, pts = [A_MOVE], [rng.uniform(-60, 60, 2)]
        for _ in range(int(rng.integers(1, 6))):
            k = int(rng.choice([A_LINE, A_QUAD, A_CUBIC]))
            npt = {A_LINE: 1, A_QUAD: 2, A_CUBIC: 3}[k]
            scale = 1e-3 if i % 9 == 0 else 40.0  # tiny curves next to a wide stroke
            for _ in range(npt):
                pts.append(pts[-1] + rng.uniform(-scale, scale, 2))
            if i % 11 == 0 and k == A_CUBIC:
                pts[-2] = pts[-3].copy()  # a degenerate control point
            verbs.append(k)
        if i % 3 == 0:
            verbs.append(A_CLOSE)
        width = float(rng.choice([0.5, 2.0, 9.0, 30.0, 120.0]))
        out.append((verbs, np.array(pts, np.float32), width, float(rng.choice([1.0, 4.0, 10.0])),
                    int(rng.integers(0, 3)), int(rng.integers(0, 4)), float(rng.choice([0.5, 1.0, 3.7, 40.0]))))
    return out


def test_device_outlines_equal_host_random(R):
    rng = np.random.default_rng(2026)
    paths = _random_paths(rng, 3000)
    dev = R.stroke_paths(paths, on_device=True)
    host = R.stroke_paths(paths, on_device=False)
    diff = [i for i in range(len(paths)) if not _same(dev[i], host[i])]
    assert not diff, f"{len(diff)} of {len(paths)} outlines differ, first {diff[:5]}"
    assert sum(len(h[0]) for h in host) > 30 * len(paths)


def test_device_outlines_equal_host_benchmark_strokes(R):
    """Every stroked path of config 1 and of 64 config-3 scenes, at their own
    widths and at the resolution scales of a 1x and a 4x render."""
    paths = []
    for cfg, idx in [(1, 0)] + [(3, i) for i in range(64)]:
        t = R.Tree.generate(cfg, seed=2026, index=idx)
        v = t.view().contents
        for i in range(v.path_count):
            p = v.paths[i]
            if p.stroke_paint < 0:
                continue
            verbs = np.array([v.verbs[p.verb_offset + k] for k in range(p.verb_count)], np.uint8)
            pts = np.array([v.points[2 * p.point_offset + k] for k in range(2 * p.point_count)], np.float32)
            for rs in (1.0, 4.0):
                paths.append((verbs, pts.reshape(-1, 2), p.stroke_width, p.miter_limit, p.line_cap, p.line_join, rs))
    assert len(paths) > 1000
    dev = R.stroke_paths(paths, on_device=True)
    host = R.stroke_paths(paths, on_device=False)
    diff = [i for i in range(len(paths)) if not _same(dev[i], host[i])]
    assert not diff, f"{len(diff)} of {len(paths)} outlines differ"


def test_outline_larger_than_first_slice(R):
    """A cubic at a large resolution scale needs more than the first slice
    (32 verbs per source verb + 64): the sizing run grows it and strokes again."""
    pts = np.array([[50.71, 79.10], [-58.31, -40.98], [-5.88, 19.01], [-8.41, 14.65]], np.float32)
    paths = [([A_MOVE, A_CUBIC], pts, 78.25, 4.0, 1, 2, 1000.0)] * 3 + [([A_MOVE, A_LINE], pts[:2], 3.0, 4.0, 0, 0, 1.0)]
    dev = R.stroke_paths(paths, on_device=True)
    host = R.stroke_paths(paths, on_device=False)
    assert len(host[0][0]) > 2 * 32 + 64
    assert all(_same(d, h) for d, h in zip(dev, host))


def test_empty_and_degenerate_strokes(R):
    paths = [([A_MOVE], np.array([[1, 1]], np.float32), 2.0, 4.0, 0, 0, 1.0),
             ([A_MOVE, A_LINE], np.array([[1, 1], [1, 1]], np.float32), 2.0, 4.0, 0, 0, 1.0),
             ([A_MOVE, A_LINE], np.array([[1, 1], [1, 1]], np.float32), 2.0, 4.0, 1, 0, 1.0),
             ([A_MOVE, A_LINE, A_CLOSE], np.array([[0, 0], [5, 0]], np.float32), 2.0, 4.0, 2, 1, 1.0),
             ([A_MOVE, A_LINE], np.array([[0, 0], [5, 0]], np.float32), 0.0, 4.0, 0, 0, 1.0),
             ([A_MOVE, A_LINE], np.array([[0, 0], [np.inf, 0]], np.float32), 2.0, 4.0, 0, 0, 1.0)]
    dev = R.stroke_paths(paths, on_device=True)
    host = R.stroke_paths(paths, on_device=False)
    assert all(_same(d, h) for d, h in zip(dev, host))
    assert len(dev[0][0]) == 0 and len(dev[4][0]) == 0


@pytest.mark.parametrize("cfg,scale", [(1, 0.25), (3, 1.0)])
def test_render_device_and_host_stroking_identical(R, cfg, scale):
    import torch
    import oracle
    for idx in range(3 if cfg == 3 else 1):
        outs = []
        # a tree keeps the outlines it was given (from either stroker) for
        # later renders: each mode renders a fresh copy, and the device-stroked
        # tree is rendered twice (device outlines, then its cached copy)
        for on_dev in (True, False):
            R.set_stroke_mode(on_dev)
            t = R.Tree.generate(cfg, seed=2026, index=idx, scale=scale)
            w, h = (int(v) for v in t.size)
            for _ in range(2 if on_dev else 1):
                surf = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
                R.render_device(t, (1, 0, 0, 1, 0, 0), w, h, surf.data_ptr(), w * 4)
                torch.cuda.synchronize()
                outs.append(surf.cpu().numpy())
        R.set_stroke_mode(True)
        assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
        ref = oracle.render(t.view(), (1, 0, 0, 1, 0, 0), w, h).reshape(h, w, 4)
        assert np.array_equal(outs[0], ref)


def test_prepared_scene_replays_device_outlines(R):
    """A prepared scene strokes on its first (sizing) render and replays the
    outlines it keeps on the device; every replay equals the oracle."""
    import torch
    import oracle
    R.set_stroke_mode(True)
    trees = [R.Tree.generate(3, seed=2026, index=i) for i in range(6)]
    sizes = [tuple(int(v) for v in t.size) for t in trees]
    surfs = [torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda") for w, h in sizes]
    sc = R.Scene(trees, [(1, 0, 0, 1, 0, 0)] * len(trees), [w for w, _ in sizes], [h for _, h in sizes],
                 [s.data_ptr() for s in surfs])
    for _ in range(3):
        for s in surfs:
            s.zero_()
        torch.cuda.synchronize()
        sc.render()
        sc.check()
        torch.cuda.synchronize()
        for t, (w, h), s in zip(trees, sizes, surfs):
            ref = oracle.render(t.view(), (1, 0, 0, 1, 0, 0), w, h).reshape(h, w, 4)
            assert np.array_equal(s.cpu().numpy(), ref)


def _random_dashed(rng, n):
    out = []
    for i, (v, p, w, m, cap, join, rs) in enumerate(_random_paths(rng, n)):
        k = int(rng.choice([2, 2, 4, 6, 3]))          # an odd count is invalid: stroked undashed
        dash = rng.uniform(0.0, 15.0, k).astype(np.float32)
        if i % 13 == 0:
            dash[:] = 0.0                               # all zero: invalid
        if i % 17 == 0:
            dash[0] = -1.0                              # negative: invalid
        if i % 5 == 0:
            dash[0] = 0.0                               # zero-length dashes
        phase = float(rng.uniform(-40, 40))
        out.append((v, p, w, m, cap, join, rs, dash, phase))
    return out


def test_device_dashing_equals_host_random(R):
    rng = np.random.default_rng(7)
    paths = _random_dashed(rng, 3000)
    dev = R.stroke_paths(paths, on_device=True)
    host = R.stroke_paths(paths, on_device=False)
    diff = [i for i in range(len(paths)) if not _same(dev[i], host[i])]
    assert not diff, f"{len(diff)} of {len(paths)} dashed outlines differ, first {diff[:5]}"
    assert sum(len(h[0]) > 0 for h in host) > 2000


def test_dashing_that_outgrows_its_slices_and_gives_up(R):
    line = ([A_MOVE, A_LINE], np.array([[0, 0], [3000, 0]], np.float32))
    curve = ([A_MOVE, A_CUBIC], np.array([[0, 0], [900, 400], [-500, 800], [1200, 1200]], np.float32))
    paths = [line + (2.0, 4.0, 1, 2, 1.0, [0.75, 0.75], 0.3),      # 2000 dashes: several times the first slice
             curve + (3.0, 4.0, 0, 0, 2.0, [1.0, 2.0, 0.5, 1.5], -7.0),
             line + (1.0, 4.0, 0, 0, 1.0, [0.001, 0.001], 0.0)]    # 1.5 M dashes: dashing gives up
    dev = R.stroke_paths(paths, on_device=True)
    host = R.stroke_paths(paths, on_device=False)
    assert all(_same(d, h) for d, h in zip(dev, host))
    assert len(host[0][0]) > 4000 and len(host[2][0]) == 0
