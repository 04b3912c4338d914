"""GPU render vs the CPU oracle on the same trees (parity gate).

Every case here runs tiny-skia's lowp pipeline (solid colours, linear and
simple radial gradients, group opacity, the separable blend modes, integer
clip and mask passes) or resvg's integer / f64 filter code, so the tolerance
is 0: bit-exact, with the differing-pixel count in the failure message.
"""
import numpy as np
import pytest

import resvg_gb300 as R
from resvg_gb300 import _abi as A
from tests.helpers import base_path, diff_stats, plain_group, rect_path, solid

pytestmark = pytest.mark.gpu


def _both(tree, w, h, ts=(1, 0, 0, 1, 0, 0), bg=None):
    import oracle
    base = np.zeros((h, w, 4), np.uint8) if bg is None else bg.copy()
    g = R.render(tree, ts, pixmap=base.copy())
    o = oracle.render(tree.view(), ts, w, h, base.copy())
    return g, o


@pytest.mark.parametrize("scale", [0.05, 0.25, 1.0])
def test_config0_exact(gpu, oracle_mod, scale):
    t = R.Tree.generate(0, seed=7, index=0, scale=scale)
    g, o = _both(t, 512, 512)
    n, mx = diff_stats(g, o)
    assert n == 0, "config0 scale %s: %d px differ (max %d)" % (scale, n, mx)


@pytest.mark.parametrize("index", range(6))
def test_config0_seeds_exact(gpu, oracle_mod, index):
    t = R.Tree.generate(0, seed=100 + index, index=index, scale=0.3)
    g, o = _both(t, 512, 512)
    assert diff_stats(g, o) == (0, 0)


def test_config1_small(gpu, oracle_mod):
    t = R.Tree.generate(1, seed=3, index=0, scale=0.04)
    g, o = _both(t, 1024, 1024)
    n, mx = diff_stats(g, o)
    assert n == 0, "config1: %d px differ, max %d" % (n, mx)


def test_transform_and_clipping(gpu, oracle_mod):
    # paths that leave the canvas exercise the edge clipper
    t = R.Tree.generate(0, seed=11, index=0, scale=0.2)
    ts = (1.7, 0.3, -0.2, 1.4, -120.0, -60.0)
    g, o = _both(t, 400, 300, ts)
    assert diff_stats(g, o) == (0, 0)


def test_draws_onto_existing_content(gpu, oracle_mod):
    t = R.Tree.generate(0, seed=5, index=0, scale=0.1)
    rng = np.random.default_rng(0)
    bg = rng.integers(0, 256, (512, 512, 4), dtype=np.uint8)
    bg[..., :3] = np.minimum(bg[..., :3], bg[..., 3:4])  # premultiplied
    g, o = _both(t, 512, 512, bg=bg)
    assert diff_stats(g, o) == (0, 0)


def _scene_shapes():
    t = R.Tree(200, 200)
    root = t.add_group(-1, plain_group())
    v, p = rect_path(20.3, 30.7, 100.2, 50.1)
    t.add_path(root, base_path(fill_paint=solid(t, 200, 10, 10), fill_opacity=0.6), v, p)
    # aliased (crispEdges) fill
    v, p = rect_path(60.5, 60.5, 80, 80)
    t.add_path(root, base_path(fill_paint=solid(t, 10, 200, 10), anti_alias=0), v, p)
    # group with opacity and a blend mode
    g = t.add_group(root, plain_group(opacity=0.5, blend=A.BLEND["multiply"]))
    v, p = rect_path(0, 0, 150, 120)
    t.add_path(g, base_path(fill_paint=solid(t, 10, 10, 250)), v, p)
    # even-odd star
    star = [100, 20, 150, 180, 20, 80, 180, 80, 50, 180]
    t.add_path(root, base_path(fill_paint=solid(t, 0, 128, 0), fill_rule=A.EVENODD),
               [A.MOVE, A.LINE, A.LINE, A.LINE, A.LINE, A.CLOSE], star)
    # stroke
    t.add_path(root, base_path(stroke_paint=solid(t, 0, 0, 0), stroke_width=3.0, line_join=A.JOIN_ROUND),
               [A.MOVE, A.CUBIC], [10, 190, 60, 100, 140, 250, 190, 150])
    t.finalize()
    return t


def test_shapes_exact(gpu, oracle_mod):
    t = _scene_shapes()
    g, o = _both(t, 300, 300, (1.5, 0, 0, 1.5, 0, 0))
    n, mx = diff_stats(g, o)
    assert n == 0, "%d px differ (max %d)" % (n, mx)


def test_clip_and_mask(gpu, oracle_mod):
    t = R.Tree(200, 200)
    root = t.add_group(-1, plain_group())
    # clip path: a circle-ish quad loop
    croot = t.add_group(-1, plain_group())
    t.add_path(croot, base_path(fill_paint=solid(t, 0, 0, 0)),
               [A.MOVE, A.QUAD, A.QUAD, A.QUAD, A.QUAD, A.CLOSE],
               [100, 20, 180, 20, 180, 100, 180, 180, 100, 180, 20, 180, 20, 100, 20, 20, 100, 20])
    c = A.Clip()
    c.transform = A.Transform.identity()
    c.clip_path = -1
    c.root = croot
    ci = t.add_clip(c)
    g = t.add_group(root, plain_group(clip_path=ci))
    v, p = rect_path(0, 0, 200, 200)
    t.add_path(g, base_path(fill_paint=solid(t, 250, 100, 0)), v, p)
    # luminance mask
    mroot = t.add_group(-1, plain_group())
    v, p = rect_path(50, 0, 100, 200)
    t.add_path(mroot, base_path(fill_paint=solid(t, 255, 255, 255), fill_opacity=0.7), v, p)
    m = A.Mask()
    m.x, m.y, m.w, m.h = 10, 10, 180, 180
    m.kind = A.MASK_LUMINANCE
    m.mask = -1
    m.root = mroot
    mi = t.add_mask(m)
    g2 = t.add_group(root, plain_group(mask=mi))
    v, p = rect_path(30, 30, 140, 60)
    t.add_path(g2, base_path(fill_paint=solid(t, 0, 0, 250)), v, p)
    t.finalize()
    g, o = _both(t, 300, 300, (1.5, 0, 0, 1.5, 0, 0))
    n, mx = diff_stats(g, o)
    assert n == 0, "%d px differ (max %d)" % (n, mx)


@pytest.mark.parametrize("index", [0, 1, 2, 3, 5, 8, 13, 21])
def test_config3_scenes(gpu, oracle_mod, index):
    """Scenes of the batched workload (sizes 64..1024, 10..2000 paths, 10% with
    clip + blur) rendered one at a time through resvg_render, the largest
    included."""
    t = R.Tree.generate(3, seed=2026, index=index)
    w, h = (int(v) for v in t.size)
    g, o = _both(t, w, h)
    n, mx = diff_stats(g, o)
    assert n == 0, "%d px differ (max %d)" % (n, mx)
