"""Failure detection and edge inputs on the GPU, against the oracle.

resvg's own limits are defensive skips: a filter that fails clears its layer
(crates/resvg/src/filter/mod.rs:343-354), a layer that cannot be made skips
its group (crates/resvg/src/render.rs:108-109), non-finite geometry draws
nothing.  The backend adds bounded device waits and reports allocation
failure.  None of these tests faults, traps or hangs the GPU: the stuck wait is
made by withholding one producer arrival (the consumers' bounded wait then runs
out and the kernel drains), the allocation failure by a host-side hook.
"""
import ctypes as C

import numpy as np
import pytest

import resvg_gb300 as R
from resvg_gb300 import _abi as A
from tests.helpers import base_path, diff_stats, plain_group, rect_path, solid

pytestmark = pytest.mark.gpu

IDENT = (1, 0, 0, 1, 0, 0)
RGPU_ERR_OUT_OF_MEMORY = 4
RGPU_ERR_CAPACITY = 5
RGPU_ERR_DEVICE_FAULT = 6


def _lib():
    L = R.lib()
    for n, args in (("rgpu_set_wait_limit", [C.c_uint32]), ("rgpu_test_withhold_window", [C.c_int]),
                    ("rgpu_test_fail_allocations", [C.c_uint32]), ("rgpu_trim", [])):
        getattr(L, n).restype = C.c_int
        getattr(L, n).argtypes = args
    return L


def test_stuck_handoff_returns_device_fault_then_recovers(gpu, oracle_mod):
    import torch
    L = _lib()
    t = R.Tree.generate(0, seed=3, index=0, scale=1.0)
    ref = oracle_mod.render(t.view(), IDENT, 512, 512)
    dev = torch.zeros((512, 512, 4), dtype=torch.uint8, device="cuda")
    try:
        assert L.rgpu_set_wait_limit(1 << 14) == 0
        assert L.rgpu_test_withhold_window(1) == 0
        for _ in range(2):  # twice: each launch starts from cleared error words
            status = L.rgpu_render_device(t.handle, R._rt(IDENT), 512, 512, C.c_void_p(dev.data_ptr()), 512 * 4,
                                          None)
            torch.cuda.synchronize()
            assert status == RGPU_ERR_DEVICE_FAULT, R.lib().rgpu_last_error().decode()
            assert "0x10" in R.lib().rgpu_last_error().decode()
    finally:
        L.rgpu_test_withhold_window(0)
        L.rgpu_set_wait_limit(0)
    # the context is still usable and the next render is exact
    got = R.render(t, IDENT, 512, 512)
    assert diff_stats(got, ref) == (0, 0)


def test_forced_allocation_failure_leaves_pixmap_untouched(gpu, oracle_mod):
    L = _lib()
    t = R.Tree.generate(0, seed=4, index=0, scale=0.5)
    rng = np.random.default_rng(1)
    bg = rng.integers(0, 256, (512, 512, 4), dtype=np.uint8)
    bg[..., :3] = np.minimum(bg[..., :3], bg[..., 3:4])
    assert L.rgpu_trim() == 0  # the next render has to allocate again
    assert L.rgpu_test_fail_allocations(1) == 0
    pm = bg.copy()
    try:
        with pytest.raises(R.RenderError, match="memory"):
            R.render(t, IDENT, pixmap=pm)
    finally:
        L.rgpu_test_fail_allocations(0)
    assert np.array_equal(pm, bg)
    got = R.render(t, IDENT, pixmap=bg.copy())
    ref = oracle_mod.render(t.view(), IDENT, 512, 512, bg.copy())
    assert diff_stats(got, ref) == (0, 0)


@pytest.mark.parametrize("ts", [
    (float("nan"), 0, 0, 1, 0, 0), (1, 0, 0, 1, float("inf"), 0), (float("inf"), 0, 0, float("inf"), 0, 0),
    (1, float("nan"), 0, 1, 0, 0), (0, 0, 0, 0, 0, 0), (1e30, 0, 0, 1e30, 0, 0), (1e-30, 0, 0, 1e-30, 3, 3)])
def test_non_finite_and_degenerate_transforms(gpu, oracle_mod, ts):
    t = R.Tree.generate(1, seed=9, index=0, scale=0.02)
    rng = np.random.default_rng(2)
    bg = rng.integers(0, 256, (96, 128, 4), dtype=np.uint8)
    bg[..., :3] = np.minimum(bg[..., :3], bg[..., 3:4])
    got = R.render(t, ts, pixmap=bg.copy())
    ref = oracle_mod.render(t.view(), ts, 128, 96, bg.copy())
    assert diff_stats(got, ref) == (0, 0), ts


def _degenerate_paths_tree():
    t = R.Tree(100, 100)
    root = t.add_group(-1, plain_group())
    red = solid(t, 250, 10, 10)
    t.add_path(root, base_path(fill_paint=red), [], [])                                  # no verbs
    t.add_path(root, base_path(fill_paint=red), [A.MOVE], [10, 10])                      # a lone move
    t.add_path(root, base_path(fill_paint=red), [A.MOVE, A.CLOSE], [20, 20])             # move + close
    t.add_path(root, base_path(fill_paint=red, stroke_paint=red, stroke_width=2),
               [A.MOVE, A.LINE], [30, 30, 30, 30])                                      # zero-length line
    v, p = rect_path(40, 40, 0, 20)                                                       # zero-width rect
    t.add_path(root, base_path(fill_paint=red), v, p)
    t.add_path(root, base_path(stroke_paint=red, stroke_width=0.0), v, p)                # zero stroke width
    t.add_path(root, base_path(fill_paint=red), [A.MOVE, A.LINE, A.LINE, A.CLOSE],
               [float("nan"), 1, 50, 50, 60, 10])                                        # a NaN point
    v, p = rect_path(55.5, 55.5, 30, 30)                                                  # one ordinary fill
    t.add_path(root, base_path(fill_paint=solid(t, 10, 10, 240), fill_opacity=0.8), v, p)
    t.finalize()
    return t


def test_empty_and_degenerate_paths(gpu, oracle_mod):
    t = _degenerate_paths_tree()
    got = R.render(t, (1.5, 0, 0, 1.5, 0, 0), 150, 150)
    ref = oracle_mod.render(t.view(), (1.5, 0, 0, 1.5, 0, 0), 150, 150)
    assert diff_stats(got, ref) == (0, 0)
    assert got.any()  # the ordinary fill is drawn


@pytest.mark.parametrize("size", [(1, 1), (1, 37), (41, 1), (3, 2)])
def test_tiny_canvases(gpu, oracle_mod, size):
    w, h = size
    t = R.Tree.generate(0, seed=12, index=0, scale=0.2)
    for ts in (IDENT, (w / 512.0, 0, 0, h / 512.0, 0, 0), (1, 0, 0, 1, -200.5, -100.25)):
        got = R.render(t, ts, w, h)
        ref = oracle_mod.render(t.view(), ts, w, h)
        assert diff_stats(got, ref) == (0, 0), (size, ts)


SVG_TWO_FILTERS = """<svg xmlns="http://www.w3.org/2000/svg" width="200" height="200">
  <filter id="big" x="-50%" y="-50%" width="200%" height="200%"><feGaussianBlur stdDeviation="3"/></filter>
  <filter id="lit" x="0" y="0" width="1" height="1">
    <feDiffuseLighting surfaceScale="2"><feDistantLight azimuth="45" elevation="30"/></feDiffuseLighting>
  </filter>
  <filter id="flood" x="0" y="0" width="1" height="1">
    <feFlood flood-color="orange" flood-opacity="0.7"/><feComposite in2="SourceGraphic" operator="atop"/>
  </filter>
  <rect x="40" y="40" width="60" height="60" fill="green" filter="url(#big) url(#SECOND)"/>
  <rect x="120" y="120" width="50" height="50" fill="blue"/>
  <circle cx="150" cy="50" r="30" fill="purple" filter="url(#big)"/>
</svg>"""


@pytest.mark.parametrize("second,fails", [("lit", True), ("flood", False)])
def test_filter_region_smaller_than_its_layer_in_a_tree(gpu, oracle_mod, second, fails):
    """Two filters on one element: the layer is the union of their regions, the
    second filter's region is smaller.  Region-sized results sit at the layer
    origin (flood + composite); lighting of a layer-sized input cannot be
    computed there (the reference indexes out of range), so that filter
    clears its layer, only that one, and the render goes on."""
    from resvg_gb300 import svg
    tree = svg.load_svg(SVG_TWO_FILTERS.replace("SECOND", second))
    got = R.render(tree, (2, 0, 0, 2, 0, 0), 400, 400)
    ref = oracle_mod.render(tree.view(), (2, 0, 0, 2, 0, 0), 400, 400)
    assert diff_stats(got, ref) == (0, 0)
    assert got[300, 300, 3] == 255  # the unfiltered rect is there
    assert got[100, 300].any()      # so is the blurred circle
    warn = R.last_warning()
    assert ("layer cleared" in warn) == fails, warn
    if fails:
        assert not got[140:200, 140:200].any()  # the failed group drew nothing


def test_soft_capacity_overflow_is_reported(gpu):
    """More than 512 flattened lines of one path crossing one pixel row: the
    soft rasteriser keeps what fits, reports RGPU_ERR_CAPACITY, and the next
    batch renders."""
    import torch
    from resvg_gb300 import soft
    n = 600
    a = soft.make_scenes(seed=1, scenes=1, size=64, paths=1, min_segs=n, max_segs=n)
    # a zig-zag: every cubic runs from the top edge to the bottom or back, so
    # each pixel row is crossed by at least one line of each of the 600 cubics
    pts = np.zeros((3 * n, 2), np.float32)
    for k in range(n):
        y0, y1 = (1.0, 63.0) if k % 2 == 0 else (63.0, 1.0)
        x = 1.0 + 62.0 * k / n
        pts[3 * k] = (x, y0)
        pts[3 * k + 1] = (x + 0.2, y0 + (y1 - y0) * 0.33)
        pts[3 * k + 2] = (x + 0.4, y0 + (y1 - y0) * 0.66)
    a["points"] = pts
    sc = soft.Scenes(a)
    with pytest.raises(R.RenderError, match="512"):
        soft.forward(sc)
    b = soft.make_scenes(seed=2, scenes=2, size=64, paths=4)
    image, blurred = soft.forward(soft.Scenes(b))
    torch.cuda.synchronize()
    assert torch.isfinite(blurred).all()
