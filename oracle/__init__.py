"""CPU oracle — TEST INFRASTRUCTURE ONLY.

A C++ restatement of resvg 0.48.1's render path (crates/resvg/src/{render,path,
clip,mask,geom}.rs, crates/resvg/src/filter/*.rs) over a restatement of the
tiny-skia 0.12.0 raster pipeline (not vendored in the reference; Skia's
published algorithms).  Parity with resvg is pinned against resvg's own golden
PNGs (crates/resvg/tests/tests/**; tests/golden/pin_oracle.py and
tests/test_oracle_golden.py).  soft.cpp is the FP64 reference of the
differentiable soft-coverage renderer (forward + forward-mode gradients).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
this module.  The product (resvg_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build() -> str:
    subprocess.run([os.path.join(HERE, "build.sh")], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.oracle_render.restype = C.c_int
        L.oracle_render.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.c_void_p]
        L.oracle_render_parallel.restype = C.c_int
        L.oracle_render_parallel.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.c_void_p,
                                             C.c_uint32]
        for n in ("oracle_box_blur", "oracle_iir_blur"):
            getattr(L, n).argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_double]
        L.oracle_morphology.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_float]
        L.oracle_to_linear.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32]
        L.oracle_to_srgb.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32]
        L.oracle_filter_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                          C.POINTER(C.c_float), C.c_void_p, C.c_uint32, C.c_uint32]
        _lib = L
    return _lib


def render(tree_view_ptr, transform, width: int, height: int, pixmap: np.ndarray | None = None) -> np.ndarray:
    """Renders a tree (pointer to an rgpu_tree_view) onto `pixmap` (premultiplied
    RGBA8, (h, w, 4)); a fresh transparent pixmap when None.  Returns it."""
    if pixmap is None:
        pixmap = np.zeros((height, width, 4), dtype=np.uint8)
    assert pixmap.dtype == np.uint8 and pixmap.shape == (height, width, 4) and pixmap.flags.c_contiguous
    ts = (C.c_float * 6)(*[float(v) for v in transform])
    r = lib().oracle_render(C.cast(tree_view_ptr, C.c_void_p), ts, width, height, pixmap.ctypes.data)
    if r != 0:
        raise RuntimeError("oracle_render failed")
    return pixmap


def render_node(tree_view_ptr, node_id: str, transform, width: int, height: int,
                pixmap: np.ndarray | None = None):
    """resvg_render_node restated (lib.rs:55-70); None when the node has no box."""
    L = lib()
    L.oracle_render_node.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_float), C.c_uint32, C.c_uint32,
                                     C.c_void_p]
    if pixmap is None:
        pixmap = np.zeros((height, width, 4), dtype=np.uint8)
    ts = (C.c_float * 6)(*[float(v) for v in transform])
    r = L.oracle_render_node(C.cast(tree_view_ptr, C.c_void_p), node_id.encode(), ts, width, height,
                             pixmap.ctypes.data)
    return pixmap if r == 0 else None


def render_parallel(tree_view_ptr, transform, width: int, height: int, threads: int,
                    pixmap: np.ndarray | None = None) -> np.ndarray:
    """All-core timing variant of render(): strips of the canvas on `threads` threads."""
    if pixmap is None:
        pixmap = np.zeros((height, width, 4), dtype=np.uint8)
    ts = (C.c_float * 6)(*[float(v) for v in transform])
    r = lib().oracle_render_parallel(C.cast(tree_view_ptr, C.c_void_p), ts, width, height, pixmap.ctypes.data,
                                     threads)
    if r != 0:
        raise RuntimeError("oracle_render_parallel failed")
    return pixmap


class GeneratedTree:
    """A seeded synthetic tree built inside the oracle library (the product's
    generator source compiled in), so that no product library is loaded."""

    def __init__(self, config: int, seed: int, index: int, scale: float = 1.0):
        L = lib()
        L.oracle_tree_generate.restype = C.c_void_p
        L.oracle_tree_generate.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_float]
        L.oracle_tree_view.restype = C.c_void_p
        L.oracle_tree_view.argtypes = [C.c_void_p]
        L.oracle_tree_free.restype = None
        L.oracle_tree_free.argtypes = [C.c_void_p]
        self._h = L.oracle_tree_generate(int(config), int(seed), int(index), float(scale))
        if not self._h:
            raise ValueError("unknown config %r" % config)
        self._view = L.oracle_tree_view(self._h)
        w, h = C.cast(self._view, C.POINTER(C.c_float * 2)).contents
        self.size = (float(w), float(h))
        self.path_count = _view_path_count(self._view)

    def view(self):
        return self._view

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.oracle_tree_free(h)
            self._h = None


def _view_path_count(view_ptr) -> int:
    # rgpu_tree_view: width, height, groups*, group_count, children*, child_count, paths*, path_count
    class _Head(C.Structure):
        _fields_ = [("width", C.c_float), ("height", C.c_float), ("groups", C.c_void_p), ("group_count", C.c_uint32),
                    ("children", C.c_void_p), ("child_count", C.c_uint32), ("paths", C.c_void_p),
                    ("path_count", C.c_uint32)]
    return int(C.cast(view_ptr, C.POINTER(_Head)).contents.path_count)


def render_many(views, transforms, sizes, threads: int, pixmaps=None):
    """Renders whole trees in parallel, one tree per host thread at a time, in
    the order given; each result is identical to render() of that tree.
    `views` are rgpu_tree_view pointers, `sizes` (w, h) pairs.  Returns the
    pixmaps (fresh transparent ones when None)."""
    n = len(views)
    if pixmaps is None:
        pixmaps = [np.zeros((int(h), int(w), 4), dtype=np.uint8) for w, h in sizes]
    L = lib()
    L.oracle_render_many.restype = C.c_int
    L.oracle_render_many.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_float), C.POINTER(C.c_uint32),
                                     C.POINTER(C.c_uint32), C.POINTER(C.c_void_p), C.c_uint32, C.c_uint32]
    vs = (C.c_void_p * max(1, n))(*[C.cast(v, C.c_void_p).value for v in views])
    ts = (C.c_float * max(6, 6 * n))(*[float(x) for t in transforms for x in t])
    ws = (C.c_uint32 * max(1, n))(*[int(w) for w, _ in sizes])
    hs = (C.c_uint32 * max(1, n))(*[int(h) for _, h in sizes])
    for p, (w, h) in zip(pixmaps, sizes):
        assert p.dtype == np.uint8 and p.shape == (int(h), int(w), 4) and p.flags.c_contiguous
    ps = (C.c_void_p * max(1, n))(*[p.ctypes.data for p in pixmaps])
    if L.oracle_render_many(vs, ts, ws, hs, ps, n, max(1, int(threads))) != 0:
        raise RuntimeError("oracle_render_many failed")
    return pixmaps


def _img_op(name, img, *args):
    assert img.dtype == np.uint8 and img.ndim == 3 and img.shape[2] == 4
    out = np.ascontiguousarray(img).copy()
    getattr(lib(), name)(out.ctypes.data, out.shape[1], out.shape[0], *args)
    return out


def box_blur(img, sx, sy):
    return _img_op("oracle_box_blur", img, C.c_double(sx), C.c_double(sy))


def iir_blur(img, sx, sy):
    return _img_op("oracle_iir_blur", img, C.c_double(sx), C.c_double(sy))


def morphology(img, dilate, rx, ry):
    return _img_op("oracle_morphology", img, int(dilate), C.c_float(rx), C.c_float(ry))


def to_linear(img):
    return _img_op("oracle_to_linear", img)


def to_srgb(img):
    return _img_op("oracle_to_srgb", img)


def filter_apply(img, filt, prims, merge_inputs=(), transform=(1, 0, 0, 1, 0, 0)):
    """filter::apply on a copy of `img` (premultiplied RGBA8, (h, w, 4)); `filt`
    and `prims` are the ctypes records the product's Tree.add_filter takes."""
    assert img.dtype == np.uint8 and img.ndim == 3 and img.shape[2] == 4
    out = np.ascontiguousarray(img).copy()
    arr = (type(prims[0]) * len(prims))(*prims) if prims else None
    m = (C.c_int32 * max(1, len(merge_inputs)))(*merge_inputs)
    ts = (C.c_float * 6)(*[float(v) for v in transform])
    lib().oracle_filter_apply(C.byref(filt), arr, len(prims), m, len(merge_inputs), ts, out.ctypes.data,
                              out.shape[1], out.shape[0])
    return out


def _soft_struct(arrays):
    """rgpu_soft_batch over host numpy arrays (kept alive by the caller)."""
    from resvg_gb300 import _abi
    b = _abi.SoftBatch()
    b.scenes, b.width, b.height, b.paths_per_scene = (int(arrays[k]) for k in ("scenes", "width", "height", "paths"))
    b.total_segments = int(arrays["seg_offset"][-1])
    for f, k in (("seg_offset", "seg_offset"), ("points", "points"), ("paint_kind", "paint_kind"),
                 ("colors", "colors"), ("stop_offsets", "stop_offsets"), ("stop_colors", "stop_colors"),
                 ("grad_line", "grad_line"), ("sigma", "sigma"), ("opacity", "opacity")):
        setattr(b, f, arrays[k].ctypes.data if k in arrays else None)
    return b


def soft_forward(arrays):
    """FP64 forward: (image, blurred) as (S, H, W, 4) float64 arrays."""
    L = lib()
    L.oracle_soft_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    b = _soft_struct(arrays)
    shape = (int(arrays["scenes"]), int(arrays["height"]), int(arrays["width"]), 4)
    im = np.zeros(shape, np.float64)
    bl = np.zeros(shape, np.float64)
    L.oracle_soft_forward(C.byref(b), im.ctypes.data, bl.ctypes.data)
    return im, bl


def soft_dloss(arrays, target, direction):
    """(loss, dloss/dv) in FP64 for a parameter direction v (dict of float64
    arrays keyed like the parameters; missing keys are zero)."""
    L = lib()
    L.oracle_soft_dloss.argtypes = [C.c_void_p, C.c_void_p] + [C.c_void_p] * 6 + [C.c_void_p, C.c_void_p]
    b = _soft_struct(arrays)
    t = np.ascontiguousarray(target, dtype=np.float32)
    keep = []

    def ptr(k):
        if k not in direction:
            return None
        a = np.ascontiguousarray(direction[k], dtype=np.float64)
        keep.append(a)
        return a.ctypes.data
    loss = C.c_double()
    dl = C.c_double()
    L.oracle_soft_dloss(C.byref(b), t.ctypes.data, ptr("points"), ptr("colors"), ptr("stop_offsets"),
                        ptr("stop_colors"), ptr("sigma"), ptr("opacity"), C.byref(loss), C.byref(dl))
    return loss.value, dl.value
