"""resvg_gb300 — GB300-native rendering backend for resvg (host-side Python API).

The native library (libresvg_gb300.so, built in-tree by resvg_gb300.build)
holds the tree builder, the host flattener and the sm_103a CUDA kernels; this
module is a thin ctypes layer over its C ABI (include/resvg_gpu.h).  Rendering
always runs on the GPU; there is no CPU fallback, and a missing or unusable
device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import (Clip, Filter, Group, Mask, Paint, Path, Primitive, Stop, Transform)  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_native", "libresvg_gb300.so")
_lib = None


class RenderError(RuntimeError):
    pass


def lib() -> C.CDLL:
    """Loads libresvg_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RenderError("libresvg_gb300.so is not built; run `python -m resvg_gb300.build`")
        L = C.CDLL(LIB_PATH)
        _abi.declare(L)
        _declare_render(L)
        _lib = L
    return _lib


def _declare_render(L):
    P = C.c_void_p
    L.resvg_render.restype = None
    L.resvg_render.argtypes = [P, _abi.ResvgTransform, C.c_uint32, C.c_uint32, P]
    L.resvg_render_node.restype = C.c_bool
    L.resvg_render_node.argtypes = [P, C.c_char_p, _abi.ResvgTransform, C.c_uint32, C.c_uint32, P]
    L.rgpu_init.restype = C.c_int
    L.rgpu_init.argtypes = [C.c_int]
    L.rgpu_last_error.restype = C.c_char_p
    L.rgpu_last_warning.restype = C.c_char_p
    L.rgpu_render_device.restype = C.c_int
    L.rgpu_render_device.argtypes = [P, _abi.ResvgTransform, C.c_uint32, C.c_uint32, P, C.c_uint32, P]
    L.rgpu_render_batch.restype = C.c_int
    L.rgpu_render_batch.argtypes = [C.POINTER(P), C.POINTER(_abi.ResvgTransform), C.c_uint32,
                                    C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(P), P]
    L.rgpu_set_tuning.restype = C.c_int
    L.rgpu_set_tuning.argtypes = [C.POINTER(_abi.Tuning)]
    L.rgpu_get_tuning.restype = C.c_int
    L.rgpu_get_tuning.argtypes = [C.POINTER(_abi.Tuning)]
    L.rgpu_get_stats.restype = C.c_int
    L.rgpu_get_stats.argtypes = [C.POINTER(_abi.Stats)]
    for n in ("rgpu_filter_box_blur", "rgpu_filter_iir_blur"):
        if hasattr(L, n):
            getattr(L, n).restype = C.c_int
            getattr(L, n).argtypes = [P, C.c_uint32, C.c_uint32, C.c_double, C.c_double, P]
    if hasattr(L, "rgpu_filter_morphology"):
        L.rgpu_filter_morphology.restype = C.c_int
        L.rgpu_filter_morphology.argtypes = [P, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_float, P]
    if hasattr(L, "rgpu_filter_color_space"):
        L.rgpu_filter_color_space.restype = C.c_int
        L.rgpu_filter_color_space.argtypes = [P, C.c_uint32, C.c_uint32, C.c_int, P]
    if hasattr(L, "rgpu_filter_apply"):
        L.rgpu_filter_apply.restype = C.c_int
        L.rgpu_filter_apply.argtypes = [C.POINTER(_abi.Filter), C.POINTER(_abi.Primitive), C.c_uint32,
                                        C.POINTER(C.c_int32), C.c_uint32, _abi.ResvgTransform, P, C.c_uint32,
                                        C.c_uint32, P]


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = lib().rgpu_last_error().decode(errors="replace")
        raise RenderError("%s failed (status %d): %s" % (what, status, msg))


class Tree:
    """A resolved render tree (the usvg::Tree stand-in), built node by node or
    generated.  Group 0 is the root."""

    def __init__(self, width: float = 0, height: float = 0, _handle=None):
        self._h = _handle if _handle is not None else lib().rgpu_tree_new(float(width), float(height))
        if not self._h:
            raise ValueError("invalid tree size")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.rgpu_tree_free(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @staticmethod
    def generate(config: int, seed: int = 0, index: int = 0, scale: float = 1.0) -> "Tree":
        h = lib().rgpu_tree_generate(int(config), int(seed), int(index), float(scale))
        if not h:
            raise ValueError("unknown config %r" % config)
        return Tree(_handle=h)

    def add_group(self, parent: int, group: Group) -> int:
        return lib().rgpu_tree_add_group(self._h, parent, C.byref(group))

    def add_paint(self, paint: Paint, stops=()) -> int:
        arr = (Stop * max(1, len(stops)))(*stops)
        return lib().rgpu_tree_add_paint(self._h, C.byref(paint), arr, len(stops))

    def add_path(self, parent: int, path: Path, verbs, points, dashes=()) -> int:
        v = np.ascontiguousarray(np.asarray(verbs, dtype=np.uint8))
        p = np.ascontiguousarray(np.asarray(points, dtype=np.float32).reshape(-1))
        d = np.ascontiguousarray(np.asarray(dashes, dtype=np.float32).reshape(-1))
        return lib().rgpu_tree_add_path(
            self._h, parent, C.byref(path), v.ctypes.data_as(C.POINTER(C.c_uint8)), len(v),
            p.ctypes.data_as(C.POINTER(C.c_float)), len(p) // 2,
            d.ctypes.data_as(C.POINTER(C.c_float)) if len(d) else None, len(d))

    def add_clip(self, clip: Clip) -> int:
        return lib().rgpu_tree_add_clip(self._h, C.byref(clip))

    def add_mask(self, mask: Mask) -> int:
        return lib().rgpu_tree_add_mask(self._h, C.byref(mask))

    def add_filter(self, filt: Filter, prims, merge_inputs=()) -> int:
        arr = (Primitive * max(1, len(prims)))(*prims)
        m = (C.c_int32 * max(1, len(merge_inputs)))(*merge_inputs)
        return lib().rgpu_tree_add_filter(self._h, C.byref(filt), arr, len(prims), m, len(merge_inputs))

    def add_image(self, rgba) -> int:
        """A decoded raster image: a (h, w, 4) uint8 array, premultiplied."""
        a = np.ascontiguousarray(rgba, dtype=np.uint8)
        assert a.ndim == 3 and a.shape[2] == 4
        return lib().rgpu_tree_add_image(self._h, a.shape[1], a.shape[0], a.ctypes.data)

    def set_node_id(self, kind: int, index: int, node_id: str) -> None:
        """Gives group (kind NODE_GROUP) or path (NODE_PATH) `index` its SVG id."""
        check(lib().rgpu_tree_set_node_id(self._h, int(kind), int(index), node_id.encode()), "set_node_id")

    def find_node(self, node_id: str):
        """(kind, index) of the node resvg_render_node renders for this SVG id
        (usvg's node_by_id: first match in depth-first pre-order), or None."""
        k, i = C.c_uint32(), C.c_uint32()
        if lib().rgpu_tree_find_node(self._h, node_id.encode(), C.byref(k), C.byref(i)) != 0:
            return None
        return k.value, i.value

    def set_group_filters(self, group: int, filters) -> None:
        arr = (C.c_uint32 * max(1, len(filters)))(*filters)
        check(lib().rgpu_tree_set_group_filters(self._h, group, arr, len(filters)), "set_group_filters")

    def finalize(self) -> None:
        check(lib().rgpu_tree_finalize(self._h), "finalize")

    def view(self):
        """Pointer to the rgpu_tree_view (finalizes first if needed)."""
        return lib().rgpu_tree_get_view(self._h)

    @property
    def size(self):
        v = self.view().contents
        return v.width, v.height


def last_warning() -> str:
    """Warnings of this thread's last render or filter call: parts the
    reference skips or clears with a log message (a failing filter clears its
    layer) while the call itself succeeded."""
    return lib().rgpu_last_warning().decode(errors="replace")


def _rt(transform) -> _abi.ResvgTransform:
    return _abi.ResvgTransform(*[float(x) for x in transform])


def init(device: int = 0) -> None:
    check(lib().rgpu_init(device), "rgpu_init")


def render(tree: Tree, transform=(1, 0, 0, 1, 0, 0), width: int | None = None, height: int | None = None,
           pixmap: np.ndarray | None = None) -> np.ndarray:
    """resvg_render through the C ABI: draws `tree` onto a host pixmap
    (premultiplied RGBA8, (h, w, 4); transparent when None) and returns it."""
    if pixmap is None:
        w = int(width if width is not None else tree.size[0])
        h = int(height if height is not None else tree.size[1])
        pixmap = np.zeros((h, w, 4), dtype=np.uint8)
    h, w = pixmap.shape[:2]
    assert pixmap.dtype == np.uint8 and pixmap.flags.c_contiguous and pixmap.shape[2] == 4
    tree.view()
    lib().resvg_render(tree.handle, _rt(transform), w, h, pixmap.ctypes.data)
    err = lib().rgpu_last_error()
    if err:
        raise RenderError(err.decode(errors="replace"))
    return pixmap


def node_abs_bbox(tree: Tree, node_id: str):
    """Absolute layer bounding box (x, y, w, h) of the node with this SVG id,
    the box resvg's render_node places at the pixmap origin; None for an
    unknown id or a zero-sized box."""
    node = tree.find_node(node_id)
    return None if node is None else node_abs_bbox_at(tree, *node)


def node_abs_bbox_at(tree: Tree, kind: int, idx: int):
    """node_abs_bbox for node (kind, index): NODE_GROUP or NODE_PATH."""
    v = tree.view().contents
    is_path = kind == _abi.NODE_PATH
    gp = [-1] * v.group_count
    pp = [-1] * v.path_count
    for g in range(v.group_count):
        gr = v.groups[g]
        for k in range(gr.child_count):
            n = v.children[gr.child_offset + k]
            (gp if n.kind == _abi.NODE_GROUP else pp)[n.index] = g
    f32 = np.float32

    def concat(a, b):  # tiny-skia Transform::concat (f64 products for skewed matrices)
        if a == (1, 0, 0, 1, 0, 0):
            return b
        if b == (1, 0, 0, 1, 0, 0):
            return a
        if a[1] == 0 and a[2] == 0 and b[1] == 0 and b[2] == 0:
            return (f32(a[0] * b[0]), 0.0, 0.0, f32(a[3] * b[3]), f32(f32(a[0] * b[4]) + a[4]), f32(f32(a[3] * b[5]) + a[5]))
        m = lambda p, q, r, s_: float(f32(float(p) * float(q) + float(r) * float(s_)))  # noqa: E731
        return (m(a[0], b[0], a[2], b[1]), m(a[1], b[0], a[3], b[1]), m(a[0], b[2], a[2], b[3]),
                m(a[1], b[2], a[3], b[3]), float(f32(m(a[0], b[4], a[2], b[5]) + a[4])),
                float(f32(m(a[1], b[4], a[3], b[5]) + a[5])))
    tup = lambda t: tuple(float(x) for x in t.tuple())  # noqa: E731
    ab = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0) if is_path else tup(v.groups[idx].transform)
    g = pp[idx] if is_path else gp[idx]
    while g >= 0:
        ab = concat(tup(v.groups[g].transform), ab)
        g = gp[g]
    if is_path:
        p = v.paths[idx]
        r = (p.bbox_x, p.bbox_y, p.bbox_x + p.bbox_w, p.bbox_y + p.bbox_h)
    else:
        gr = v.groups[idx]
        if not gr.has_layer_bbox:
            return None
        r = (gr.layer_x, gr.layer_y, gr.layer_x + gr.layer_w, gr.layer_y + gr.layer_h)
    if not (r[2] > r[0] and r[3] > r[1]):
        return None
    xs, ys = [], []
    for x, y in ((r[0], r[1]), (r[2], r[1]), (r[2], r[3]), (r[0], r[3])):
        x, y = f32(x), f32(y)
        xs.append(float(f32(f32(f32(x * f32(ab[0])) + f32(y * f32(ab[2]))) + f32(ab[4]))))
        ys.append(float(f32(f32(f32(x * f32(ab[1])) + f32(y * f32(ab[3]))) + f32(ab[5]))))
    l, t, rr, b = min(xs), min(ys), max(xs), max(ys)
    return (l, t, rr - l, b - t) if rr > l and b > t else None


def render_node(tree: Tree, node_id: str, transform, width: int, height: int,
                pixmap: np.ndarray | None = None) -> np.ndarray | None:
    """resvg_render_node through the C ABI: `node_id` is an SVG id given with
    Tree.set_node_id; None when the id is unknown or the node's bounding box
    is empty."""
    if pixmap is None:
        pixmap = np.zeros((int(height), int(width), 4), dtype=np.uint8)
    tree.view()
    ok = lib().resvg_render_node(tree.handle, node_id.encode(), _rt(transform), pixmap.shape[1], pixmap.shape[0],
                                 pixmap.ctypes.data)
    return pixmap if ok else None


def render_device(tree: Tree, transform, width: int, height: int, device_ptr: int, stride: int,
                  stream: int = 0) -> None:
    """Renders onto a device pixmap (e.g. a torch.uint8 CUDA tensor's data_ptr())."""
    tree.view()
    check(lib().rgpu_render_device(tree.handle, _rt(transform), width, height, C.c_void_p(device_ptr), stride,
                                   C.c_void_p(stream)), "rgpu_render_device")


def render_batch(trees, transforms, widths, heights, device_ptrs, stream: int = 0) -> None:
    n = len(trees)
    for t in trees:
        t.view()
    th = (C.c_void_p * n)(*[t.handle for t in trees])
    ts = (_abi.ResvgTransform * n)(*[_rt(t) for t in transforms])
    ws = (C.c_uint32 * n)(*widths)
    hs = (C.c_uint32 * n)(*heights)
    ps = (C.c_void_p * n)(*device_ptrs)
    check(lib().rgpu_render_batch(th, ts, n, ws, hs, ps, C.c_void_p(stream)), "rgpu_render_batch")


def set_tuning(band_rows: int = 0, pixels_per_thread: int = 0) -> None:
    """Raster work decomposition; 0 = automatic."""
    t = _abi.Tuning(band_rows, pixels_per_thread, 0)
    check(lib().rgpu_set_tuning(C.byref(t)), "rgpu_set_tuning")


def set_batch_chunks(chunks: int) -> None:
    """Chunks of render_batch's host/device pipeline: 0 automatic (8 for 64
    scenes or more), 1 one submission, n n chunks."""
    L = lib()
    L.rgpu_set_batch_chunks.restype = C.c_int
    L.rgpu_set_batch_chunks.argtypes = [C.c_uint32]
    check(L.rgpu_set_batch_chunks(int(chunks)))


def set_stroke_mode(on_device: bool) -> None:
    """Build stroke outlines on the device (default) or on the host; both run
    the same stroker and give identical outlines."""
    L = lib()
    L.rgpu_set_stroke_mode.restype = C.c_int
    L.rgpu_set_stroke_mode.argtypes = [C.c_int]
    check(L.rgpu_set_stroke_mode(1 if on_device else 0))


class StrokeDesc(C.Structure):
    _fields_ = [("verb_off", C.c_uint32), ("verb_cnt", C.c_uint32), ("pt_off", C.c_uint32), ("pt_cnt", C.c_uint32),
                ("width", C.c_float), ("miter_limit", C.c_float), ("res_scale", C.c_float),
                ("cap", C.c_uint32), ("join", C.c_uint32), ("dash_off", C.c_uint32), ("dash_cnt", C.c_uint32),
                ("dash_phase", C.c_float)]


def stroke_paths(paths, on_device: bool = True):
    """tiny-skia's Path::dash + Path::stroke for many paths at once
    (rgpu_stroke_paths).  `paths`: (verbs, points (n, 2), width, miter_limit,
    cap, join, res_scale[, dashes, dash_phase]) tuples.  Returns one (verbs
    uint8, points float32 (m, 2)) outline per path (empty arrays when the
    stroke produces nothing)."""
    L = lib()
    L.rgpu_stroke_paths.restype = C.c_int
    P = C.c_void_p
    L.rgpu_stroke_paths.argtypes = [C.POINTER(StrokeDesc), C.c_uint32, P, C.c_uint32, P, C.c_uint32, P, C.c_uint32,
                                    C.c_int, P, C.c_uint32, P, C.c_uint32, P]
    n = len(paths)
    descs = (StrokeDesc * max(n, 1))()
    vs, ps, ds = [], [], []
    vo = po = do = 0
    for i, path in enumerate(paths):
        v, pt, width, miter, cap, join, rs = path[:7]
        dash = np.asarray(path[7] if len(path) > 7 and path[7] is not None else [], np.float32).reshape(-1)
        phase = float(path[8]) if len(path) > 8 else 0.0
        v = np.ascontiguousarray(np.asarray(v, dtype=np.uint8))
        pt = np.ascontiguousarray(np.asarray(pt, dtype=np.float32).reshape(-1, 2))
        descs[i] = StrokeDesc(vo, len(v), po, len(pt), width, miter, rs, cap, join, do, len(dash), phase)
        vs.append(v)
        ps.append(pt)
        ds.append(dash)
        vo += len(v)
        po += len(pt)
        do += len(dash)
    verbs = np.concatenate(vs) if vs else np.zeros(1, np.uint8)
    pts = np.concatenate(ps) if ps else np.zeros((1, 2), np.float32)
    dashes = np.concatenate(ds + [np.zeros(1, np.float32)]).astype(np.float32)
    vcap, pcap = 64 * max(vo, 1) + 256 * n + 64, 64 * max(po, 1) + 256 * n + 64
    while True:
        ov = np.zeros(vcap, np.uint8)
        op = np.zeros((pcap, 2), np.float32)
        counts = np.zeros(2 * max(n, 1), np.uint32)
        r = L.rgpu_stroke_paths(descs, n, verbs.ctypes.data, len(verbs), pts.ctypes.data, len(pts),
                                dashes.ctypes.data, len(dashes), 1 if on_device else 0, ov.ctypes.data, vcap,
                                op.ctypes.data, pcap, counts.ctypes.data)
        if r == 5:  # RGPU_ERR_CAPACITY: larger output arrays
            vcap, pcap = 4 * vcap, 4 * pcap
            continue
        check(r, "rgpu_stroke_paths")
        break
    out, a, b = [], 0, 0
    for i in range(n):
        nv, np_ = int(counts[2 * i]), int(counts[2 * i + 1])
        out.append((ov[a:a + nv].copy(), op[b:b + np_].copy()))
        a += nv
        b += np_
    return out


def set_tuning_table(entries) -> None:
    """Band rows per (max stream width, max stream draws) bucket, used for
    streams whose band rows the tuning leaves automatic: entries are
    (max_width, max_draws, band_rows) tuples, first match wins."""
    L = lib()
    L.rgpu_set_tuning_table.restype = C.c_int
    L.rgpu_set_tuning_table.argtypes = [C.POINTER(_abi.TuningEntry), C.c_uint32]
    arr = (_abi.TuningEntry * max(1, len(entries)))(*[_abi.TuningEntry(int(w), int(d), int(b), 0)
                                                       for w, d, b in entries])
    check(L.rgpu_set_tuning_table(arr, len(entries)), "rgpu_set_tuning_table")


def get_tuning_table():
    L = lib()
    L.rgpu_get_tuning_table.restype = C.c_int
    L.rgpu_get_tuning_table.argtypes = [C.POINTER(_abi.TuningEntry), C.c_uint32, C.POINTER(C.c_uint32)]
    n = C.c_uint32(0)
    check(L.rgpu_get_tuning_table(None, 0, C.byref(n)), "rgpu_get_tuning_table")
    arr = (_abi.TuningEntry * max(1, n.value))()
    check(L.rgpu_get_tuning_table(arr, n.value, C.byref(n)), "rgpu_get_tuning_table")
    return [(e.max_width, e.max_draws, e.band_rows) for e in arr[:n.value]]


def get_tuning():
    t = _abi.Tuning()
    check(lib().rgpu_get_tuning(C.byref(t)), "rgpu_get_tuning")
    return t.band_rows, t.pixels_per_thread


def autotune(trees, transforms, widths, heights, device_ptrs, candidates, reps: int = 3, strides=None):
    """Times each (band_rows, pixels_per_thread) candidate on the given scenes
    (rgpu_autotune), keeps the fastest as the current tuning and returns
    ((band_rows, pixels_per_thread), ms per render)."""
    L = lib()
    P = C.c_void_p
    L.rgpu_autotune.restype = C.c_int
    L.rgpu_autotune.argtypes = [C.POINTER(P), C.POINTER(_abi.ResvgTransform), C.c_uint32, C.POINTER(C.c_uint32),
                                C.POINTER(C.c_uint32), C.POINTER(P), C.POINTER(C.c_uint32),
                                C.POINTER(_abi.Tuning), C.c_uint32, C.c_uint32, C.POINTER(_abi.Tuning),
                                C.POINTER(C.c_float)]
    n = len(trees)
    for t in trees:
        t.view()
    th = (P * n)(*[t.handle for t in trees])
    ts = (_abi.ResvgTransform * n)(*[_rt(t) for t in transforms])
    ws = (C.c_uint32 * n)(*[int(w) for w in widths])
    hs = (C.c_uint32 * n)(*[int(h) for h in heights])
    ps = (P * n)(*[int(p) for p in device_ptrs])
    ss = (C.c_uint32 * n)(*[int(s) for s in strides]) if strides is not None else None
    cand = (_abi.Tuning * len(candidates))(*[_abi.Tuning(b, p, 0) for b, p in candidates])
    best = _abi.Tuning()
    ms = C.c_float(0)
    check(L.rgpu_autotune(th, ts, n, ws, hs, ps, ss, cand, len(candidates), reps, C.byref(best), C.byref(ms)),
          "rgpu_autotune")
    return (best.band_rows, best.pixels_per_thread), ms.value


def stats():
    s = _abi.Stats()
    check(lib().rgpu_get_stats(C.byref(s)), "rgpu_get_stats")
    return {k: getattr(s, k) for k, _ in _abi.Stats._fields_}


class SceneStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("streams", "draws", "commands", "segments", "edges", "binned_edges",
                                           "work_items", "grid", "pixels_per_thread", "kernel_launches",
                                           "output_pixels", "layer_pixels", "record_bytes")]


def _declare_scene(L):
    P = C.c_void_p
    L.rgpu_scene_prepare.restype = C.c_int
    L.rgpu_scene_prepare.argtypes = [C.POINTER(P), C.POINTER(_abi.ResvgTransform), C.c_uint32,
                                     C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(P),
                                     C.POINTER(C.c_uint32), C.POINTER(P)]
    L.rgpu_scene_render.restype = C.c_int
    L.rgpu_scene_render.argtypes = [P, P]
    L.rgpu_scene_set_timing.restype = C.c_int
    L.rgpu_scene_set_timing.argtypes = [P, C.c_int]
    L.rgpu_scene_check.restype = C.c_int
    L.rgpu_scene_check.argtypes = [P, C.POINTER(C.c_float)]
    L.rgpu_scene_info.restype = C.c_int
    L.rgpu_scene_info.argtypes = [P, C.POINTER(SceneStats)]
    L.rgpu_scene_free.restype = None
    L.rgpu_scene_free.argtypes = [P]


class Scene:
    """A prepared scene (device-resident display list) over one or many trees.

    `device_ptrs` are the device pixmaps rendered into (premultiplied RGBA8,
    e.g. torch uint8 CUDA tensors' data_ptr()).  render() enqueues the whole
    pipeline on `stream` (a cudaStream_t handle; 0 = the library's stream);
    from the second render on it replays a captured CUDA graph."""

    def __init__(self, trees, transforms, widths, heights, device_ptrs, strides=None):
        L = lib()
        if not hasattr(L, "_scene_declared"):
            _declare_scene(L)
            L._scene_declared = True
        n = len(trees)
        self._trees = list(trees)  # keep alive
        for t in trees:
            t.view()
        th = (C.c_void_p * n)(*[t.handle for t in trees])
        ts = (_abi.ResvgTransform * n)(*[_rt(t) for t in transforms])
        ws = (C.c_uint32 * n)(*[int(w) for w in widths])
        hs = (C.c_uint32 * n)(*[int(h) for h in heights])
        ps = (C.c_void_p * n)(*[int(p) for p in device_ptrs])
        ss = (C.c_uint32 * n)(*[int(s) for s in strides]) if strides is not None else None
        out = C.c_void_p()
        check(L.rgpu_scene_prepare(th, ts, n, ws, hs, ps, ss, C.byref(out)), "rgpu_scene_prepare")
        self._h = out

    def render(self, stream: int = 0) -> None:
        check(lib().rgpu_scene_render(self._h, C.c_void_p(stream)), "rgpu_scene_render")

    def set_timing(self, enabled: bool) -> None:
        check(lib().rgpu_scene_set_timing(self._h, int(bool(enabled))), "rgpu_scene_set_timing")

    def check(self) -> float:
        """Synchronises; raises on kernel error flags; returns the raster kernel ms of the last render."""
        ms = C.c_float(0)
        check(lib().rgpu_scene_check(self._h, C.byref(ms)), "rgpu_scene_check")
        return ms.value

    def info(self) -> dict:
        st = SceneStats()
        check(lib().rgpu_scene_info(self._h, C.byref(st)), "rgpu_scene_info")
        return {k: getattr(st, k) for k, _ in SceneStats._fields_}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.rgpu_scene_free(h)
            self._h = None


def _dev_filter(name, tensor, *args, stream=None):
    """Runs a filter kernel in place on a CUDA uint8 tensor of shape (h, w, 4):
    synchronously on the library's stream, or enqueued on `stream` (a CUDA
    stream handle) and returning at once."""
    assert tensor.is_cuda and tensor.dtype.itemsize == 1 and tensor.dim() == 3 and tensor.shape[2] == 4
    assert tensor.is_contiguous()
    h, w = tensor.shape[0], tensor.shape[1]
    check(getattr(lib(), name)(C.c_void_p(tensor.data_ptr()), w, h, *args, C.c_void_p(stream) if stream else None),
          name)
    return tensor


def box_blur(tensor, sx, sy, stream=None):
    return _dev_filter("rgpu_filter_box_blur", tensor, C.c_double(sx), C.c_double(sy), stream=stream)


def iir_blur(tensor, sx, sy, stream=None):
    return _dev_filter("rgpu_filter_iir_blur", tensor, C.c_double(sx), C.c_double(sy), stream=stream)


def set_iir_precision(mode: int) -> None:
    """0: the IIR blur in f64 in the reference's order (bit-exact, default);
    1: an FP32 chunked parallel scan (within 1 per channel)."""
    L = lib()
    L.rgpu_set_iir_precision.restype = C.c_int
    L.rgpu_set_iir_precision.argtypes = [C.c_uint32]
    check(L.rgpu_set_iir_precision(int(mode)), "rgpu_set_iir_precision")


def morphology(tensor, dilate, rx, ry, stream=None):
    return _dev_filter("rgpu_filter_morphology", tensor, int(dilate), C.c_float(rx), C.c_float(ry), stream=stream)


def color_space(tensor, to_linear, stream=None):
    return _dev_filter("rgpu_filter_color_space", tensor, int(to_linear), stream=stream)


def filter_apply(tensor, filt: Filter, prims, merge_inputs=(), transform=(1, 0, 0, 1, 0, 0), stream=None):
    """Applies a whole filter (region and primitive chain, as Tree.add_filter
    takes them) in place to a CUDA uint8 tensor (h, w, 4) holding the filtered
    layer, under the layer transform (crates/resvg/src/filter/mod.rs:335)."""
    assert tensor.is_cuda and tensor.dtype.itemsize == 1 and tensor.dim() == 3 and tensor.shape[2] == 4
    assert tensor.is_contiguous()
    h, w = tensor.shape[0], tensor.shape[1]
    arr = (Primitive * max(1, len(prims)))(*prims)
    m = (C.c_int32 * max(1, len(merge_inputs)))(*merge_inputs)
    check(lib().rgpu_filter_apply(C.byref(filt), arr, len(prims), m, len(merge_inputs), _rt(transform),
                                  C.c_void_p(tensor.data_ptr()), w, h, C.c_void_p(stream) if stream else None),
          "rgpu_filter_apply")
    return tensor
