"""ctypes mirror of include/rgpu_tree.h and include/resvg_gpu.h."""
from __future__ import annotations

import ctypes as C

u8, u32, i32, f32 = C.c_uint8, C.c_uint32, C.c_int32, C.c_float


class Transform(C.Structure):
    _fields_ = [("sx", f32), ("ky", f32), ("kx", f32), ("sy", f32), ("tx", f32), ("ty", f32)]

    @staticmethod
    def identity():
        return Transform(1, 0, 0, 1, 0, 0)

    @staticmethod
    def of(t):
        return Transform(*[float(v) for v in t])

    def tuple(self):
        return (self.sx, self.ky, self.kx, self.sy, self.tx, self.ty)


class Stop(C.Structure):
    _fields_ = [("offset", f32), ("r", u8), ("g", u8), ("b", u8), ("_pad", u8), ("opacity", f32)]


class Paint(C.Structure):
    _fields_ = [("kind", u32), ("r", u8), ("g", u8), ("b", u8), ("_pad", u8),
                ("x1", f32), ("y1", f32), ("x2", f32), ("y2", f32),
                ("cx", f32), ("cy", f32), ("r_", f32), ("fx", f32), ("fy", f32), ("fr", f32),
                ("spread", u32), ("transform", Transform), ("stop_offset", u32), ("stop_count", u32)]


class Path(C.Structure):
    _fields_ = [("verb_offset", u32), ("verb_count", u32), ("point_offset", u32), ("point_count", u32),
                ("fill_paint", i32), ("fill_opacity", f32), ("fill_rule", u32),
                ("stroke_paint", i32), ("stroke_opacity", f32), ("stroke_width", f32), ("miter_limit", f32),
                ("line_cap", u32), ("line_join", u32), ("dash_offset", u32), ("dash_count", u32),
                ("dash_phase", f32), ("stroke_first", u32), ("anti_alias", u32), ("visible", u32),
                ("bbox_x", f32), ("bbox_y", f32), ("bbox_w", f32), ("bbox_h", f32)]


class Node(C.Structure):
    _fields_ = [("kind", u32), ("index", u32)]


class Group(C.Structure):
    _fields_ = [("transform", Transform), ("opacity", f32), ("blend", u32), ("isolate", u32),
                ("clip_path", i32), ("mask", i32), ("filter_offset", u32), ("filter_count", u32),
                ("child_offset", u32), ("child_count", u32), ("has_layer_bbox", u32),
                ("layer_x", f32), ("layer_y", f32), ("layer_w", f32), ("layer_h", f32)]


class Clip(C.Structure):
    _fields_ = [("transform", Transform), ("clip_path", i32), ("root", u32)]


class Mask(C.Structure):
    _fields_ = [("x", f32), ("y", f32), ("w", f32), ("h", f32), ("kind", u32), ("mask", i32), ("root", u32)]


PRIM_F = 64


class Primitive(C.Structure):
    _fields_ = [("kind", u32), ("x", f32), ("y", f32), ("w", f32), ("h", f32), ("linear_rgb", u32),
                ("in1", i32), ("in2", i32), ("i", i32 * 8), ("f", f32 * PRIM_F)]


class Filter(C.Structure):
    _fields_ = [("x", f32), ("y", f32), ("w", f32), ("h", f32), ("prim_offset", u32), ("prim_count", u32)]


class TreeView(C.Structure):
    _fields_ = [("width", f32), ("height", f32),
                ("groups", C.POINTER(Group)), ("group_count", u32),
                ("children", C.POINTER(Node)), ("child_count", u32),
                ("paths", C.POINTER(Path)), ("path_count", u32),
                ("verbs", C.POINTER(u8)), ("verb_count", u32),
                ("points", C.POINTER(f32)), ("point_count", u32),
                ("paints", C.POINTER(Paint)), ("paint_count", u32),
                ("stops", C.POINTER(Stop)), ("stop_count", u32),
                ("dashes", C.POINTER(f32)), ("dash_count", u32),
                ("clips", C.POINTER(Clip)), ("clip_count", u32),
                ("masks", C.POINTER(Mask)), ("mask_count", u32),
                ("filter_refs", C.POINTER(u32)), ("filter_ref_count", u32),
                ("filters", C.POINTER(Filter)), ("filter_count", u32),
                ("prims", C.POINTER(Primitive)), ("prim_count", u32),
                ("merge_inputs", C.POINTER(i32)), ("merge_input_count", u32),
                ("images", C.c_void_p), ("image_count", u32),
                ("image_pixels", C.c_void_p), ("image_pixel_bytes", C.c_uint64)]


class ResvgTransform(C.Structure):
    _fields_ = [("a", f32), ("b", f32), ("c", f32), ("d", f32), ("e", f32), ("f", f32)]


class Tuning(C.Structure):
    _fields_ = [("band_rows", u32), ("pixels_per_thread", u32), ("reserved", u32)]


class TuningEntry(C.Structure):
    _fields_ = [("max_width", u32), ("max_draws", u32), ("band_rows", u32), ("reserved", u32)]


class Stats(C.Structure):
    _fields_ = [("draws", C.c_uint64), ("edges", C.c_uint64), ("crossings_capacity", C.c_uint64),
                ("work_items", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("raster_ms", f32),
                ("stroke_ms", f32), ("stroke_jobs", C.c_uint64)]


class SoftBatch(C.Structure):
    """rgpu_soft_batch (resvg_gpu.h): pointers are device pointers for the
    product and host pointers for the FP64 reference."""
    _fields_ = [("scenes", u32), ("width", u32), ("height", u32), ("paths_per_scene", u32),
                ("total_segments", u32), ("seg_offset", C.c_void_p), ("points", C.c_void_p),
                ("paint_kind", C.c_void_p), ("colors", C.c_void_p), ("stop_offsets", C.c_void_p),
                ("stop_colors", C.c_void_p), ("grad_line", C.c_void_p), ("sigma", C.c_void_p),
                ("opacity", C.c_void_p)]


class SoftGrads(C.Structure):
    _fields_ = [("points", C.c_void_p), ("colors", C.c_void_p), ("stop_offsets", C.c_void_p),
                ("stop_colors", C.c_void_p), ("sigma", C.c_void_p), ("opacity", C.c_void_p)]


# enums (rgpu_tree.h)
MOVE, LINE, QUAD, CUBIC, CLOSE = range(5)
NONZERO, EVENODD = 0, 1
PAINT_SOLID, PAINT_LINEAR, PAINT_RADIAL, PAINT_PATTERN, PAINT_IMAGE = 0, 1, 2, 3, 4
IMAGE_NEAREST, IMAGE_BILINEAR, IMAGE_BICUBIC = 0, 1, 2
SPREAD_PAD, SPREAD_REFLECT, SPREAD_REPEAT = 0, 1, 2
CAP_BUTT, CAP_ROUND, CAP_SQUARE = 0, 1, 2
JOIN_MITER, JOIN_MITER_CLIP, JOIN_ROUND, JOIN_BEVEL = 0, 1, 2, 3
NODE_GROUP, NODE_PATH = 0, 1
MASK_LUMINANCE, MASK_ALPHA = 0, 1
BLEND = {n: i for i, n in enumerate([
    "clear", "source", "destination", "source-over", "destination-over", "source-in", "destination-in",
    "source-out", "destination-out", "source-atop", "destination-atop", "xor", "plus", "modulate", "screen",
    "overlay", "darken", "lighten", "color-dodge", "color-burn", "hard-light", "soft-light", "difference",
    "exclusion", "multiply", "hue", "saturation", "color", "luminosity"])}
FE_BLUR, FE_COLOR_MATRIX, FE_MORPHOLOGY, FE_COMPOSITE, FE_CONVOLVE, FE_DIFFUSE, FE_SPECULAR, FE_FLOOD, \
    FE_OFFSET, FE_MERGE, FE_BLEND, FE_COMPONENT_TRANSFER, FE_DROP_SHADOW, FE_TURBULENCE, FE_TILE, \
    FE_DISPLACEMENT_MAP, FE_IMAGE = range(17)
IN_SOURCE_GRAPHIC, IN_SOURCE_ALPHA = -1, -2
CM_MATRIX, CM_SATURATE, CM_HUE_ROTATE, CM_LUM_TO_ALPHA = range(4)
OP_OVER, OP_IN, OP_OUT, OP_ATOP, OP_XOR, OP_ARITHMETIC = range(6)
EDGE_NONE, EDGE_DUPLICATE, EDGE_WRAP = range(3)
LIGHT_DISTANT, LIGHT_POINT, LIGHT_SPOT = range(3)
TF_IDENTITY, TF_TABLE, TF_DISCRETE, TF_LINEAR, TF_GAMMA = range(5)
TF_MAX_VALUES = 16
TURB_MAX_OCTAVES = 1024


def declare(lib: C.CDLL) -> C.CDLL:
    """Declares argument/return types of the product's C ABI."""
    P = C.c_void_p
    lib.rgpu_tree_new.restype = P
    lib.rgpu_tree_new.argtypes = [f32, f32]
    lib.rgpu_tree_free.argtypes = [P]
    lib.rgpu_tree_add_group.restype = i32
    lib.rgpu_tree_add_group.argtypes = [P, i32, C.POINTER(Group)]
    lib.rgpu_tree_add_path.restype = i32
    lib.rgpu_tree_add_path.argtypes = [P, i32, C.POINTER(Path), C.POINTER(u8), u32, C.POINTER(f32), u32,
                                       C.POINTER(f32), u32]
    lib.rgpu_tree_add_paint.restype = i32
    lib.rgpu_tree_add_paint.argtypes = [P, C.POINTER(Paint), C.POINTER(Stop), u32]
    lib.rgpu_tree_add_clip.restype = i32
    lib.rgpu_tree_add_clip.argtypes = [P, C.POINTER(Clip)]
    lib.rgpu_tree_add_mask.restype = i32
    lib.rgpu_tree_add_mask.argtypes = [P, C.POINTER(Mask)]
    lib.rgpu_tree_add_image.restype = i32
    lib.rgpu_tree_add_image.argtypes = [P, u32, u32, C.c_void_p]
    lib.rgpu_tree_add_filter.restype = i32
    lib.rgpu_tree_add_filter.argtypes = [P, C.POINTER(Filter), C.POINTER(Primitive), u32, C.POINTER(i32), u32]
    lib.rgpu_tree_set_node_id.restype = C.c_int
    lib.rgpu_tree_set_node_id.argtypes = [P, u32, u32, C.c_char_p]
    lib.rgpu_tree_find_node.restype = C.c_int
    lib.rgpu_tree_find_node.argtypes = [P, C.c_char_p, C.POINTER(u32), C.POINTER(u32)]
    lib.rgpu_tree_set_group_filters.restype = C.c_int
    lib.rgpu_tree_set_group_filters.argtypes = [P, i32, C.POINTER(u32), u32]
    lib.rgpu_tree_finalize.restype = C.c_int
    lib.rgpu_tree_finalize.argtypes = [P]
    lib.rgpu_tree_get_view.restype = C.POINTER(TreeView)
    lib.rgpu_tree_get_view.argtypes = [P]
    lib.rgpu_tree_generate.restype = P
    lib.rgpu_tree_generate.argtypes = [C.c_int, C.c_uint64, C.c_uint64, f32]
    return lib
