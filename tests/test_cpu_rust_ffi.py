"""The Rust FFI crate (resvg_gb300/rust) against the C headers and the library.

No Rust toolchain is needed: the crate's `extern "C"` declarations must name
functions that include/*.h declares and the library exports, and its
`#[repr(C)]` structs must list the same fields in the same order as the
header structs (mirrored by resvg_gb300/_abi.py).
"""
import ctypes as C
import os
import re

from resvg_gb300 import _abi as A
from tests.test_cpu_abi import declared_functions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_RS = os.path.join(ROOT, "resvg_gb300", "rust", "src", "lib.rs")


def _rust_externs():
    text = open(LIB_RS).read()
    block = text[text.index('extern "C" {'):]
    block = block[:block.index("\n}\n")]
    return re.findall(r"pub fn (\w+)\(", block)


def _rust_struct_fields(name):
    text = open(LIB_RS).read()
    m = re.search(r"pub struct %s \{(.*?)\n\}" % name, text, flags=re.S)
    assert m, name
    return re.findall(r"pub (\w+):", m.group(1))


def test_externs_are_declared_and_exported(native):
    names = _rust_externs()
    assert "resvg_render" in names and "resvg_render_node" in names and "rgpu_tree_set_node_id" in names
    declared = set(declared_functions())
    lib = C.CDLL(native.LIB_PATH)
    assert [n for n in names if n not in declared] == []
    assert [n for n in names if not hasattr(lib, n)] == []


def test_repr_c_structs_match_the_header():
    pairs = {"rgpu_transform": A.Transform, "rgpu_stop": A.Stop, "rgpu_paint": A.Paint, "rgpu_path": A.Path,
             "rgpu_node": A.Node, "rgpu_group": A.Group, "rgpu_clip": A.Clip, "rgpu_mask": A.Mask,
             "rgpu_primitive": A.Primitive, "rgpu_filter": A.Filter, "resvg_transform": A.ResvgTransform,
             "rgpu_tuning": A.Tuning, "rgpu_stats": A.Stats}
    import resvg_gb300 as R
    pairs["rgpu_stroke_desc"] = R.StrokeDesc
    for rust, cstruct in pairs.items():
        assert _rust_struct_fields(rust) == [f[0] for f in cstruct._fields_], rust
