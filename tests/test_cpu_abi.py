"""The C-ABI library loads and exports every function include/*.h declares
(no GPU needed; nothing is called)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("resvg_gpu.h", "rgpu_tree.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^[ \t]*(?!typedef)[A-Za-z_][\w \t\*]*?\b((?:rgpu|resvg)_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_drop_in():
    names = declared_functions()
    assert "resvg_render" in names and "resvg_render_node" in names
    assert len(names) > 20


def test_library_exports_every_declared_function(native):
    lib = C.CDLL(native.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_oracle_is_not_linked_into_the_product(native):
    """The product library must not contain the oracle's entry points."""
    lib = C.CDLL(native.LIB_PATH)
    for n in ("oracle_render", "oracle_render_parallel", "oracle_box_blur"):
        assert not hasattr(lib, n), n
