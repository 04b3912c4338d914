"""resvg_render_node on the GPU, called through the C ABI with SVG ids.

The C API resolves `id` with usvg's Tree::node_by_id (crates/c-api/lib.rs:931)
and renders the node at its absolute layer bounding box
(crates/resvg/src/lib.rs:55-70).  Here the ids are SVG ids set on the tree
(rgpu_tree_set_node_id, or by the SVG front end), and the output is compared
bit-exactly with the oracle's render of the same node, and, for resvg's own
render_node golden cases (crates/resvg/tests/integration/extra.rs), with the
golden image under the suite's rule.
"""
import os
import zlib

import numpy as np
import pytest

import resvg_gb300 as R
from resvg_gb300 import _abi as A
from tests import golden_fixtures as G

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _oracle_id(kind, index):
    return ("p%d" if kind == A.NODE_PATH else "%d") % index


def _check(tree, svg_id, oracle_mod, ts=(1, 0, 0, 1, 0, 0)):
    node = tree.find_node(svg_id)
    assert node is not None, svg_id
    b = R.node_abs_bbox(tree, svg_id)
    if b is None:
        assert R.render_node(tree, svg_id, ts, 8, 8) is None
        return
    w, h = max(1, int(round(b[2]))), max(1, int(round(b[3])))
    g = R.render_node(tree, svg_id, ts, w, h)
    o = oracle_mod.render_node(tree.view(), _oracle_id(*node), ts, w, h)
    assert g is not None and o is not None
    n = int((g != o).any(axis=2).sum())
    assert n == 0, "%s: %d pixels differ" % (svg_id, n)


def _named(tree):
    """Every group gets id "group-<n>", every path "shape-<n>"."""
    v = tree.view().contents
    for g in range(v.group_count):
        tree.set_node_id(A.NODE_GROUP, g, "group-%d" % g)
    for p in range(v.path_count):
        tree.set_node_id(A.NODE_PATH, p, "shape-%d" % p)
    return tree


@pytest.mark.parametrize("svg_id", ["shape-0", "shape-3", "shape-7"])
def test_generated_scene_nodes(gpu, oracle_mod, svg_id):
    t = _named(R.Tree.generate(0, seed=5, index=0, scale=0.05))
    _check(t, svg_id, oracle_mod)


def test_clip_mask_groups(gpu, oracle_mod):
    """Groups with clips and masks; detached groups (clip and mask content)
    are not below the root, so node_by_id does not find them."""
    t = _named(R.Tree.generate(1, seed=3, index=0, scale=0.02))
    v = t.view().contents
    below_root = set()
    stack = [0]
    while stack:
        g = stack.pop()
        gr = v.groups[g]
        for k in range(gr.child_count):
            n = v.children[gr.child_offset + k]
            if n.kind == A.NODE_GROUP:
                below_root.add(n.index)
                stack.append(n.index)
    checked = 0
    for g in range(min(v.group_count, 16)):
        if g in below_root:
            _check(t, "group-%d" % g, oracle_mod)
            checked += 1
        else:
            assert t.find_node("group-%d" % g) is None
    assert checked >= 2


def test_unknown_and_empty_ids(gpu):
    t = _named(R.Tree.generate(0, seed=5, index=0, scale=0.05))
    for bad in ("9999", "p1", "shape-99999", "", "group-0"):  # the root itself is not a searched node
        assert R.render_node(t, bad, (1, 0, 0, 1, 0, 0), 8, 8) is None, bad


def _extra_node_fixtures():
    d = np.load(os.path.join(HERE, "golden", "extra_nodes.npz"))
    out = []
    for i, name in enumerate(d["names"]):
        text = zlib.decompress(d["svg_%d" % i].tobytes()).decode("utf-8")
        shape = tuple(int(v) for v in d["shape_%d" % i])
        img = np.frombuffer(zlib.decompress(d["png_%d" % i].tobytes()), dtype=np.uint8).reshape(shape)
        out.append((str(name), text, str(d["id_%d" % i]), img))
    return out


EXTRA = _extra_node_fixtures()


@pytest.mark.parametrize("idx", range(len(EXTRA)), ids=[e[0] for e in EXTRA])
def test_resvg_render_node_golden_by_svg_id(gpu, oracle_mod, idx):
    """crates/resvg/tests/integration/main.rs:90-95: the pixmap is the node's
    absolute layer bbox size, the transform identity, the id an SVG id."""
    from resvg_gb300 import png, svg
    name, text, svg_id, expected = EXTRA[idx]
    tree = svg.load_svg(text)
    b = R.node_abs_bbox(tree, svg_id)
    assert b is not None, name
    rnd = lambda v: int(np.floor(v + 0.5))  # noqa: E731  (IntSize from a positive f32 size)
    w, h = max(1, rnd(b[2])), max(1, rnd(b[3]))
    got = R.render_node(tree, svg_id, (1, 0, 0, 1, 0, 0), w, h)
    assert got is not None, name
    assert G.pixel_diff(expected, png.demultiply(got)) == 0, name
    ref = oracle_mod.render_node(tree.view(), _oracle_id(*tree.find_node(svg_id)), (1, 0, 0, 1, 0, 0), w, h)
    assert int((got != ref).any(axis=2).sum()) == 0, name
