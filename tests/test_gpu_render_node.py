"""resvg_render_node on the GPU against the oracle (bit-exact): groups and
paths of generated scenes and of SVG fixtures, at the node's absolute layer
bounding box size (crates/resvg/src/lib.rs:55-70)."""
import numpy as np
import pytest

import resvg_gb300 as R

pytestmark = pytest.mark.gpu


def _check(tree, node_id, oracle_mod, ts=(1, 0, 0, 1, 0, 0)):
    b = R.node_abs_bbox(tree, node_id)
    if b is None:
        assert R.render_node(tree, node_id, ts, 8, 8) is None
        return
    w, h = max(1, int(round(b[2]))), max(1, int(round(b[3])))
    g = R.render_node(tree, node_id, ts, w, h)
    o = oracle_mod.render_node(tree.view(), node_id, ts, w, h)
    assert g is not None and o is not None
    n = int((g != o).any(axis=2).sum())
    assert n == 0, "%s: %d pixels differ" % (node_id, n)


@pytest.mark.parametrize("node_id", ["0", "p0", "p3", "p7"])
def test_generated_scene_nodes(gpu, oracle_mod, node_id):
    t = R.Tree.generate(0, seed=5, index=0, scale=0.05)
    _check(t, node_id, oracle_mod)


def test_clip_mask_groups(gpu, oracle_mod):
    t = R.Tree.generate(1, seed=3, index=0, scale=0.02)
    v = t.view().contents
    for g in range(min(v.group_count, 12)):
        _check(t, str(g), oracle_mod)


def test_unknown_ids(gpu):
    t = R.Tree.generate(0, seed=5, index=0, scale=0.05)
    assert R.render_node(t, "9999", (1, 0, 0, 1, 0, 0), 8, 8) is None
    assert R.render_node(t, "q1", (1, 0, 0, 1, 0, 0), 8, 8) is None
    assert R.render_node(t, "", (1, 0, 0, 1, 0, 0), 8, 8) is None
