"""Anti-aliased hairline strokes (device width <= 1 px) on the GPU against the
oracle, bit-exact: butt/round/square caps, lines/quads/cubics, rotation and
down-scaling, solid and gradient paints, lines leaving the canvas, lines
longer than 511 px (split), and dashes."""
import numpy as np
import pytest

import resvg_gb300 as R
from resvg_gb300 import _abi as A
from tests.helpers import base_path, plain_group, solid

pytestmark = pytest.mark.gpu


def _stroke(t, parent, verbs, pts, width, cap=0, join=0, paint=None, opacity=1.0, dashes=()):
    p = base_path(fill_paint=-1)
    p.stroke_paint = paint if paint is not None else solid(t, 20, 40, 200)
    p.stroke_opacity = opacity
    p.stroke_width = width
    p.line_cap = cap
    p.line_join = join
    p.miter_limit = 4.0
    t.add_path(parent, p, verbs, pts, dashes)


def _scene(seed, size=160):
    rng = np.random.default_rng(seed)
    t = R.Tree(size, size)
    root = t.add_group(-1, plain_group())
    g = A.Paint()
    g.kind = A.PAINT_LINEAR
    g.x1, g.y1, g.x2, g.y2 = 0, 0, size, size
    g.transform = A.Transform.identity()
    stops = []
    for o, c in ((0.0, (255, 0, 0)), (1.0, (0, 0, 255))):
        s = A.Stop()
        s.offset = o
        s.r, s.g, s.b = c
        s.opacity = 0.8
        stops.append(s)
    grad = t.add_paint(g, stops)
    for i in range(24):
        kind = i % 3
        pts = rng.uniform(-0.2 * size, 1.2 * size, size=8).tolist()
        if kind == 0:
            verbs, pts = [A.MOVE, A.LINE, A.LINE], pts[:6]
        elif kind == 1:
            verbs, pts = [A.MOVE, A.QUAD], pts[:6]
        else:
            verbs = [A.MOVE, A.CUBIC]
        _stroke(t, root, verbs, pts, width=float(rng.choice([0.25, 0.6, 1.0])), cap=i % 3,
                paint=grad if i % 4 == 0 else None, opacity=float(rng.uniform(0.4, 1.0)),
                dashes=(5.0, 3.0) if i % 5 == 0 else ())
    # closed contour and a long line that is split (> 511 px)
    _stroke(t, root, [A.MOVE, A.LINE, A.LINE, A.CLOSE], [10, 10, 150, 30, 40, 140], width=0.8, cap=1)
    _stroke(t, root, [A.MOVE, A.LINE], [-700, 5, size + 700, size - 5], width=1.0)
    t.finalize()
    return t


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("ts", [(1, 0, 0, 1, 0, 0), (0.5, 0, 0, 0.5, 20, 10), (0.7, 0.5, -0.5, 0.7, 60, -10)])
def test_hairlines_exact(gpu, oracle_mod, seed, ts):
    t = _scene(seed)
    w, h = 160, 160
    g = R.render(t, ts, w, h)
    o = oracle_mod.render(t.view(), ts, w, h)
    n = int((g != o).any(axis=2).sum())
    assert n == 0, "%d pixels differ" % n
    assert int(g[..., 3].astype(np.int64).sum()) > 0


def test_hairline_under_layers(gpu, oracle_mod):
    """Hairlines inside an opacity group, a clip and a mask, at a layer offset."""
    t = R.Tree.generate(1, seed=9, index=0, scale=0.05)
    g = R.render(t, (0.3, 0, 0, 0.3, 0, 0), 307, 307)
    o = oracle_mod.render(t.view(), (0.3, 0, 0, 0.3, 0, 0), 307, 307)
    n = int((g != o).any(axis=2).sum())
    assert n == 0, "%d pixels differ" % n
