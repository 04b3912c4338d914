"""Shared test helpers: scene construction and image comparison."""
from __future__ import annotations

import numpy as np

import resvg_gb300 as R
from resvg_gb300 import _abi as A


def diff_stats(a: np.ndarray, b: np.ndarray):
    """(number of differing pixels, max per-channel abs difference)."""
    d = np.abs(a.astype(np.int16) - b.astype(np.int16))
    return int((d.max(axis=-1) > 0).sum()), int(d.max()) if d.size else 0


def plain_group(**kw):
    g = A.Group()
    g.transform = A.Transform.identity()
    g.opacity = 1.0
    g.blend = A.BLEND["source-over"]
    g.clip_path = -1
    g.mask = -1
    for k, v in kw.items():
        setattr(g, k, v)
    return g


def base_path(**kw):
    p = A.Path()
    p.fill_paint = -1
    p.stroke_paint = -1
    p.fill_opacity = 1.0
    p.stroke_opacity = 1.0
    p.stroke_width = 1.0
    p.miter_limit = 4.0
    p.anti_alias = 1
    p.visible = 1
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def solid(tree, r, g, b):
    p = A.Paint()
    p.kind = A.PAINT_SOLID
    p.r, p.g, p.b = r, g, b
    p.transform = A.Transform.identity()
    return tree.add_paint(p)


def rect_path(x, y, w, h):
    return [A.MOVE, A.LINE, A.LINE, A.LINE, A.CLOSE], [x, y, x + w, y, x + w, y + h, x, y + h]
