"""Loader for tests/golden/fixtures.npz (written by tests/golden/pin_oracle.py).

Each fixture is one test of resvg's integration suite that the oracle
reproduces with zero differing pixels: its SVG text and its golden image
(demultiplied RGBA8), both zlib-compressed.
"""
import math
import os
import zlib

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
IMAGE_SIZE = 300


def load():
    d = np.load(os.path.join(HERE, "fixtures.npz"))
    out = []
    for i, name in enumerate(d["names"]):
        text = zlib.decompress(d["svg_%d" % i].tobytes()).decode("utf-8")
        shape = tuple(int(v) for v in d["shape_%d" % i])
        img = np.frombuffer(zlib.decompress(d["png_%d" % i].tobytes()), dtype=np.uint8).reshape(shape)
        out.append((str(name), text, img))
    return out


def render_size(tw, th):
    """tiny-skia Size::to_int_size then IntSize::scale_to_width(300)."""
    def rnd(v):
        return math.floor(v + 0.5) if v >= 0 else -math.floor(-v + 0.5)
    iw, ih = max(1, int(rnd(tw))), max(1, int(rnd(th)))
    return IMAGE_SIZE, int(math.ceil(np.float32(IMAGE_SIZE) * np.float32(ih) / np.float32(iw)))


def render_transform(tree):
    tw, th = tree.size
    w, h = render_size(tw, th)
    return w, h, (float(np.float32(w) / np.float32(tw)), 0.0, 0.0, float(np.float32(h) / np.float32(th)), 0.0, 0.0)


def pixel_diff(expected, actual):
    """resvg's suite rule (tests/integration/main.rs:148-220): a pixel differs
    when any channel differs by more than 1, unless transparent in both."""
    if expected.shape != actual.shape:
        return expected.shape[0] * expected.shape[1]
    both_clear = (expected[..., 3] == 0) & (actual[..., 3] == 0)
    d = np.abs(expected.astype(np.int16) - actual.astype(np.int16)).max(axis=2) > 1
    return int((d & ~both_clear).sum())
