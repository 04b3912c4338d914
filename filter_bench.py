"""Device time of each filter primitive on one image, through rgpu_filter_apply.

    python filter_bench.py [--size 2048] [--reps 20]

Every case is one filter whose region is the whole image (identity layer
transform, sRGB interpolation so no colour-space passes are added) applied to
a seeded random premultiplied image.  The time is CUDA events around `reps`
back-to-back applications on one stream, after warm-up; the image (16.8 MB at
2048^2) stays in L2 between applications, so these are warm figures.  The
bytes column is the algorithmic traffic of the primitive's own kernels: 4 B
per pixel per image read or written by each pass (a box blur is 10 passes),
not counting the job's input and result copies.  `primitive_cases` is shared
with the GPU parity test of rgpu_filter_apply.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from resvg_gb300 import _abi as A  # noqa: E402

_IN = A.IN_SOURCE_GRAPHIC


def _prim(w, h, kind, in1=_IN, in2=_IN, i=(), f=(), sub=None):
    p = A.Primitive()
    p.kind = kind
    p.x, p.y, p.w, p.h = sub if sub is not None else (0.0, 0.0, float(w), float(h))
    p.linear_rgb = 0
    p.in1, p.in2 = in1, in2
    for k, v in enumerate(i):
        p.i[k] = int(v)
    for k, v in enumerate(f):
        p.f[k] = float(v)
    return p


def primitive_cases(w, h):
    """(name, primitives, merge inputs, algorithmic bytes per pixel)."""
    P = lambda *a, **k: _prim(w, h, *a, **k)  # noqa: E731
    tf = [A.TF_TABLE, A.TF_GAMMA, A.TF_LINEAR, A.TF_DISCRETE, 4, 0, 3, 3]
    ct = P(A.FE_COMPONENT_TRANSFER, i=tf)
    for k, v in enumerate([1.0, 0.2, 0.8, 0.0]):
        ct.f[k] = v
    ct.f[16], ct.f[17], ct.f[18] = 1.1, 0.6, -0.05
    ct.f[32], ct.f[33] = 1.4, -0.2
    ct.f[48], ct.f[49], ct.f[50] = 0.0, 0.5, 1.0
    conv = [1, 2, 1, 0, 0, 0, -1, -2, -1]
    return [
        ("blur, box sigma 10", [P(A.FE_BLUR, f=(10, 10))], (), 10 * 8),
        ("blur, IIR sigma 1.5", [P(A.FE_BLUR, f=(1.5, 1.5))], (), 8),
        ("colour matrix, saturate 0.4", [P(A.FE_COLOR_MATRIX, i=(A.CM_SATURATE,), f=(0.4,))], (), 8),
        ("morphology, dilate r 3", [P(A.FE_MORPHOLOGY, i=(1,), f=(3, 3))], (), 8),
        ("composite, arithmetic", [P(A.FE_COMPOSITE, i=(A.OP_ARITHMETIC,), f=(0.5, 0.3, 0.4, -0.1))], (), 12),
        ("component transfer, 4 functions", [ct], (), 8),
        ("drop shadow, sigma 4", [P(A.FE_DROP_SHADOW, i=(30, 60, 200), f=(4, 4, 6, 5, 0.7))], (), 10 * 8 + 12),
        ("turbulence, 4 octaves", [P(A.FE_TURBULENCE, i=(4, 3, 0, 0), f=(0.02, 0.03))], (), 4),
        ("tile", [P(A.FE_OFFSET, f=(5, 5), sub=(40.0, 40.0, 64.0, 48.0)), P(A.FE_TILE, in1=0)], (), 8),
        ("displacement map", [P(A.FE_DISPLACEMENT_MAP, i=(0, 1), f=(12,))], (), 12),
        ("convolve 3x3", [P(A.FE_CONVOLVE, i=(3, 3, 1, 1, A.EDGE_DUPLICATE, 0), f=[1.0, 0.0] + conv)], (), 8),
        ("diffuse lighting, distant", [P(A.FE_DIFFUSE, i=(A.LIGHT_DISTANT, 255, 255, 255),
                                         f=(3, 1, 1, 0, 45, 45))], (), 8),
        ("flood", [P(A.FE_FLOOD, i=(20, 120, 60), f=(0.8,))], (), 4),
        ("offset", [P(A.FE_OFFSET, f=(7, -3))], (), 8),
        ("merge, 2 inputs", [P(A.FE_MERGE, i=(0, 2))], (_IN, A.IN_SOURCE_ALPHA), 4 + 2 * 8),
        ("blend, multiply", [P(A.FE_BLEND, i=(A.BLEND["multiply"],))], (), 12),
    ]


def measured_hbm():
    """(GB/s, label): the measured copy bandwidth when the peaks file is there."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        for k in ("hbm_gbs", "hbm_GBps", "hbm"):
            if k in d and isinstance(d[k], (int, float)):
                return float(d[k]), "measured"
    except (OSError, ValueError):
        pass
    return 6800.0, "fallback"


def main():
    import torch
    import resvg_gb300 as R
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args()
    w = h = a.size
    R.init(0)
    dev = torch.device("cuda", 0)
    g = torch.Generator().manual_seed(7)
    base = torch.randint(0, 256, (h, w, 4), dtype=torch.uint8, generator=g)
    base[..., 3] = torch.where(base[..., 3] > 100, 255, base[..., 3])
    base[..., :3] = torch.minimum(base[..., :3], base[..., 3:4])
    base = base.to(dev)
    img = torch.empty_like(base)
    stream = torch.cuda.current_stream().cuda_stream
    peak, label = measured_hbm()
    filt = A.Filter()
    filt.x, filt.y, filt.w, filt.h = 0.0, 0.0, float(w), float(h)
    print("%-34s %10s %10s %8s" % ("primitive (%dx%d)" % (w, h), "us", "GB/s", "of HBM"))
    for name, prims, merge, bpp in primitive_cases(w, h):
        img.copy_(base)
        for _ in range(3):
            R.filter_apply(img, filt, prims, merge, stream=stream)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(a.reps):
            R.filter_apply(img, filt, prims, merge, stream=stream)
        t1.record()
        torch.cuda.synchronize()
        us = t0.elapsed_time(t1) * 1e3 / a.reps
        gbs = bpp * w * h / us / 1e3
        print("%-34s %10.1f %10.1f %7.1f%%" % (name, us, gbs, 100.0 * gbs / peak), flush=True)
    # the IIR blur in its FP32 chunked-scan mode (rgpu_set_iir_precision(1))
    iir = [c for c in primitive_cases(w, h) if c[0].startswith("blur, IIR")][0]
    R.set_iir_precision(1)
    try:
        img.copy_(base)
        for _ in range(3):
            R.filter_apply(img, filt, iir[1], iir[2], stream=stream)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(a.reps):
            R.filter_apply(img, filt, iir[1], iir[2], stream=stream)
        t1.record()
        torch.cuda.synchronize()
    finally:
        R.set_iir_precision(0)
    us = t0.elapsed_time(t1) * 1e3 / a.reps
    gbs = iir[3] * w * h / us / 1e3
    print("%-34s %10.1f %10.1f %7.1f%%" % (iir[0] + ", FP32 scan", us, gbs, 100.0 * gbs / peak), flush=True)
    print("HBM peak %.0f GB/s (%s); times include the job's input and result copies" % (peak, label))


if __name__ == "__main__":
    main()
