"""rgpu_filter_apply (filter::apply on a device pixmap) vs the oracle.

Each case is one filter over the whole image (the cases the filter benchmark
times) on a seeded premultiplied image, under an identity and a scaling layer
transform.  Every primitive is bit-exact except lighting, whose powf / sqrt may
differ from the host libm in the last ulp: 1/255 per channel there.
"""
import numpy as np
import pytest

import oracle
import resvg_gb300 as R
from resvg_gb300 import _abi as A
from filter_bench import primitive_cases
from tests.helpers import diff_stats

pytestmark = pytest.mark.gpu

W, H = 320, 256
CASES = primitive_cases(W, H)


def _image(seed):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    img[..., 3] = np.where(img[..., 3] > 100, 255, img[..., 3])
    img[..., :3] = np.minimum(img[..., :3], img[..., 3:4])
    return img


@pytest.mark.parametrize("ts", [(1, 0, 0, 1, 0, 0), (1.5, 0, 0, 1.25, 0, 0)])
@pytest.mark.parametrize("k", range(len(CASES)))
def test_filter_apply_matches_oracle(gpu, k, ts):
    import torch
    name, prims, merge, _ = CASES[k]
    filt = A.Filter()
    filt.x, filt.y, filt.w, filt.h = 0.0, 0.0, W / ts[0], H / ts[3]
    for p in prims:
        if p.w == W and p.h == H:
            p.w, p.h = filt.w, filt.h
    img = _image(k)
    ref = oracle.filter_apply(img, filt, prims, merge, ts)
    t = torch.from_numpy(img).cuda()
    R.filter_apply(t, filt, prims, merge, ts)
    got = t.cpu().numpy()
    n, worst = diff_stats(got, ref)
    if "lighting" in name:
        assert worst <= 1, name
    else:
        assert (n, worst) == (0, 0), name


# A filter region inside a larger layer (the layer of a group with several
# filters is the union of their regions): primitives that make region-sized
# images make them at the layer origin (crates/resvg/src/filter/mod.rs, e.g.
# apply_flood / apply_composite / apply_merge: Pixmap::try_create(region.w,
# region.h), inputs drawn at (0, 0)), the last result is drawn at the origin of
# the cleared layer (apply_to_canvas, :1100-1114).
SUB_REGION = (40.0, 30.0, 200.0, 150.0)


def _sub_filter():
    filt = A.Filter()
    filt.x, filt.y, filt.w, filt.h = SUB_REGION
    return filt


def _in_region(prims):
    for p in prims:
        if p.w == W and p.h == H:
            p.x, p.y, p.w, p.h = SUB_REGION
    return prims


def _run_both(filt, prims, merge, ts, seed):
    import torch
    img = _image(seed)
    ref = oracle.filter_apply(img, filt, prims, merge, ts)
    t = torch.from_numpy(img).cuda()
    R.filter_apply(t, filt, prims, merge, ts)
    return t.cpu().numpy(), ref


@pytest.mark.parametrize("k", range(len(CASES)))
def test_filter_region_smaller_than_layer(gpu, k):
    name, prims, merge, _ = CASES[k]
    got, ref = _run_both(_sub_filter(), _in_region(prims), merge, (1, 0, 0, 1, 0, 0), 100 + k)
    n, worst = diff_stats(got, ref)
    if "lighting" in name or "displacement" in name:
        # a layer-sized input under a smaller region: the reference indexes
        # out of range here, both renderers fail the filter and clear the layer
        assert not got.any() and not ref.any(), name
        assert "layer cleared" in R.last_warning(), name
    else:
        assert (n, worst) == (0, 0), "%s: %d px differ (max %d)" % (name, n, worst)


def _P(kind, in1=A.IN_SOURCE_GRAPHIC, in2=A.IN_SOURCE_GRAPHIC, i=(), f=(), sub=SUB_REGION):
    p = A.Primitive()
    p.kind = kind
    p.x, p.y, p.w, p.h = sub
    p.in1, p.in2 = in1, in2
    for k, v in enumerate(i):
        p.i[k] = int(v)
    for k, v in enumerate(f):
        p.f[k] = float(v)
    return p


CHAINS = [
    # region-sized results feeding input-sized primitives and each other
    ("flood, blur, composite over the source",
     [_P(A.FE_FLOOD, i=(200, 40, 10), f=(0.7,)), _P(A.FE_BLUR, in1=0, f=(3, 3)),
      _P(A.FE_COMPOSITE, in1=1, in2=A.IN_SOURCE_GRAPHIC, i=(A.OP_IN,))], ()),
    ("merge of source and flood, then colour matrix",
     [_P(A.FE_FLOOD, i=(10, 90, 250), f=(0.5,)), _P(A.FE_MERGE, i=(0, 2)),
      _P(A.FE_COLOR_MATRIX, in1=1, i=(A.CM_SATURATE,), f=(0.3,))], (A.IN_SOURCE_GRAPHIC, 0)),
    ("turbulence, arithmetic with the source",
     [_P(A.FE_TURBULENCE, i=(2, 5, 0, 1), f=(0.05, 0.04)),
      _P(A.FE_COMPOSITE, in1=0, in2=A.IN_SOURCE_GRAPHIC, i=(A.OP_ARITHMETIC,), f=(0.3, 0.5, 0.5, 0.0))], ()),
    ("flood lit by a point light (region-sized input)",
     [_P(A.FE_FLOOD, i=(255, 255, 255), f=(0.6,)),
      _P(A.FE_DIFFUSE, in1=0, i=(A.LIGHT_POINT, 250, 200, 100), f=(2, 1, 1, 0, 80, 60, 40))], ()),
    ("subregion crop of a blend",
     [_P(A.FE_FLOOD, i=(0, 200, 0), f=(1.0,)),
      _P(A.FE_BLEND, in1=A.IN_SOURCE_GRAPHIC, in2=0, i=(A.BLEND["screen"],), sub=(60.0, 50.0, 90.0, 70.0))], ()),
    ("offset of the source, tiled over the region",
     [_P(A.FE_OFFSET, f=(4, 6), sub=(70.0, 60.0, 40.0, 30.0)), _P(A.FE_TILE, in1=0)], ()),
]


@pytest.mark.parametrize("ts", [(1, 0, 0, 1, 0, 0), (1.25, 0, 0, 1.25, -20, -10)])
@pytest.mark.parametrize("k", range(len(CHAINS)))
def test_mixed_size_chains_under_a_smaller_region(gpu, k, ts):
    name, prims, merge = CHAINS[k]
    got, ref = _run_both(_sub_filter(), prims, merge, ts, 200 + k)
    n, worst = diff_stats(got, ref)
    if "lit" in name:
        assert worst <= 1, name  # powf / sqrt against the host libm
    else:
        assert (n, worst) == (0, 0), "%s: %d px differ (max %d)" % (name, n, worst)


def test_invalid_region_clears_layer_and_succeeds(gpu):
    """filter::apply clears the layer on an invalid region and logs a warning
    (mod.rs:343-354); the call itself does not fail."""
    filt = A.Filter()
    filt.x, filt.y, filt.w, filt.h = 5000.0, 5000.0, 10.0, 10.0  # entirely outside the layer
    got, ref = _run_both(filt, [_P(A.FE_FLOOD, i=(1, 2, 3), f=(1.0,), sub=(5000.0, 5000.0, 10.0, 10.0))], (),
                         (1, 0, 0, 1, 0, 0), 7)
    assert not got.any() and not ref.any()
    assert "invalid region" in R.last_warning()
