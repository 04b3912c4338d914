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
from resvg_gb300.filter_bench import primitive_cases
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
