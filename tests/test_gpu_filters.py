"""Filter kernels on the GPU vs the CPU restatement of resvg's filter module.

Integer / deterministic-f32 paths (box blur, morphology, colour-space LUTs,
colour matrix, arithmetic composite) must be bit-exact.  The IIR blur runs the
same f64 recursions in the same order and is checked bit-exact too; the
spec tolerance for it would be 1/255.
"""
import numpy as np
import pytest

import resvg_gb300 as R
from tests.helpers import diff_stats

pytestmark = pytest.mark.gpu


def _premul_image(h, w, seed):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    # blobs of transparency and opaque areas, as rendered content has
    img[rng.random((h, w)) < 0.3, 3] = 0
    img[rng.random((h, w)) < 0.3, 3] = 255
    a = img[..., 3:4].astype(np.uint16)
    img[..., :3] = (img[..., :3].astype(np.uint16) * a // 255).astype(np.uint8)
    return img


def _on_gpu(fn, img, *args):
    import torch
    t = torch.from_numpy(img.copy()).cuda()
    fn(t, *args)
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("shape", [(1, 1), (7, 300), (300, 7), (257, 513)])
@pytest.mark.parametrize("sigma", [(2.0, 2.0), (5.5, 0.0), (0.0, 9.0), (20.0, 3.0)])
def test_box_blur_exact(gpu, oracle_mod, shape, sigma):
    img = _premul_image(*shape, seed=1)
    g = _on_gpu(R.box_blur, img, *sigma)
    o = oracle_mod.box_blur(img, *sigma)
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("sigma", [(0.5, 0.5), (1.7, 0.3), (0.0, 1.9)])
def test_iir_blur(gpu, oracle_mod, sigma):
    img = _premul_image(133, 211, seed=2)
    g = _on_gpu(R.iir_blur, img, *sigma)
    o = oracle_mod.iir_blur(img, *sigma)
    n, mx = diff_stats(g, o)
    assert mx <= 1, (n, mx)


@pytest.mark.parametrize("shape", [(1, 1), (7, 300), (300, 7), (257, 513), (2048, 96), (40, 4097)])
@pytest.mark.parametrize("sigma", [(0.5, 0.5), (1.7, 0.3), (0.0, 1.9), (1.9, 0.0)])
def test_iir_blur_fp32_scan_mode(gpu, oracle_mod, shape, sigma):
    """The FP32 chunked-scan IIR (rgpu_set_iir_precision(1)) against the f64
    reference restatement: at most 1 per channel (the benchmark spec's 1/255 for the
    IIR blur), differing pixels under 2% of the image; lines longer than 4096
    fall back to the f64 recursions and stay bit-exact."""
    img = _premul_image(*shape, seed=5)
    R.set_iir_precision(1)
    try:
        g = _on_gpu(R.iir_blur, img, *sigma)
    finally:
        R.set_iir_precision(0)
    o = oracle_mod.iir_blur(img, *sigma)
    n, mx = diff_stats(g, o)
    assert mx <= 1, (n, mx)
    assert n <= max(2, 0.02 * shape[0] * shape[1]), (n, mx)
    if shape[1] > 4096:
        assert n == 0


@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("r", [(1.0, 1.0), (2.5, 4.0), (5.0, 5.0), (0.3, 3.0)])
def test_morphology_exact(gpu, oracle_mod, op, r):
    img = _premul_image(97, 151, seed=3)
    g = _on_gpu(R.morphology, img, op, *r)
    o = oracle_mod.morphology(img, op, *r)
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("to_linear", [True, False])
def test_color_space_exact(gpu, oracle_mod, to_linear):
    img = _premul_image(64, 64, seed=4)
    g = _on_gpu(R.color_space, img, to_linear)
    o = oracle_mod.to_linear(img) if to_linear else oracle_mod.to_srgb(img)
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_config2_filter_chain(gpu, oracle_mod, seed):
    """The blur -> saturate -> morphology -> arithmetic chain in linearRGB on a
    2048x2048 canvas (fewer paths than the benchmark scene to keep the CPU
    oracle fast)."""
    t = R.Tree.generate(2, seed=seed, index=0, scale=0.05)
    w = h = 2048
    g = R.render(t, (1, 0, 0, 1, 0, 0), w, h)
    o = oracle_mod.render(t.view(), (1, 0, 0, 1, 0, 0), w, h)
    n, mx = diff_stats(g, o)
    assert mx <= 1, "%d px differ, max %d" % (n, mx)


def _all_pairs():
    """256 x 256 pixels: row = alpha, column = channel value (premultiplied or
    not), so every (alpha, value) pair meets the demultiply / multiply code."""
    c = np.arange(256, dtype=np.uint8)
    img = np.zeros((256, 256, 4), dtype=np.uint8)
    img[..., 0] = c[None, :]
    img[..., 1] = 255 - c[None, :]
    img[..., 2] = (c[None, :].astype(np.uint16) * 7 % 256).astype(np.uint8)
    img[..., 3] = c[:, None]
    return img


@pytest.mark.parametrize("to_linear", [True, False])
def test_color_space_every_alpha_value_pair(gpu, oracle_mod, to_linear):
    img = _all_pairs()
    g = _on_gpu(R.color_space, img, to_linear)
    o = oracle_mod.to_linear(img) if to_linear else oracle_mod.to_srgb(img)
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("kind", ["saturate", "transfer"])
def test_demultiply_multiply_every_pair(gpu, oracle_mod, kind):
    # colour matrix and component transfer both demultiply, map and multiply
    from resvg_gb300 import _abi as A
    img = _all_pairs()
    p = A.Primitive()
    p.x, p.y, p.w, p.h = 0.0, 0.0, 256.0, 256.0
    p.in1 = p.in2 = A.IN_SOURCE_GRAPHIC
    if kind == "saturate":
        p.kind, p.i[0], p.f[0] = A.FE_COLOR_MATRIX, A.CM_SATURATE, 0.7
    else:
        p.kind = A.FE_COMPONENT_TRANSFER
        p.i[0], p.i[4], p.f[0], p.f[1] = A.TF_TABLE, 2, 0.1, 0.9
        p.i[3], p.f[48], p.f[49] = A.TF_LINEAR, 1.0, 0.0
    f = A.Filter()
    f.x, f.y, f.w, f.h = 0.0, 0.0, 256.0, 256.0
    o = oracle_mod.filter_apply(img, f, [p])
    g = _on_gpu(lambda t: R.filter_apply(t, f, [p]), img)
    assert diff_stats(g, o) == (0, 0)
