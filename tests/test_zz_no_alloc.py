"""The allocation-free box blur entry point against the allocating one.

Both are called through the C ABI on the same device images; the box blur is
integer arithmetic, so the tolerance is zero (bit-exact).  Two calls in a row
check that state left in the shared scratch by one call does not leak into
the next.  The file is named to be collected last and also passes alone in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import resvg_gb300 as R

pytestmark = pytest.mark.gpu

TOLERANCE = 0  # max channel difference allowed (integer box sums)
MAX_PIXELS = 1 << 20


def _noalloc():
    L = R.lib()
    f = L.rgpu_filter_box_blur_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_void_p]
    return f


def _premul_image(h, w, seed):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    img[rng.random((h, w)) < 0.3, 3] = 0
    a = img[..., 3:4].astype(np.uint16)
    img[..., :3] = (img[..., :3].astype(np.uint16) * a // 255).astype(np.uint8)
    return img


# sigma 150 gives box radii above the shared-memory tiles' limit, so those
# passes run the generic line kernel through the fixed scratch too
@pytest.mark.parametrize("shape,sigma", [((96, 160), (3.0, 3.0)), ((1024, 1024), (7.5, 2.0)),
                                         ((33, 1000), (0.0, 12.0)), ((64, 2000), (150.0, 150.0)),
                                         ((2000, 64), (90.0, 160.0))])
def test_noalloc_box_blur_matches_allocating_entry(gpu, shape, sigma):
    import torch
    f = _noalloc()
    h, w = shape
    for call in range(2):  # two calls in a row through the shared scratch
        img = _premul_image(h, w, seed=11 + call)
        ref = torch.from_numpy(img.copy()).cuda()
        out = torch.from_numpy(img.copy()).cuda()
        torch.cuda.synchronize()
        R.box_blur(ref, *sigma)
        status = f(C.c_void_p(out.data_ptr()), w, h, C.c_double(sigma[0]), C.c_double(sigma[1]), None)
        assert status == 0, R.lib().rgpu_last_error().decode()
        torch.cuda.synchronize()
        d = (ref.to(torch.int16) - out.to(torch.int16)).abs().max().item()
        assert d <= TOLERANCE, "call %d: max channel difference %d" % (call, d)
        assert not torch.equal(out, torch.from_numpy(img).cuda()) or sigma == (0.0, 0.0)


def test_noalloc_rejects_oversized_image(gpu):
    f = _noalloc()
    # rejected before any device work: the pointer is never dereferenced
    status = f(C.c_void_p(16), 1025, 1024, C.c_double(2.0), C.c_double(2.0), None)
    assert status == 1  # RGPU_ERR_INVALID_ARG
    assert "1048576" in R.lib().rgpu_last_error().decode()
    assert 1025 * 1024 > MAX_PIXELS


def test_noalloc_on_a_caller_stream(gpu):
    """On a caller stream the call is enqueued and returns at once; the result
    after synchronising that stream matches the allocating entry point."""
    import torch
    f = _noalloc()
    h, w = 300, 700
    stream = torch.cuda.Stream()
    for call in range(2):
        img = _premul_image(h, w, seed=31 + call)
        ref = torch.from_numpy(img.copy()).cuda()
        out = torch.from_numpy(img.copy()).cuda()
        torch.cuda.synchronize()
        R.box_blur(ref, 4.0, 9.0)
        status = f(C.c_void_p(out.data_ptr()), w, h, C.c_double(4.0), C.c_double(9.0), C.c_void_p(stream.cuda_stream))
        assert status == 0, R.lib().rgpu_last_error().decode()
        stream.synchronize()
        torch.cuda.synchronize()
        d = (ref.to(torch.int16) - out.to(torch.int16)).abs().max().item()
        assert d <= TOLERANCE, "call %d on a caller stream: max channel difference %d" % (call, d)


@pytest.mark.parametrize("sigma", [float("nan"), float("inf"), -1.0, 2.0e8])
def test_noalloc_rejects_bad_sigma(gpu, sigma):
    f = _noalloc()
    # rejected before any device work: the pointer is never dereferenced
    status = f(C.c_void_p(16), 8, 8, C.c_double(sigma), C.c_double(1.0), None)
    assert status == 1  # RGPU_ERR_INVALID_ARG
    assert "standard deviation" in R.lib().rgpu_last_error().decode()
