"""Arithmetic identities the filter kernels rely on, checked exhaustively."""
import numpy as np


def test_box_rounding_is_an_integer_quotient():
    # box_blur.rs rounds the f32 product sum * (1 / (2r + 1)) half to even; the
    # kernels compute (sum + r) / (2r + 1) as a multiply-high by
    # ceil(2^32 / (2r + 1)).  All three agree for every window sum of u8 values.
    for r in range(1, 128):
        d = 2 * r + 1
        s = np.arange(0, 255 * d + 1, dtype=np.int64)
        iarr = np.float32(1.0) / np.float32(d)
        ref = np.rint(s.astype(np.float32) * iarr).astype(np.int64)
        q = (s + r) // d
        m = (2 ** 32 + 2 * r) // d
        assert m < 2 ** 32
        mh = ((s + r) * m) >> 32
        assert np.array_equal(ref, q), r
        assert np.array_equal(mh, q), r
