"""The GPU path against resvg's golden images.

Every committed fixture (a subset of resvg's integration suite that the
oracle reproduces with zero differing pixels) is parsed by the SVG-subset
front end and rendered through the drop-in C ABI `resvg_render` on the GPU,
then compared with the golden image under resvg's own rule (a channel
difference above 1 counts, tests/integration/main.rs:148-220).  Tolerance:
zero differing pixels, and the premultiplied output must equal the oracle's
bit for bit.
"""
import numpy as np
import pytest

import resvg_gb300 as R
from tests import golden_fixtures as G

pytestmark = pytest.mark.gpu

FIXTURES = G.load()


@pytest.mark.parametrize("idx", range(len(FIXTURES)), ids=[f[0] for f in FIXTURES])
def test_gpu_matches_golden(gpu, oracle_mod, idx):
    from resvg_gb300 import png, svg
    name, text, expected = FIXTURES[idx]
    tree = svg.load_svg(text)
    w, h, ts = G.render_transform(tree)
    got = R.render(tree, ts, w, h)
    assert G.pixel_diff(expected, png.demultiply(got)) == 0, name
    ref = oracle_mod.render(tree.view(), ts, w, h)
    n = int((got != ref).any(axis=2).sum())
    assert n == 0, "%s: %d pixels differ from the oracle" % (name, n)
