"""Pattern fills and strokes, and raster images, on the GPU vs the CPU oracle.

The tile is rendered by its own command stream, the Pattern shader (repeat
tiling, bicubic or nearest sampling, clamp, opacity) is evaluated per layer
pixel in f32 with the oracle's operation order, and the raster kernel blends
it in the highp pipeline: bit-exact.
"""
import pytest

import resvg_gb300 as R
from resvg_gb300 import svg
from tests.helpers import diff_stats

pytestmark = pytest.mark.gpu

DEFS = """
  <pattern id="p1" patternUnits="userSpaceOnUse" width="20" height="20">
    <rect width="10" height="10" fill="#2a6"/><circle cx="15" cy="15" r="5" fill="#d33" fill-opacity="0.7"/>
  </pattern>
  <pattern id="p2" width="0.25" height="0.2" patternTransform="rotate(20) skewX(10)">
    <path d="M0 0 L12 3 L4 15 Z" fill="#36c"/>
  </pattern>
  <pattern id="p3" patternContentUnits="objectBoundingBox" width="0.5" height="0.5">
    <rect width="0.25" height="0.25" fill="#fa0"/>
  </pattern>
  <pattern id="p4" patternUnits="userSpaceOnUse" width="30" height="24" viewBox="0 0 10 8"
           preserveAspectRatio="xMaxYMin slice">
    <circle cx="5" cy="4" r="4" fill="url(#p1)" stroke="#000" stroke-width="0.5"/>
  </pattern>
  <linearGradient id="lg"><stop offset="0" stop-color="#f0f"/><stop offset="1" stop-color="#0ff"/></linearGradient>
  <pattern id="p5" patternUnits="userSpaceOnUse" width="16" height="16">
    <rect width="16" height="8" fill="url(#lg)"/>
  </pattern>
"""

SCENES = [
    '<rect x="10" y="10" width="180" height="180" fill="url(#p1)"/>',
    '<ellipse cx="100" cy="100" rx="90" ry="60" fill="url(#p2)" fill-opacity="0.8"/>',
    '<rect x="20" y="30" width="160" height="120" fill="url(#p3)" stroke="url(#p1)" stroke-width="12"/>',
    '<g opacity="0.7"><circle cx="100" cy="100" r="85" fill="url(#p4)"/></g>',
    '<path d="M20 20 C 180 0 0 180 180 180" fill="none" stroke="url(#p5)" stroke-width="0.6"/>'
    '<rect x="40" y="40" width="120" height="120" fill="url(#p5)" transform="rotate(30 100 100)"/>',
]

TRANSFORMS = [(1.5, 0, 0, 1.5, 0, 0), (1, 0, 0, 1, 0, 0), (0.8660254, 0.5, -0.5, 0.8660254, 80, -30)]


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("k", range(len(SCENES)))
def test_pattern_exact(gpu, oracle_mod, k, ts):
    text = ('<svg viewBox="0 0 200 200" xmlns="http://www.w3.org/2000/svg"><defs>%s</defs>%s</svg>'
            % (DEFS, SCENES[k]))
    tree = svg.load_svg(text)
    g = R.render(tree, ts, 300, 300)
    o = oracle_mod.render(tree.view(), ts, 300, 300)
    assert o[..., 3].any()
    assert diff_stats(g, o) == (0, 0)


def _png_data_url(seed, w, h):
    import base64
    import numpy as np
    from resvg_gb300 import png
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    img[rng.random((h, w)) < 0.4, 3] = 255
    return "data:image/png;base64," + base64.b64encode(png.encode_png(img)).decode()


IMAGES = [
    '<image x="20" y="30" width="160" height="100" href="%s"/>',
    '<image x="20" y="30" width="160" height="100" preserveAspectRatio="xMaxYMid slice" '
    'image-rendering="optimizeSpeed" href="%s"/>',
    '<image x="10" y="10" width="170" href="%s" style="image-rendering:smooth" opacity="0.6" '
    'transform="rotate(12 100 100)"/>',
    '<g transform="translate(7 5)"><image width="40" height="30" href="%s" preserveAspectRatio="none"/></g>',
]


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("k", range(len(IMAGES)))
def test_raster_image_exact(gpu, oracle_mod, k, ts):
    text = ('<svg viewBox="0 0 200 200" xmlns="http://www.w3.org/2000/svg">%s</svg>'
            % (IMAGES[k] % _png_data_url(k, 23 + k, 17)))
    tree = svg.load_svg(text)
    g = R.render(tree, ts, 300, 300)
    o = oracle_mod.render(tree.view(), ts, 300, 300)
    assert o[..., 3].any()
    assert diff_stats(g, o) == (0, 0)
