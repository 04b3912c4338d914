"""feConvolveMatrix and the lighting filters on the GPU vs the CPU oracle.

Scenes are SVG text through the subset front end, rendered by the device
(resvg_render) and by the oracle under the same transform.  Convolution is
deterministic f32 in kernel order and must be bit-exact.  Lighting uses powf
for specular exponents and spot-light falloff, where CUDA's powf may differ
from the host libm in the last ulp: the tolerance there is 1/255 per channel.
"""
import numpy as np
import pytest

import resvg_gb300 as R
from resvg_gb300 import svg
from tests.helpers import diff_stats

pytestmark = pytest.mark.gpu

CONTENT = """
  <radialGradient id="rg" r="0.5"><stop offset="0.3" stop-color="#fe8"/>
    <stop offset="1" stop-color="#239" stop-opacity="0"/></radialGradient>
  <g filter="url(#f)">
    <rect x="20" y="20" width="160" height="160" fill="url(#rg)"/>
    <circle cx="70" cy="80" r="30" fill="#0a6" fill-opacity="0.7"/>
    <path d="M40 160 L160 40 L170 170 Z" fill="none" stroke="#c13" stroke-width="9"/>
  </g>"""


def _scene(filt, cif="sRGB"):
    return ('<svg viewBox="0 0 200 200" xmlns="http://www.w3.org/2000/svg">'
            '<filter id="f" x="0" y="0" width="200" height="200" filterUnits="userSpaceOnUse" '
            'color-interpolation-filters="%s">%s</filter>%s</svg>' % (cif, filt, CONTENT))


CONVOLVE = [
    '<feConvolveMatrix order="3" kernelMatrix="1 2 1 0 0 0 -1 -2 -1"/>',
    '<feConvolveMatrix order="3" kernelMatrix="0 -1 0 -1 5 -1 0 -1 0" edgeMode="none"/>',
    '<feConvolveMatrix order="4 2" kernelMatrix="1 1 1 1 2 2 2 2" edgeMode="wrap" targetX="0" targetY="1"/>',
    '<feConvolveMatrix order="5" kernelMatrix="%s" divisor="7" bias="0.1"/>' % " ".join(
        str((i * 7) % 5 - 2) for i in range(25)),
    '<feConvolveMatrix order="3" kernelMatrix="1 1 1 1 1 1 1 1 1" preserveAlpha="true" bias="-0.2"/>',
    '<feConvolveMatrix order="2 3" kernelMatrix="1 -1 2 0.5 0.25 3" edgeMode="wrap" preserveAlpha="true"/>',
]

LIGHTING = [
    '<feDiffuseLighting surfaceScale="10"><feDistantLight azimuth="45" elevation="45"/></feDiffuseLighting>',
    '<feDiffuseLighting surfaceScale="-3" diffuseConstant="1.7" lighting-color="seagreen">'
    '<fePointLight x="60" y="40" z="30"/></feDiffuseLighting>',
    '<feDiffuseLighting surfaceScale="5"><feSpotLight x="20" y="30" z="60" pointsAtX="120" pointsAtY="150" '
    'pointsAtZ="0" specularExponent="3" limitingConeAngle="35"/></feDiffuseLighting>',
    '<feSpecularLighting surfaceScale="4" specularConstant="1.3" specularExponent="12" lighting-color="#fc6">'
    '<fePointLight x="150" y="50" z="40"/></feSpecularLighting>',
    '<feSpecularLighting in="SourceAlpha" specularExponent="1"><feDistantLight azimuth="-30" elevation="60"/>'
    '</feSpecularLighting>',
    '<feSpecularLighting surfaceScale="2" specularExponent="100"><feSpotLight x="100" y="100" z="80" '
    'specularExponent="0.5"/></feSpecularLighting>',
]

TRANSFORMS = [(1.5, 0, 0, 1.5, 0, 0), (0.8660254, 0.5, -0.5, 0.8660254, 80, -30)]


def _render_both(oracle_mod, text, ts, size=300):
    tree = svg.load_svg(text)
    g = R.render(tree, ts, size, size)
    o = oracle_mod.render(tree.view(), ts, size, size)
    return g, o


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("cif", ["sRGB", "linearRGB"])
@pytest.mark.parametrize("k", range(len(CONVOLVE)))
def test_convolve_exact(gpu, oracle_mod, k, cif, ts):
    g, o = _render_both(oracle_mod, _scene(CONVOLVE[k], cif), ts)
    assert o[..., 3].any()
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("cif", ["sRGB", "linearRGB"])
@pytest.mark.parametrize("k", range(len(LIGHTING)))
def test_lighting(gpu, oracle_mod, k, cif, ts):
    g, o = _render_both(oracle_mod, _scene(LIGHTING[k], cif), ts)
    assert o[..., 3].any()
    n, mx = diff_stats(g, o)
    assert mx <= 1, (n, mx)
    # outside the powf paths the arithmetic is identical
    if "specularExponent" not in LIGHTING[k] and "feSpotLight" not in LIGHTING[k]:
        assert n == 0, n


def test_lighting_tiny_region(gpu, oracle_mod):
    """Regions narrower than 3 px stay transparent (lighting.rs apply)."""
    text = ('<svg viewBox="0 0 20 20" xmlns="http://www.w3.org/2000/svg"><filter id="f" x="5" y="5" width="2" '
            'height="10" filterUnits="userSpaceOnUse"><feDiffuseLighting><feDistantLight/></feDiffuseLighting>'
            '</filter><rect width="20" height="20" fill="red" filter="url(#f)"/></svg>')
    g, o = _render_both(oracle_mod, text, (1, 0, 0, 1, 0, 0), 20)
    assert diff_stats(g, o) == (0, 0)
