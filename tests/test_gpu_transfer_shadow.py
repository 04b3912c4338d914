"""feComponentTransfer, feDropShadow, feTurbulence, feTile,
feDisplacementMap, feImage and the CSS filter functions on the GPU vs the CPU
oracle.

The transfer functions are evaluated on the host into one 256-entry table per
channel with the same f32 operations as the oracle (powf included), so the
device result is bit-exact.  The drop shadow runs the blur kernels (box or
IIR, both exact), a per-alpha flood table and two source-over draws: also
bit-exact.  Turbulence is f64 arithmetic in the reference's order, without
contraction, with the generator's tables rebuilt on the device: bit-exact.
"""
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


TRANSFER = [
    '<feComponentTransfer><feFuncR type="table" tableValues="1 0.2 0.8 0"/>'
    '<feFuncG type="discrete" tableValues="0 0.5 1"/><feFuncB type="linear" slope="1.7" intercept="-0.3"/>'
    '<feFuncA type="gamma" amplitude="1.2" exponent="0.45" offset="-0.05"/></feComponentTransfer>',
    '<feComponentTransfer><feFuncA type="table" tableValues="0 0 1 1 0.5"/></feComponentTransfer>',
    '<feComponentTransfer><feFuncR type="gamma" amplitude="0" exponent="-2"/>'
    '<feFuncG type="gamma" exponent="3.3"/><feFuncB type="table" tableValues="9999 -9999"/>'
    '</feComponentTransfer>',
    '<feComponentTransfer><feFuncR type="discrete" tableValues="%s"/><feFuncG type="table" tableValues="%s"/>'
    '</feComponentTransfer>' % (" ".join(str((k * 37 % 11) / 10) for k in range(16)),
                                " ".join(str((k * 5 % 7) / 6) for k in range(16))),
]

SHADOW = [
    '<feDropShadow stdDeviation="6" dx="10" dy="-7"/>',
    '<feDropShadow stdDeviation="1.2 0.4" dx="-4" dy="9" flood-color="#3af" flood-opacity="0.6"/>',
    '<feDropShadow stdDeviation="0" dx="3" dy="3" flood-color="rgba(200, 40, 90, 0.5)"/>',
    '<feDropShadow in="SourceAlpha" stdDeviation="3 9" dx="0" dy="12" flood-color="seagreen"/>',
]

TURBULENCE = [
    '<feTurbulence baseFrequency="0.05"/>',
    '<feTurbulence baseFrequency="0.02 0.07" numOctaves="4" seed="7" type="fractalNoise"/>',
    '<feTurbulence baseFrequency="0.03" numOctaves="3" seed="-20" stitchTiles="stitch"/>',
    '<feTurbulence baseFrequency="0.011 0.013" numOctaves="2" seed="1e10" stitchTiles="stitch" '
    'type="fractalNoise"/>',
    '<feTurbulence baseFrequency="0.1" numOctaves="0" type="fractalNoise" seed="-1e10"/>',
    '<feTurbulence baseFrequency="0.04" numOctaves="6" seed="2.9"/>'
    '<feComposite in2="SourceGraphic" operator="in"/>',
]

TILE_DISPLACE = [
    '<feFlood flood-color="seagreen" flood-opacity="0.7" x="28" y="28" width="10" height="13"/>'
    '<feOffset dx="5" dy="5"/><feTile/>',
    '<feOffset dx="-7" dy="3" x="30" y="40" width="23" height="17"/><feTile x="20" y="30" width="150" height="120"/>',
    '<feFlood flood-color="red" x="0" y="0" width="10" height="10"/><feOffset dx="5" dy="5"/><feTile/>',
    '<feTurbulence baseFrequency="0.03" numOctaves="2" result="t"/>'
    '<feDisplacementMap in="SourceGraphic" in2="t" scale="12" xChannelSelector="R" yChannelSelector="G"/>',
    '<feDisplacementMap in2="SourceAlpha" scale="-3" xChannelSelector="A" yChannelSelector="B"/>',
]

# feImage of an element: each scene defines #img (the scene content's own
# gradient is reused) before the filter
FE_IMAGE_DEFS = ('<defs><g id="img" opacity="0.8"><rect x="10" y="30" width="90" height="60" fill="#3a7" '
                 'transform="rotate(15 50 60)"/><circle cx="120" cy="100" r="40" fill="url(#rg)"/></g>'
                 '<filter id="inner" x="0" y="0" width="200" height="200" filterUnits="userSpaceOnUse">'
                 '<feGaussianBlur stdDeviation="2"/></filter>'
                 '<rect id="blurred" x="30" y="30" width="100" height="80" fill="#e52" filter="url(#inner)"/></defs>')
FE_IMAGE = [
    '<feImage href="#img"/>',
    '<feImage href="#img" x="20" y="10" width="150" height="120"/><feComposite in2="SourceGraphic" operator="over"/>',
    '<feImage href="#blurred"/><feBlend in2="SourceGraphic" mode="multiply"/>',
    '<feImage href="#missing"/><feMerge><feMergeNode/><feMergeNode in="SourceGraphic"/></feMerge>',
]

FUNCTIONS = [
    'blur(3)',
    'drop-shadow(blue 4 5 6) grayscale(0.3)',
    'sepia(0.8) hue-rotate(0.1turn) saturate(2.5)',
    'brightness(140%) contrast(0.6) invert(0.25) opacity(0.8)',
    'url(#f) drop-shadow(-6 -3 1 rgba(0, 0, 0, 0.5))',
]

TRANSFORMS = [(1.5, 0, 0, 1.5, 0, 0), (0.8660254, 0.5, -0.5, 0.8660254, 80, -30)]


def _render_both(oracle_mod, text, ts, size=300):
    tree = svg.load_svg(text)
    g = R.render(tree, ts, size, size)
    o = oracle_mod.render(tree.view(), ts, size, size)
    return g, o


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("cif", ["sRGB", "linearRGB"])
@pytest.mark.parametrize("k", range(len(TRANSFER)))
def test_component_transfer_exact(gpu, oracle_mod, k, cif, ts):
    g, o = _render_both(oracle_mod, _scene(TRANSFER[k], cif), ts)
    assert o[..., 3].any()
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("cif", ["sRGB", "linearRGB"])
@pytest.mark.parametrize("k", range(len(SHADOW)))
def test_drop_shadow_exact(gpu, oracle_mod, k, cif, ts):
    g, o = _render_both(oracle_mod, _scene(SHADOW[k], cif), ts)
    assert o[..., 3].any()
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("cif", ["sRGB", "linearRGB"])
@pytest.mark.parametrize("k", range(len(TURBULENCE)))
def test_turbulence_exact(gpu, oracle_mod, k, cif, ts):
    g, o = _render_both(oracle_mod, _scene(TURBULENCE[k], cif), ts)
    assert o[..., 3].any()
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("cif", ["sRGB", "linearRGB"])
@pytest.mark.parametrize("k", range(len(TILE_DISPLACE)))
def test_tile_displacement_exact(gpu, oracle_mod, k, cif, ts):
    g, o = _render_both(oracle_mod, _scene(TILE_DISPLACE[k], cif), ts)
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("k", range(len(FE_IMAGE)))
def test_fe_image_exact(gpu, oracle_mod, k, ts):
    text = _scene(FE_IMAGE[k]).replace("<filter id=\"f\"", FE_IMAGE_DEFS + "<filter id=\"f\"", 1)
    g, o = _render_both(oracle_mod, text, ts)
    assert o[..., 3].any()
    assert diff_stats(g, o) == (0, 0)


@pytest.mark.parametrize("ts", TRANSFORMS)
@pytest.mark.parametrize("k", range(len(FUNCTIONS)))
def test_filter_functions_exact(gpu, oracle_mod, k, ts):
    text = _scene('<feOffset dx="3" dy="2"/>').replace('filter="url(#f)"', 'filter="%s"' % FUNCTIONS[k])
    g, o = _render_both(oracle_mod, text, ts)
    assert o[..., 3].any()
    assert diff_stats(g, o) == (0, 0)
