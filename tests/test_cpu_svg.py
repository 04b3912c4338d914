"""The SVG-subset front end (usvg stand-in) on its own."""
import math

import numpy as np
import pytest

from resvg_gb300 import _abi as A
from resvg_gb300 import svg


def test_arc_to_cubics_endpoints_and_count():
    # a quarter circle of radius 50: kurbo needs ceil(n_err * 0.25) cubics
    cubics = svg.svg_arc_to_cubics((100, 50), (50, 100), 50, 50, 0, False, True)
    n_err = max((1.1163 * 50 / 0.1) ** (1 / 6), 3.999999)
    assert len(cubics) == math.ceil(n_err * 0.25)
    assert cubics[-1][4] == pytest.approx(50, abs=1e-9) and cubics[-1][5] == pytest.approx(100, abs=1e-9)
    # every on-curve point lies on the circle
    for c in cubics:
        assert math.hypot(c[4] - 50, c[5] - 50) == pytest.approx(50, abs=1e-9)


def test_degenerate_arc_is_a_line():
    assert svg.svg_arc_to_cubics((0, 0), (10, 0), 0, 5, 0, False, True) is None
    b = svg.parse_path_data("M0 0 A0 5 0 0 1 10 0")
    assert b.verbs == [A.MOVE, A.LINE]


def test_path_data_semantics():
    b = svg.parse_path_data("m10 10 20 0 0 20 z l 5 5")
    # implicit lineto after moveto; a segment after close starts at the subpath start
    assert b.verbs == [A.MOVE, A.LINE, A.LINE, A.CLOSE, A.MOVE, A.LINE]
    assert b.pts[-1] == (15.0, 15.0)
    b = svg.parse_path_data("M0 0 H10 V10 h-10 Z")
    assert b.pts == [(0, 0), (10, 0), (10, 10), (0, 10)]


def test_smooth_curves_reflect_control_points():
    b = svg.parse_path_data("M0 0 Q10 10 20 0 T40 0")
    assert b.verbs == [A.MOVE, A.QUAD, A.QUAD]
    assert b.pts[3] == (30.0, -10.0)


def test_colors():
    assert svg.parse_color("#0f0") == ((0, 255, 0), 1.0)
    assert svg.parse_color("rgb(10%, 20%, 30%)")[0] == (26, 51, 76)
    assert svg.parse_color("none") is None


def test_transform_list():
    t = svg.parse_transform("translate(10 20) scale(2)")
    assert t == (2, 0, 0, 2, 10, 20)
    t = svg.parse_transform("rotate(90)")
    assert t[1] == pytest.approx(1) and t[2] == pytest.approx(-1)


def test_rect_corners_in_f32(native):
    text = ('<svg viewBox="0 0 1 1" xmlns="http://www.w3.org/2000/svg">'
            '<rect x="0.2" y="0.2" width="0.6" height="0.6" rx="0.1"/></svg>')
    tree = svg.load_svg(text)
    v = tree.view().contents
    p = v.paths[0]
    pts = np.ctypeslib.as_array(v.points, shape=(v.point_count * 2,))[2 * p.point_offset:2 * (p.point_offset + 2)]
    f = np.float32
    assert pts[0] == f(0.2) + f(0.1) and pts[2] == (f(0.2) + f(0.6)) - f(0.1)


def test_number_lists_as_usvg_reads_them():
    assert svg.number_list_strict("1 0,0.5 -1e1") == [1.0, 0.0, 0.5, -10.0]
    assert svg.number_list_strict("100-100") == [100.0, -100.0]
    assert svg.number_list_strict("1px") is None
    assert svg.number_list_strict("") == []
    assert svg.number_strict(" 0.5 ") == 0.5
    assert svg.number_strict("0.5px") is None and svg.number_strict("50%") is None
    # stdDeviation: one or two numbers, else 0 0; negative components become 0
    assert svg.std_dev_attr("3") == (3.0, 3.0)
    assert svg.std_dev_attr("3 -1") == (3.0, 0.0)
    assert svg.std_dev_attr("1 2 3") == (0.0, 0.0)
    assert svg.std_dev_attr("4 x") == (4.0, 4.0)
    assert svg.opacity_value("50%") == 0.5 and svg.opacity_value("2") == 1.0


def test_filter_function_list():
    fl = svg.parse_filter_list("grayscale() url(#a) hue-rotate(0.25turn) blur(1mm) opacity(50%)")
    assert fl[0] == ("grayscale", 1.0) and fl[1] == ("url", "a")
    assert fl[2] == ("hue-rotate", 90.0) and fl[3] == ("blur", (1.0, "mm")) and fl[4] == ("opacity", 0.5)
    ds = svg.parse_filter_list("drop-shadow(4 5 6 blue)")[0]
    assert ds[0] == "drop-shadow" and ds[1][0] == ((0, 0, 255), 1.0) and ds[1][3] == (6.0, "")
    assert svg.parse_filter_list("drop-shadow(currentColor 1 2)")[0][1][0] is None
    # any item that does not parse drops the whole list
    for bad in ("blur(4 2)", "blur(50%)", "blur(-5)", "drop-shadow(red, 10, 15)", "drop-shadow(4)",
                "drop-shadow(blue 4 5 6 7)", "drop-shadow(blue 3% 4% 5%)", "hue-rotate(45)",
                "grayscale() hue-rotate(random) opacity(0.5)", "contrast(-1)", "bogus(1)"):
        assert svg.parse_filter_list(bad) is None, bad
    assert svg.parse_filter_list("hue-rotate(0)") == [("hue-rotate", 0.0)]


def test_component_transfer_record():
    text = ('<svg viewBox="0 0 10 10" xmlns="http://www.w3.org/2000/svg"><filter id="f">'
            '<feComponentTransfer><feFuncB type="table" tableValues="0 0 1 1"/>'
            '<feFuncB type="table" tableValues="1 1 0 0"/><feFuncR type="random"/>'
            '<feFuncA type="gamma" amplitude="2px" offset="0.5"/></feComponentTransfer></filter>'
            '<rect width="5" height="5" filter="url(#f)"/></svg>')
    tree = svg.load_svg(text)
    p = tree.view().contents.prims[0]
    assert p.kind == A.FE_COMPONENT_TRANSFER
    assert p.i[0] == A.TF_IDENTITY and p.i[2] == A.TF_TABLE and p.i[6] == 4
    assert list(p.f[32:36]) == [1.0, 1.0, 0.0, 0.0]       # the later feFuncB wins
    assert p.i[3] == A.TF_GAMMA and list(p.f[48:51]) == [1.0, 1.0, 0.5]   # invalid amplitude: default


def test_node_by_id_follows_usvg_order():
    """rgpu_tree_find_node restates usvg's node_by_id (crates/usvg/src/tree/
    mod.rs:1718-1732): depth-first pre-order below the root, first match wins,
    the root group and detached groups are not searched, "" never matches."""
    import resvg_gb300 as R
    from resvg_gb300 import _abi as A
    from tests.helpers import base_path, plain_group, rect_path
    t = R.Tree(100, 100)
    root = t.add_group(-1, plain_group())
    g1 = t.add_group(root, plain_group())
    v, p = rect_path(0, 0, 10, 10)
    p0 = t.add_path(g1, base_path(), v, p)
    g2 = t.add_group(root, plain_group())
    p1 = t.add_path(g2, base_path(), v, p)
    detached = t.add_group(-1, plain_group())
    p2 = t.add_path(detached, base_path(), v, p)
    t.set_node_id(A.NODE_GROUP, root, "root")
    t.set_node_id(A.NODE_PATH, p0, "dup")     # inside g1: visited before g2
    t.set_node_id(A.NODE_GROUP, g2, "dup")
    t.set_node_id(A.NODE_PATH, p1, "leaf")
    t.set_node_id(A.NODE_PATH, p2, "hidden")
    t.set_node_id(A.NODE_GROUP, detached, "clip-content")
    t.finalize()
    assert t.find_node("dup") == (A.NODE_PATH, p0)
    assert t.find_node("leaf") == (A.NODE_PATH, p1)
    assert t.find_node("root") is None
    assert t.find_node("hidden") is None and t.find_node("clip-content") is None
    assert t.find_node("") is None and t.find_node("missing") is None
    import pytest
    with pytest.raises(R.RenderError):
        t.set_node_id(A.NODE_PATH, 99, "x")


def test_front_end_keeps_svg_ids():
    from resvg_gb300 import svg
    tree = svg.load_svg('<svg xmlns="http://www.w3.org/2000/svg" width="50" height="50">'
                        '<g id="outer"><rect id="box" x="5" y="5" width="20" height="20" fill="red"/></g>'
                        '<circle id="dot" cx="30" cy="30" r="5"/></svg>')
    from resvg_gb300 import _abi as A
    assert tree.find_node("box")[0] == A.NODE_PATH
    assert tree.find_node("dot")[0] == A.NODE_PATH
    assert tree.find_node("nope") is None


def _paths(tree):
    v = tree.view().contents
    out = []
    for i in range(v.path_count):
        p = v.paths[i]
        pts = [v.points[j] for j in range(p.point_offset * 2, (p.point_offset + p.point_count) * 2)]
        out.append((p, pts))
    return v, out


def test_root_background_color_is_a_viewbox_rect():
    """usvg converter.rs:393-521: a plain-colour background-color on the root
    becomes the first path, a rect of the viewBox with the alpha as opacity;
    none, currentColor and links add nothing."""
    tree = svg.load_svg('<svg xmlns="http://www.w3.org/2000/svg" viewBox="10 20 200 100" width="400" '
                        'style="background-color: #0000ff80"><rect width="5" height="5"/></svg>')
    v, paths = _paths(tree)
    assert len(paths) == 2
    p, pts = paths[0]
    assert pts == [10.0, 20.0, 210.0, 20.0, 210.0, 120.0, 10.0, 120.0]
    assert p.fill_opacity == pytest.approx(128 / 255, abs=1e-7)
    paint = v.paints[p.fill_paint]
    assert (paint.r, paint.g, paint.b) == (0, 0, 255)
    for bg in ("none", "currentColor", "url(#x)", "#12"):
        tree = svg.load_svg('<svg xmlns="http://www.w3.org/2000/svg" width="50" height="50" '
                            f'background-color="{bg}"><rect width="5" height="5"/></svg>')
        assert len(_paths(tree)[1]) == 1


def test_url_reference_allows_spaces():
    tree = svg.load_svg('<svg xmlns="http://www.w3.org/2000/svg" width="50" height="50">'
                        '<linearGradient id="lg1"><stop offset="0"/><stop offset="1" stop-color="white"/>'
                        '</linearGradient><rect width="40" height="40" fill="  url(  #lg1   )  "/></svg>')
    v, paths = _paths(tree)
    assert v.paints[paths[0][0].fill_paint].kind == A.PAINT_LINEAR


def test_concentric_equal_radii_radial_is_a_ring():
    """The two-point conical constructor's degenerate case: focus = centre and
    fr = r under pad spread become a plain radial gradient of radius r whose
    stops are (0, first), (1, first), (1, last)."""
    tree = svg.load_svg('<svg xmlns="http://www.w3.org/2000/svg" width="50" height="50">'
                        '<radialGradient id="g" fr="0.5"><stop offset="0.2" stop-color="black"/>'
                        '<stop offset="0.5" stop-color="red"/><stop offset="1" stop-color="white"/>'
                        '</radialGradient><rect width="40" height="40" fill="url(#g)"/></svg>')
    v, paths = _paths(tree)
    paint = v.paints[paths[0][0].fill_paint]
    assert paint.kind == A.PAINT_RADIAL and paint.fr == 0.0 and paint.r_ == pytest.approx(0.5)
    stops = [v.stops[paint.stop_offset + i] for i in range(paint.stop_count)]
    assert [s.offset for s in stops] == [0.0, 1.0, 1.0]
    assert [(s.r, s.g, s.b) for s in stops] == [(0, 0, 0), (0, 0, 0), (255, 255, 255)]
    with pytest.raises(svg.Unsupported):
        svg.load_svg('<svg xmlns="http://www.w3.org/2000/svg" width="50" height="50">'
                     '<radialGradient id="g" fr="0.5" spreadMethod="repeat"><stop offset="0"/>'
                     '<stop offset="1" stop-color="white"/></radialGradient>'
                     '<rect width="40" height="40" fill="url(#g)"/></svg>')
