"""SVG-subset front end: parses SVG text into the backend's render tree.

A stand-in for the parts of usvg (crates/usvg/src/parser/**) that produce the
tree resvg renders: shapes to paths (parser/shapes.rs: rect with rx/ry,
circle/ellipse as four arcs, line/polyline/polygon), path data with arcs
converted to cubics the way usvg does it (kurbo's SvgArc -> Arc ->
to_cubic_beziers(0.1), parser/shapes.rs:276-330), presentation attributes and
`style`, inheritance, transforms, `use`, gradients with objectBoundingBox units
and normalised stops (parser/paint_server.rs:277-405), clipPath, mask and the
filter primitives the backend implements, with usvg's default regions
(parser/filter.rs:185-214).

Unsupported features raise `Unsupported`; the golden-image harness uses that
to select the reference tests this front end can express.
"""
from __future__ import annotations

import math
import re
import xml.etree.ElementTree as ET

import numpy as np

from . import _abi as A

SVG_NS = "{http://www.w3.org/2000/svg}"
XLINK = "{http://www.w3.org/1999/xlink}href"


class Unsupported(Exception):
    pass


# ---------------------------------------------------------------- colours
# the CSS Color Module keywords (the SVG 1.1 set plus rebeccapurple)
NAMED = {
    "aliceblue": (240, 248, 255), "antiquewhite": (250, 235, 215), "aqua": (0, 255, 255),
    "aquamarine": (127, 255, 212), "azure": (240, 255, 255), "beige": (245, 245, 220), "bisque": (255, 228, 196),
    "black": (0, 0, 0), "blanchedalmond": (255, 235, 205), "blue": (0, 0, 255), "blueviolet": (138, 43, 226),
    "brown": (165, 42, 42), "burlywood": (222, 184, 135), "cadetblue": (95, 158, 160),
    "chartreuse": (127, 255, 0), "chocolate": (210, 105, 30), "coral": (255, 127, 80),
    "cornflowerblue": (100, 149, 237), "cornsilk": (255, 248, 220), "crimson": (220, 20, 60),
    "cyan": (0, 255, 255), "darkblue": (0, 0, 139), "darkcyan": (0, 139, 139), "darkgoldenrod": (184, 134, 11),
    "darkgray": (169, 169, 169), "darkgreen": (0, 100, 0), "darkgrey": (169, 169, 169),
    "darkkhaki": (189, 183, 107), "darkmagenta": (139, 0, 139), "darkolivegreen": (85, 107, 47),
    "darkorange": (255, 140, 0), "darkorchid": (153, 50, 204), "darkred": (139, 0, 0),
    "darksalmon": (233, 150, 122), "darkseagreen": (143, 188, 143), "darkslateblue": (72, 61, 139),
    "darkslategray": (47, 79, 79), "darkslategrey": (47, 79, 79), "darkturquoise": (0, 206, 209),
    "darkviolet": (148, 0, 211), "deeppink": (255, 20, 147), "deepskyblue": (0, 191, 255),
    "dimgray": (105, 105, 105), "dimgrey": (105, 105, 105), "dodgerblue": (30, 144, 255),
    "firebrick": (178, 34, 34), "floralwhite": (255, 250, 240), "forestgreen": (34, 139, 34),
    "fuchsia": (255, 0, 255), "gainsboro": (220, 220, 220), "ghostwhite": (248, 248, 255),
    "gold": (255, 215, 0), "goldenrod": (218, 165, 32), "gray": (128, 128, 128), "grey": (128, 128, 128),
    "green": (0, 128, 0), "greenyellow": (173, 255, 47), "honeydew": (240, 255, 240),
    "hotpink": (255, 105, 180), "indianred": (205, 92, 92), "indigo": (75, 0, 130), "ivory": (255, 255, 240),
    "khaki": (240, 230, 140), "lavender": (230, 230, 250), "lavenderblush": (255, 240, 245),
    "lawngreen": (124, 252, 0), "lemonchiffon": (255, 250, 205), "lightblue": (173, 216, 230),
    "lightcoral": (240, 128, 128), "lightcyan": (224, 255, 255), "lightgoldenrodyellow": (250, 250, 210),
    "lightgray": (211, 211, 211), "lightgreen": (144, 238, 144), "lightgrey": (211, 211, 211),
    "lightpink": (255, 182, 193), "lightsalmon": (255, 160, 122), "lightseagreen": (32, 178, 170),
    "lightskyblue": (135, 206, 250), "lightslategray": (119, 136, 153), "lightslategrey": (119, 136, 153),
    "lightsteelblue": (176, 196, 222), "lightyellow": (255, 255, 224), "lime": (0, 255, 0),
    "limegreen": (50, 205, 50), "linen": (250, 240, 230), "magenta": (255, 0, 255), "maroon": (128, 0, 0),
    "mediumaquamarine": (102, 205, 170), "mediumblue": (0, 0, 205), "mediumorchid": (186, 85, 211),
    "mediumpurple": (147, 112, 219), "mediumseagreen": (60, 179, 113), "mediumslateblue": (123, 104, 238),
    "mediumspringgreen": (0, 250, 154), "mediumturquoise": (72, 209, 204), "mediumvioletred": (199, 21, 133),
    "midnightblue": (25, 25, 112), "mintcream": (245, 255, 250), "mistyrose": (255, 228, 225),
    "moccasin": (255, 228, 181), "navajowhite": (255, 222, 173), "navy": (0, 0, 128),
    "oldlace": (253, 245, 230), "olive": (128, 128, 0), "olivedrab": (107, 142, 35), "orange": (255, 165, 0),
    "orangered": (255, 69, 0), "orchid": (218, 112, 214), "palegoldenrod": (238, 232, 170),
    "palegreen": (152, 251, 152), "paleturquoise": (175, 238, 238), "palevioletred": (219, 112, 147),
    "papayawhip": (255, 239, 213), "peachpuff": (255, 218, 185), "peru": (205, 133, 63), "pink": (255, 192, 203),
    "plum": (221, 160, 221), "powderblue": (176, 224, 230), "purple": (128, 0, 128),
    "rebeccapurple": (102, 51, 153), "red": (255, 0, 0), "rosybrown": (188, 143, 143),
    "royalblue": (65, 105, 225), "saddlebrown": (139, 69, 19), "salmon": (250, 128, 114),
    "sandybrown": (244, 164, 96), "seagreen": (46, 139, 87), "seashell": (255, 245, 238),
    "sienna": (160, 82, 45), "silver": (192, 192, 192), "skyblue": (135, 206, 235),
    "slateblue": (106, 90, 205), "slategray": (112, 128, 144), "slategrey": (112, 128, 144),
    "snow": (255, 250, 250), "springgreen": (0, 255, 127), "steelblue": (70, 130, 180), "tan": (210, 180, 140),
    "teal": (0, 128, 128), "thistle": (216, 191, 216), "tomato": (255, 99, 71), "turquoise": (64, 224, 208),
    "violet": (238, 130, 238), "wheat": (245, 222, 179), "white": (255, 255, 255),
    "whitesmoke": (245, 245, 245), "yellow": (255, 255, 0), "yellowgreen": (154, 205, 50),
}


class InvalidColor(Unsupported):
    """A colour value svgtypes would reject."""


def parse_color(s: str, current=(0, 0, 0)):
    """Returns ((r, g, b), alpha) or None for 'none'; InvalidColor for text
    svgtypes rejects (including a trailing icc-color(...))."""
    s = s.strip()
    low = s.lower()
    if low == "none":
        return None
    if low == "transparent":
        return (0, 0, 0), 0.0
    if low == "currentcolor":
        return current, 1.0
    if low in NAMED:
        return NAMED[low], 1.0
    if s.startswith("#"):
        h = s[1:]
        if not re.fullmatch(r"[0-9a-fA-F]*", h):
            raise InvalidColor("color " + s)
        if len(h) == 3:
            return tuple(int(c * 2, 16) for c in h), 1.0
        if len(h) == 4:
            return tuple(int(c * 2, 16) for c in h[:3]), int(h[3] * 2, 16) / 255.0
        if len(h) == 6:
            return (int(h[0:2], 16), int(h[2:4], 16), int(h[4:6], 16)), 1.0
        if len(h) == 8:
            return (int(h[0:2], 16), int(h[2:4], 16), int(h[4:6], 16)), int(h[6:8], 16) / 255.0
        raise InvalidColor("color " + s)
    m = re.match(r"rgba?\(([^)]*)\)$", low)
    if m:
        parts = [p.strip() for p in re.split(r"[,\s/]+", m.group(1).strip()) if p.strip()]
        # svgtypes: the three channels all numbers or all percentages, alpha a number
        if len(parts) < 3 or len({q.endswith("%") for q in parts[:3]}) != 1 or \
                (len(parts) > 3 and parts[3].endswith("%")):
            raise InvalidColor("color " + s)
        vals = []
        for p in parts[:3]:
            if p.endswith("%"):
                vals.append(int(round(float(p[:-1]) * 2.55)))
            else:
                vals.append(int(round(float(p))))
        vals = [max(0, min(255, v)) for v in vals]
        a = 1.0
        if len(parts) > 3:
            a = float(parts[3][:-1]) / 100 if parts[3].endswith("%") else float(parts[3])
        return tuple(vals), max(0.0, min(1.0, a))
    m = re.match(r"hsla?\(([^)]*)\)", low)
    if m:
        # CSS Color 3 hsl(): hue in degrees, saturation and lightness in
        # [0, 1], each channel rounded to u8 (f32 arithmetic)
        parts = [p.strip() for p in re.split(r"[,\s/]+", m.group(1).strip()) if p.strip()]
        if len(parts) < 3:
            raise Unsupported("color " + s)

        def frac(v):
            return float(v[:-1]) / 100 if v.endswith("%") else float(v)
        hue = (float(parts[0]) % 360.0 + 360.0) % 360.0
        sat, lig = F(max(0.0, min(1.0, frac(parts[1])))), F(max(0.0, min(1.0, frac(parts[2]))))
        h6 = F(F(hue) / F(60.0))
        t2 = F(lig * F(sat + F(1.0))) if lig <= 0.5 else F(F(lig + sat) - F(lig * sat))
        t1 = F(F(lig * F(2.0)) - t2)

        def channel(hh):
            hh = F(hh)
            if hh < 0:
                hh = F(hh + F(6.0))
            if hh >= 6:
                hh = F(hh - F(6.0))
            if hh < 1:
                v = F(F(F(t2 - t1) * hh) + t1)
            elif hh < 3:
                v = t2
            elif hh < 4:
                v = F(F(F(t2 - t1) * F(F(4.0) - hh)) + t1)
            else:
                v = t1
            x = F(v * F(255.0))
            return int(np.floor(x + 0.5)) if x >= 0 else -int(np.floor(-x + 0.5))
        rgb = tuple(max(0, min(255, channel(h6 + d))) for d in (F(2.0), F(0.0), F(-2.0)))
        a = 1.0
        if len(parts) > 3:
            a = frac(parts[3])
        return rgb, max(0.0, min(1.0, a))
    raise InvalidColor("color " + s)


# ---------------------------------------------------------------- numbers, lengths, transforms
NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _approx_zero_ulps(v):
    """usvg's approx_zero_ulps(4) for an f32."""
    a = int(np.array([v], dtype=np.float32).view(np.int32)[0])
    if a < 0:
        return float(v) == 0.0
    return a <= 4


def numbers(s):
    return [float(x) for x in re.findall(NUM, s or "")]


def number_strict(s):
    """svgtypes Number::from_str: one number with optional surrounding spaces,
    else None (usvg then uses the attribute's default)."""
    if s is None:
        return None
    m = re.fullmatch(r"\s*(" + NUM + r")\s*", s)
    return float(m.group(1)) if m else None


_WS = re.compile(r"[ \t\n\r]*")
_SEP = re.compile(r"[ \t\n\r]*,?")
_NUM_RE = re.compile(NUM)


def number_list_items(s):
    """svgtypes NumberListParser: numbers separated by spaces and at most one
    comma; an item that does not parse yields None and ends the list."""
    out, pos, n = [], 0, len(s or "")
    while True:
        pos = _WS.match(s, pos).end()
        if pos >= n:
            return out
        m = _NUM_RE.match(s, pos)
        if not m:
            out.append(None)
            return out
        out.append(float(m.group(0)))
        pos = _SEP.match(s, m.end()).end()


def number_list_strict(s):
    """usvg's Vec<f32> attribute: the whole list, or None when any item fails."""
    items = number_list_items(s)
    return None if None in items else items


def std_dev_attr(text):
    """parser/filter.rs convert_std_dev_attr: one or two numbers (a third one,
    or none, gives 0 0); each negative component becomes 0."""
    n1, n2, n3 = (number_list_items(text) + [None, None, None])[:3]
    if n1 is not None and n2 is not None and n3 is None:
        x, y = n1, n2
    elif n1 is not None and n2 is None:
        x, y = n1, n1
    else:
        x, y = 0.0, 0.0
    x, y = F(x), F(y)
    return (float(x) if x >= 0 else 0.0), (float(y) if y >= 0 else 0.0)


def opacity_value(s, default=1.0):
    """usvg's Opacity attribute: a number or a percentage, clamped to [0, 1]."""
    if s is None:
        return default
    m = re.fullmatch(r"\s*(" + NUM + r")\s*(%?)\s*", s)
    if not m:
        return default
    v = float(m.group(1)) / (100.0 if m.group(2) else 1.0)
    return float(min(max(F(v), F(0.0)), F(1.0)))


_LEN_UNITS = ("px", "em", "ex", "in", "cm", "mm", "pt", "pc", "%")


def _split_top(s):
    """Splits at whitespace outside parentheses."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch in " \t\n\r" and depth == 0:
            if cur:
                out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur:
        out.append(cur)
    return out


def _css_length(tok):
    m = re.fullmatch("(" + NUM + r")(px|em|ex|in|cm|mm|pt|pc|%)?", tok)
    return (float(m.group(1)), m.group(2) or "") if m else None


def parse_filter_list(value):
    """The `filter` property's value as a list of ("url", id) and filter
    functions (Filter Effects 1, section 12: blur, brightness, contrast,
    drop-shadow, grayscale, hue-rotate, invert, opacity, saturate, sepia),
    following svgtypes' FilterValueListParser as usvg consumes it
    (parser/filter.rs:86-148).  None when any item does not parse: usvg then
    drops the whole list.  Arguments: a length (number, unit; no percentage)
    for blur; an amount (a number or a percentage, not negative) for the colour
    functions; degrees for hue-rotate (a unit is required unless the angle is
    0); (colour or None, dx, dy, std) for drop-shadow, two or three lengths
    without percentages and the colour first or last."""
    out, pos, n = [], 0, len(value)
    while True:
        pos = _WS.match(value, pos).end()
        if pos >= n:
            return out
        m = re.compile(r"([A-Za-z-]+)\(").match(value, pos)
        if not m:
            return None
        depth, k = 1, m.end()
        while k < n and depth:
            depth += {"(": 1, ")": -1}.get(value[k], 0)
            k += 1
        if depth:
            return None
        name, arg = m.group(1), value[m.end():k - 1].strip()
        pos = k
        if name == "url":
            out.append(("url", arg.strip("'\"").lstrip("#")))
        elif name == "blur":
            if not arg:
                out.append(("blur", (0.0, "")))
                continue
            ln = _css_length(arg)
            if ln is None or ln[1] == "%" or ln[0] < 0:
                return None
            out.append(("blur", ln))
        elif name in ("brightness", "contrast", "grayscale", "invert", "opacity", "saturate", "sepia"):
            if not arg:
                out.append((name, 1.0))
                continue
            mm = re.fullmatch("(" + NUM + r")(%?)", arg)
            if not mm or float(mm.group(1)) < 0:
                return None
            out.append((name, float(mm.group(1)) / (100.0 if mm.group(2) else 1.0)))
        elif name == "hue-rotate":
            if not arg:
                out.append((name, 0.0))
                continue
            mm = re.fullmatch("(" + NUM + r")(deg|grad|rad|turn)?", arg)
            if not mm or (mm.group(2) is None and float(mm.group(1)) != 0.0):
                return None  # an angle needs its unit; only zero may go without
            v, u = float(mm.group(1)), mm.group(2) or "deg"
            deg = {"deg": v, "grad": v * 180.0 / 200.0, "rad": math.degrees(v), "turn": v * 360.0}[u]
            out.append((name, deg))
        elif name == "drop-shadow":
            toks = _split_top(arg)
            color, lens = None, []
            for i, t in enumerate(toks):
                ln = _css_length(t)
                if ln is not None:
                    if ln[1] == "%":
                        return None  # lengths only, no percentages
                    lens.append(ln)
                    continue
                if color is not None or (i != 0 and i != len(toks) - 1):
                    return None
                if t.lower() == "currentcolor":
                    color = "current"
                    continue
                try:
                    c = parse_color(t)
                except (InvalidColor, Unsupported):
                    return None
                if c is None:
                    return None
                color = c
            if len(lens) not in (2, 3):
                return None
            out.append((name, (None if color == "current" else color, lens[0], lens[1],
                               lens[2] if len(lens) == 3 else (0.0, ""))))
        else:
            return None


class InvalidLength(Unsupported):
    """A length svgtypes does not parse (an unknown unit or stray text)."""


def parse_length(s, ref=0.0, font_size=12.0):
    s = s.strip()
    m = re.match(r"(" + NUM + r")\s*([a-z%]*)$", s)
    if not m:
        raise InvalidLength("length " + s)
    v, u = float(m.group(1)), m.group(2)
    if u in ("", "px"):
        return v
    if u == "%":
        return v * ref / 100.0
    if u == "em":
        return v * font_size
    if u == "ex":
        return v * font_size / 2.0
    if u == "in":
        return v * 96.0
    if u == "cm":
        return v * 96.0 / 2.54
    if u == "mm":
        return v * 96.0 / 25.4
    if u == "pt":
        return v * 4.0 / 3.0
    if u == "pc":
        return v * 16.0
    raise InvalidLength("unit " + u)


_CSS_NOT_PRESENTATION = {"x", "y", "width", "height", "rx", "ry", "cx", "cy", "r", "d", "points", "x1", "y1",
                         "x2", "y2", "href", "id", "class", "viewBox", "preserveAspectRatio", "offset"}
_CSS_SIMPLE = re.compile(r"\*|[A-Za-z][\w-]*|#[\w-]+|\.[\w-]+|:first-child|"
                         r"\[\s*([\w-]+)\s*(?:([~|^$*]?=)\s*[\"']?([^\"'\]]*)[\"']?\s*)?\]")


def _css_compound(text):
    """A compound selector as a list of (kind, value) tests, None if unsupported."""
    out, pos = [], 0
    while pos < len(text):
        m = _CSS_SIMPLE.match(text, pos)
        if not m:
            return None
        t = m.group(0)
        if t.startswith("["):
            out.append(("attr", (m.group(1), m.group(2), m.group(3))))
        elif t == ":first-child":
            out.append(("first", None))
        elif t[0] in "#.":
            out.append(("id" if t[0] == "#" else "class", t[1:]))
        elif t != "*":
            out.append(("type", t))
        pos = m.end()
    return out


def _css_selector(text):
    """(parts, specificity): parts right to left as (compound, combinator to the left)."""
    toks = re.findall(r">|[^\s>]+", text.strip())
    parts, comb = [], " "
    seq = []
    for t in toks:
        if t == ">":
            comb = ">"
            continue
        c = _css_compound(t)
        if c is None:
            return None
        seq.append((c, comb))
        comb = " "
    if not seq:
        return None
    spec = [0, 0, 0]
    for c, _ in seq:
        for kind, _v in c:
            spec[0 if kind == "id" else (2 if kind == "type" else 1)] += 1
    for i, (c, cb) in enumerate(seq):
        parts.append((c, seq[i][1]))
    return list(reversed(parts)), tuple(spec)


def stylesheet_rules(root):
    """{element: [(name, value, important)]} from the document's <style> sheets
    (type text/css or none), in cascade order (specificity, then source order)."""
    rules = []
    for st in root.iter():
        if not isinstance(st.tag, str) or _tag(st) != "style":
            continue
        if (st.get("type") or "text/css").strip() not in ("text/css", ""):
            continue
        text = re.sub(r"/\*.*?\*/", "", "".join(st.itertext()), flags=re.S)
        for sel, body in re.findall(r"([^{}@]+)\{([^}]*)\}", text):
            decls = []
            for d in body.split(";"):
                if ":" not in d:
                    continue
                k, v = d.split(":", 1)
                v = v.strip()
                imp = v.endswith("!important")
                if imp:
                    v = v[:-len("!important")].strip()
                if k.strip() in _CSS_NOT_PRESENTATION:
                    continue  # only presentation attributes come from style sheets
                decls.append((k.strip(), v, imp))
            for one in sel.split(","):
                parsed = _css_selector(one)
                if parsed is not None:
                    rules.append((parsed[1], len(rules), parsed[0], decls))
    if not rules:
        return {}
    parent = {c: p for p in root.iter() for c in p}

    def test(e, comp):
        for kind, v in comp:
            if kind == "type" and _tag(e) != v:
                return False
            if kind == "id" and e.get("id") != v:
                return False
            if kind == "class" and v not in (e.get("class") or "").split():
                return False
            if kind == "first":
                p = parent.get(e)
                if p is None or [c for c in p if isinstance(c.tag, str)][0] is not e:
                    return False
            if kind == "attr":
                name, op, val = v
                got = e.get(name)
                if got is None or (op == "=" and got != val) or (op == "~=" and val not in got.split()) or \
                        (op == "^=" and not got.startswith(val)) or (op == "$=" and not got.endswith(val)) or \
                        (op == "*=" and val not in got):
                    return False
        return True

    def match(e, parts):
        comp, comb = parts[0]
        if not test(e, comp):
            return False
        if len(parts) == 1:
            return True
        p = parent.get(e)
        if comb == ">":
            return p is not None and match(p, parts[1:])
        while p is not None:
            if match(p, parts[1:]):
                return True
            p = parent.get(p)
        return False
    out = {}
    for e in root.iter():
        if not isinstance(e.tag, str):
            continue
        hits = sorted((spec, order, decls) for spec, order, parts, decls in rules if match(e, parts))
        if hits:
            out[e] = [d for _, _, decls in hits for d in decls]
    return out


def struct_error():
    import struct
    return struct.error


def zlib_error():
    import zlib
    return zlib.error


def view_box_transform(vb, par, w, h):
    """usvg ViewBox::to_transform (utils.rs view_box_to_transform): the viewBox
    (x, y, w, h) fitted into a w x h viewport by preserveAspectRatio."""
    F = np.float32
    sx, sy = F(w) / F(vb[2]), F(h) / F(vb[3])
    parts = par.split()
    if parts and parts[0] == "defer":
        parts = parts[1:]
    align = parts[0] if parts else "xMidYMid"
    slice_ = len(parts) > 1 and parts[1] == "slice"
    if align == "none":
        return (float(sx), 0.0, 0.0, float(sy), float(-F(vb[0]) * sx), float(-F(vb[1]) * sy))
    sc = max(sx, sy) if slice_ else min(sx, sy)
    x, y = -F(vb[0]) * sc, -F(vb[1]) * sc
    nw, nh = F(vb[2]) * sc, F(vb[3]) * sc
    ax = align[1:4] if len(align) >= 8 else "Mid"
    ay = align[5:8] if len(align) >= 8 else "Mid"
    if ax == "Mid":
        x = x + (F(w) - nw) / F(2)
    elif ax == "Max":
        x = x + (F(w) - nw)
    if ay == "Mid":
        y = y + (F(h) - nh) / F(2)
    elif ay == "Max":
        y = y + (F(h) - nh)
    return (float(sc), 0.0, 0.0, float(sc), float(x), float(y))


def mat_mul(a, b):
    """a * b for (sx, ky, kx, sy, tx, ty) row-form transforms (f64)."""
    return (a[0] * b[0] + a[2] * b[1], a[1] * b[0] + a[3] * b[1],
            a[0] * b[2] + a[2] * b[3], a[1] * b[2] + a[3] * b[3],
            a[0] * b[4] + a[2] * b[5] + a[4], a[1] * b[4] + a[3] * b[5] + a[5])


IDENT = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)


def _f32(v):
    return float(np.float32(v))


def sk_concat(a, b):
    """tiny-skia Transform::concat(a, b) = a * b on f32 components: a scale
    and translate pair multiplies in f32, otherwise each entry is a sum of two
    products in f64 rounded once to f32, then the translation added in f32."""
    if a == IDENT:
        return b
    if b == IDENT:
        return a
    if a[1] == 0 and a[2] == 0 and b[1] == 0 and b[2] == 0:
        return (_f32(a[0] * b[0]), 0.0, 0.0, _f32(a[3] * b[3]),
                _f32(_f32(a[0] * b[4]) + a[4]), _f32(_f32(a[3] * b[5]) + a[5]))
    return (_f32(a[0] * b[0] + a[2] * b[1]), _f32(a[1] * b[0] + a[3] * b[1]),
            _f32(a[0] * b[2] + a[2] * b[3]), _f32(a[1] * b[2] + a[3] * b[3]),
            _f32(_f32(a[0] * b[4] + a[2] * b[5]) + a[4]), _f32(_f32(a[1] * b[4] + a[3] * b[5]) + a[5]))


def sk_rotate(deg):
    """tiny-skia Transform::from_rotate: degrees to radians and cos / sin in f32."""
    f = np.float32
    v = f(deg) * (f(math.pi) / f(180.0))
    c, s = float(np.cos(f(v))), float(np.sin(f(v)))
    return (c, s, -s, c, 0.0, 0.0)


def ulps_eq(a, b, ulps=4):
    """float-cmp approx_eq_ulps on f32: equal, or of one sign and at most
    `ulps` representable values apart."""
    a, b = np.float32(a), np.float32(b)
    if a == b:
        return True
    if np.signbit(a) != np.signbit(b):
        return False
    ia, ib = int(a.view(np.int32)), int(b.view(np.int32))
    return abs(ia - ib) <= ulps


def paint_order(v):
    """svgtypes PaintOrder: up to three of fill / stroke / markers, the missing
    ones appended in the default order (fill, stroke, markers); `normal`, an
    unknown word, a repeated word or trailing data give the default order."""
    default = ["fill", "stroke", "markers"]
    words = (v or "").split()
    if not words or len(words) > 3 or any(w not in default for w in words) or len(set(words)) != len(words):
        return default
    return words + [w for w in default if w not in words]


def parse_angle_deg(s):
    """svgtypes Angle in degrees: a number with an optional deg, grad, rad or
    turn unit; None when it does not parse."""
    m = re.fullmatch(r"\s*([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)(deg|grad|rad|turn)?\s*", s or "")
    if not m:
        return None
    v, unit = float(m.group(1)), m.group(2)
    if unit == "grad":
        return v * 180.0 / 200.0
    if unit == "rad":
        return math.degrees(v)
    if unit == "turn":
        return v * 360.0
    return v


# Attributes CSS cannot set: svgtree/parse.rs takes only presentation
# attributes from style sheets and style attributes (geometry and element
# attributes are left to the XML attributes)
NOT_PRESENTATION = {
    "x", "y", "width", "height", "r", "rx", "ry", "cx", "cy", "fx", "fy", "fr", "d", "points", "x1", "y1", "x2",
    "y2", "offset", "viewBox", "preserveAspectRatio", "gradientUnits", "gradientTransform", "spreadMethod",
    "patternUnits", "patternContentUnits", "patternTransform", "clipPathUnits", "maskUnits", "maskContentUnits",
    "filterUnits", "primitiveUnits", "refX", "refY", "markerWidth", "markerHeight", "markerUnits", "orient", "href",
    "id", "class", "pathLength"}

# switch.rs FEATURES: the SVG 1.1 feature strings usvg supports
SVG_FEATURES = {"http://www.w3.org/TR/SVG11/feature#" + f for f in (
    "SVGDOM-static", "SVG-static", "CoreAttribute", "Structure", "BasicStructure", "ContainerAttribute",
    "ConditionalProcessing", "Image", "Style", "Shape", "Text", "BasicText", "PaintAttribute",
    "BasicPaintAttribute", "OpacityAttribute", "GraphicsAttribute", "BasicGraphicsAttribute", "Marker", "Gradient",
    "Pattern", "Clip", "BasicClip", "Mask", "Filter", "BasicFilter", "XlinkAttribute")}
LANGUAGES = ("en",)  # usvg Options::languages default


def condition_passed(e):
    """switch.rs is_condition_passed: no requiredExtensions, every
    requiredFeatures string supported, and a systemLanguage entry equal to a
    user language or to one followed by '-'."""
    if e.get("requiredExtensions") is not None:
        return False
    rf = e.get("requiredFeatures")
    if rf is not None and any(f not in SVG_FEATURES for f in rf.split(" ")):
        return False
    sl = e.get("systemLanguage")
    if sl is not None:
        for lang in sl.split(","):
            lang = lang.strip()
            if lang in LANGUAGES:
                return True
            if "-" in lang and lang[:lang.index("-")] in LANGUAGES:
                return True
        return False
    return True


def parse_transform_origin(s):
    """svgtypes TransformOrigin (CSS transform-origin): one to three values,
    keywords (left / center / right, top / bottom) or lengths; a single value
    sets x (or y for top / bottom) with the other at center; a y keyword first
    swaps the pair; a third value (z) is ignored.  Returns the (x, y) lengths
    as strings, or None when the value does not parse."""
    toks = (s or "").replace(",", " ").split()
    if not 1 <= len(toks) <= 3:
        return None
    kw = {"left": "0%", "center": "50%", "right": "100%", "top": "0%", "bottom": "100%"}

    def ok(t):
        return t in kw or re.fullmatch(NUM + r"(px|%|em|ex|in|cm|mm|pt|pc)?", t) is not None
    if not all(ok(t) for t in toks[:2]):
        return None
    if len(toks) == 1:
        t = toks[0]
        return ("50%", kw[t]) if t in ("top", "bottom") else (kw.get(t, t), "50%")
    x, y = toks[0], toks[1]
    if x in ("top", "bottom") or y in ("left", "right"):
        x, y = y, x
    if x in ("top", "bottom") or y in ("left", "right"):
        return None
    return kw.get(x, x), kw.get(y, y)


def parse_transform(s):
    ts = IDENT
    for name, args in re.findall(r"(\w+)\s*\(([^)]*)\)", s or ""):
        v = numbers(args)
        if name == "matrix" and len(v) == 6:
            t = tuple(v)
        elif name == "translate":
            t = (1, 0, 0, 1, v[0], v[1] if len(v) > 1 else 0.0)
        elif name == "scale":
            t = (v[0], 0, 0, v[1] if len(v) > 1 else v[0], 0, 0)
        elif name == "rotate":
            a = math.radians(v[0])
            c, s_ = math.cos(a), math.sin(a)
            t = (c, s_, -s_, c, 0, 0)
            if len(v) == 3:
                t = mat_mul(mat_mul((1, 0, 0, 1, v[1], v[2]), t), (1, 0, 0, 1, -v[1], -v[2]))
        elif name == "skewX":
            t = (1, 0, math.tan(math.radians(v[0])), 1, 0, 0)
        elif name == "skewY":
            t = (1, math.tan(math.radians(v[0])), 0, 1, 0, 0)
        else:
            raise Unsupported("transform " + name)
        ts = mat_mul(ts, t)
    return ts


# ---------------------------------------------------------------- path data
class PathB:
    """tiny-skia PathBuilder semantics (f32 points, move_to after close)."""

    def __init__(self):
        self.verbs, self.pts = [], []
        self.move_req = True
        self.last_move = None

    def _f(self, v):
        return float(np.float32(v))

    def last(self):
        return self.pts[-1] if self.pts else None

    def move_to(self, x, y):
        x, y = self._f(x), self._f(y)
        if self.verbs and self.verbs[-1] == A.MOVE:
            self.pts[-1] = (x, y)
        else:
            self.verbs.append(A.MOVE)
            self.pts.append((x, y))
        self.last_move = (x, y)
        self.move_req = False

    def _inject(self):
        if self.move_req:
            p = self.last_move if self.last_move is not None else (0.0, 0.0)
            self.move_to(*p)

    def line_to(self, x, y):
        self._inject()
        self.verbs.append(A.LINE)
        self.pts.append((self._f(x), self._f(y)))

    def quad_to(self, x1, y1, x, y):
        self._inject()
        self.verbs.append(A.QUAD)
        self.pts += [(self._f(x1), self._f(y1)), (self._f(x), self._f(y))]

    def cubic_to(self, x1, y1, x2, y2, x, y):
        self._inject()
        self.verbs.append(A.CUBIC)
        self.pts += [(self._f(x1), self._f(y1)), (self._f(x2), self._f(y2)), (self._f(x), self._f(y))]

    def close(self):
        if self.verbs and self.verbs[-1] != A.CLOSE:
            self.verbs.append(A.CLOSE)
        self.move_req = True

    def arc_to(self, rx, ry, rot, large, sweep, x, y, prev=None):
        """usvg's PathBuilderExt::arc_to: kurbo arc -> cubics, or a line when
        the arc is degenerate.  `prev` overrides the start point (f64)."""
        if prev is None:
            prev = self.last()
        if prev is None:
            return
        cubics = svg_arc_to_cubics(prev, (x, y), rx, ry, rot, large, sweep)
        if cubics is None:
            self.line_to(x, y)
            return
        for c in cubics:
            self.cubic_to(*c)

    def finish(self):
        if len(self.verbs) <= 1:
            return None
        # drop a trailing move
        while self.verbs and self.verbs[-1] == A.MOVE:
            self.verbs.pop()
            self.pts.pop()
        if len(self.verbs) <= 1:
            return None
        return self.verbs, [c for p in self.pts for c in p]


def svg_arc_to_cubics(p0, p1, rx, ry, rot_deg, large, sweep, tol=0.1):
    """kurbo::Arc::from_svg_arc + to_cubic_beziers(0.1), in f64."""
    fx, fy = float(p0[0]), float(p0[1])
    tx, ty = float(p1[0]), float(p1[1])
    rx, ry = abs(float(rx)), abs(float(ry))
    if rx <= 1e-5 or ry <= 1e-5 or (fx == tx and fy == ty):
        return None  # SvgArc::is_straight_line: Arc::from_svg_arc gives None
    xr = math.radians(rot_deg) % (2 * math.pi)
    sp, cp = math.sin(xr), math.cos(xr)
    hdx, hdy = (fx - tx) * 0.5, (fy - ty) * 0.5
    hsx, hsy = (fx + tx) * 0.5, (fy + ty) * 0.5
    px = cp * hdx + sp * hdy
    py = -sp * hdx + cp * hdy
    rf = px * px / (rx * rx) + py * py / (ry * ry)
    if rf > 1.0:
        rx *= math.sqrt(rf)
        ry *= math.sqrt(rf)
    rxry = rx * ry
    rxpy = rx * py
    rypx = ry * px
    ssq = rxpy * rxpy + rypx * rypx
    coe = (-1.0 if large == sweep else 1.0) * math.sqrt(abs((rxry * rxry - ssq) / ssq))
    tcx = coe * rxpy / ry
    tcy = -coe * rypx / rx
    cx = cp * tcx - sp * tcy + hsx
    cy = sp * tcx + cp * tcy + hsy
    sa = math.atan2((py - tcy) / ry, (px - tcx) / rx)
    ea = math.atan2((-py - tcy) / ry, (-px - tcx) / rx)
    sweep_a = math.fmod(ea - sa, 2 * math.pi)
    if sweep and sweep_a < 0:
        sweep_a += 2 * math.pi
    elif not sweep and sweep_a > 0:
        sweep_a -= 2 * math.pi
    rot = math.radians(rot_deg)

    def sample(angle):
        u, v = rx * math.cos(angle), ry * math.sin(angle)
        s, c = math.sin(rot), math.cos(rot)
        return u * c - v * s, u * s + v * c

    sign = math.copysign(1.0, sweep_a)
    scaled_err = max(rx, ry) / tol
    n_err = max((1.1163 * scaled_err) ** (1.0 / 6.0), 3.999999)
    n = math.ceil(n_err * abs(sweep_a) * (1.0 / (2.0 * math.pi)))
    if n <= 0:
        return []
    step = sweep_a / n
    arm = (4.0 / 3.0) * abs(math.tan(step / 4.0)) * sign
    a0 = sa
    q0 = sample(a0)
    out = []
    for _ in range(int(n)):
        a1 = a0 + step
        d0 = sample(a0 + math.pi / 2)
        q3 = sample(a1)
        d1 = sample(a1 + math.pi / 2)
        p1 = (q0[0] + arm * d0[0], q0[1] + arm * d0[1])
        p2 = (q3[0] - arm * d1[0], q3[1] - arm * d1[1])
        out.append((cx + p1[0], cy + p1[1], cx + p2[0], cy + p2[1], cx + q3[0], cy + q3[1]))
        a0, q0 = a1, q3
    return out


def parse_path_data(d: str) -> PathB:
    """svgtypes SimplifyingPathParser semantics: absolute coordinates, H/V as
    lines, S/T as reflected curves, arcs as cubics."""
    # tokens up to the first character that is neither a command, a number,
    # whitespace nor a comma: svgtypes stops parsing there
    d = d or ""
    stop = re.search(r"[^MmLlHhVvCcSsQqTtAaZz0-9eE+\-.,\s]", d)
    toks = re.findall(r"[MmLlHhVvCcSsQqTtAaZz]|" + NUM, d[:stop.start()] if stop else d)
    b = PathB()
    i, cmd = 0, None
    cx = cy = sx = sy = 0.0
    last_ctrl = None  # (kind, x, y) of the previous curve's second control point
    first = True

    def nums(k):
        nonlocal i
        out = []
        for _ in range(k):
            if i >= len(toks) or re.match(r"[A-Za-z]", toks[i]):
                raise ValueError("missing number")
            out.append(float(toks[i]))
            i += 1
        return out

    while i < len(toks):
        t = toks[i]
        if re.match(r"[A-Za-z]", t):
            cmd = t
            i += 1
            if first and cmd not in "Mm":
                break
            first = False
            if cmd in "Zz":
                b.close()
                cx, cy = sx, sy
                last_ctrl = None
                continue
        elif cmd is None:
            break
        try:
            rel = cmd.islower()
            c = cmd.upper()
            if c == "M":
                x, y = nums(2)
                if rel:
                    x, y = cx + x, cy + y
                b.move_to(x, y)
                cx, cy, sx, sy = x, y, x, y
                cmd = "l" if rel else "L"
                last_ctrl = None
            elif c == "L":
                x, y = nums(2)
                if rel:
                    x, y = cx + x, cy + y
                b.line_to(x, y)
                cx, cy = x, y
                last_ctrl = None
            elif c == "H":
                (x,) = nums(1)
                if rel:
                    x = cx + x
                b.line_to(x, cy)
                cx = x
                last_ctrl = None
            elif c == "V":
                (y,) = nums(1)
                if rel:
                    y = cy + y
                b.line_to(cx, y)
                cy = y
                last_ctrl = None
            elif c == "C":
                x1, y1, x2, y2, x, y = nums(6)
                if rel:
                    x1, y1, x2, y2, x, y = cx + x1, cy + y1, cx + x2, cy + y2, cx + x, cy + y
                b.cubic_to(x1, y1, x2, y2, x, y)
                last_ctrl = ("C", x2, y2)
                cx, cy = x, y
            elif c == "S":
                x2, y2, x, y = nums(4)
                if rel:
                    x2, y2, x, y = cx + x2, cy + y2, cx + x, cy + y
                if last_ctrl and last_ctrl[0] == "C":
                    x1, y1 = 2 * cx - last_ctrl[1], 2 * cy - last_ctrl[2]
                else:
                    x1, y1 = cx, cy
                b.cubic_to(x1, y1, x2, y2, x, y)
                last_ctrl = ("C", x2, y2)
                cx, cy = x, y
            elif c == "Q":
                x1, y1, x, y = nums(4)
                if rel:
                    x1, y1, x, y = cx + x1, cy + y1, cx + x, cy + y
                b.quad_to(x1, y1, x, y)
                last_ctrl = ("Q", x1, y1)
                cx, cy = x, y
            elif c == "T":
                x, y = nums(2)
                if rel:
                    x, y = cx + x, cy + y
                if last_ctrl and last_ctrl[0] == "Q":
                    x1, y1 = 2 * cx - last_ctrl[1], 2 * cy - last_ctrl[2]
                else:
                    x1, y1 = cx, cy
                b.quad_to(x1, y1, x, y)
                last_ctrl = ("Q", x1, y1)
                cx, cy = x, y
            elif c == "A":
                rx, ry, rot = nums(3)
                # flags may be glued: "A5 5 0 01 10 10"
                flags = []
                while len(flags) < 2:
                    tok = toks[i]
                    if tok in ("0", "1"):
                        flags.append(tok == "1")
                        i += 1
                    elif re.match(r"[01]", tok):
                        flags.append(tok[0] == "1")
                        toks[i] = tok[1:]
                    else:
                        raise ValueError("bad arc flag")
                x, y = nums(2)
                if rel:
                    x, y = cx + x, cy + y
                b._inject()
                b.arc_to(rx, ry, rot, flags[0], flags[1], x, y, prev=(cx, cy))
                cx, cy = x, y
                last_ctrl = None
            else:
                break
        except (ValueError, IndexError):
            break
    return b


# ---------------------------------------------------------------- tight bounds (usvg compute_tight_bounds)
# ---------------------------------------------------------------- markers
def marker_segments(verbs, pts):
    """The path as usvg's marker code walks it (marker.rs:128-160): moves,
    lines, cubics (a quad raised to a cubic in f32) and closes; each segment
    ("M", p), ("L", p), ("C", p1, p2, p) or ("Z",)."""
    f = np.float32
    segs, k = [], 0
    prev = prev_move = (0.0, 0.0)
    for v in verbs:
        if v == A.MOVE:
            p = (pts[k], pts[k + 1])
            k += 2
            segs.append(("M", p))
            prev = prev_move = p
        elif v == A.LINE:
            p = (pts[k], pts[k + 1])
            k += 2
            segs.append(("L", p))
            prev = p
        elif v == A.QUAD:
            c, p = (pts[k], pts[k + 1]), (pts[k + 2], pts[k + 3])
            k += 4
            lift = lambda a, b: float(f(f(f(a) + f(f(b) * f(2.0))) / f(3.0)))  # noqa: E731
            segs.append(("C", (lift(prev[0], c[0]), lift(prev[1], c[1])), (lift(p[0], c[0]), lift(p[1], c[1])), p))
            prev = p
        elif v == A.CUBIC:
            c1, c2, p = (pts[k], pts[k + 1]), (pts[k + 2], pts[k + 3]), (pts[k + 4], pts[k + 5])
            k += 6
            segs.append(("C", c1, c2, p))
            prev = p
        else:
            segs.append(("Z",))
            prev = prev_move
    return segs


def _subpath_start(segs, idx):
    for i in range(idx - 1, -1, -1):
        if segs[i][0] == "M":
            return segs[i][1]
    return (0.0, 0.0)


def _prev_vertex(segs, idx):
    s = segs[idx - 1]
    return _subpath_start(segs, idx) if s[0] == "Z" else s[-1]


def _bisector_deg(x1, y1, x2, y2, x3, y3, x4, y4):
    """Direction halfway between the incoming (1->2) and outgoing (3->4)
    vectors, in degrees within [0, 360), computed in f32 (marker.rs calc_angle)."""
    f = np.float32
    two_pi = f(math.pi) * f(2.0)

    def norm(r):
        v = np.fmod(f(r), two_pi)
        return f(v + two_pi) if v < 0 else f(v)

    def vec(vx, vy):
        r = np.arctan2(f(vy), f(vx))
        return f(0.0) if np.isnan(r) else norm(r)
    a_in = vec(f(x2) - f(x1), f(y2) - f(y1))
    a_out = vec(f(x4) - f(x3), f(y4) - f(y3))
    d = f(f(a_out - a_in) * f(0.5))
    ang = f(a_in + d)
    if f(math.pi / 2) < abs(d):
        ang = f(ang - f(math.pi))
    return f(norm(ang) * f(57.29577951308232))


def _line_deg(x1, y1, x2, y2):
    return _bisector_deg(x1, y1, x2, y2, x1, y1, x2, y2)


def _curves_deg(px, py, cx1, cy1, x, y, cx2, cy2, nx, ny):
    if ulps_eq(cx1, x) and ulps_eq(cy1, y):
        return _bisector_deg(px, py, x, y, x, y, cx2, cy2)
    if ulps_eq(x, cx2) and ulps_eq(y, cy2):
        return _bisector_deg(cx1, cy1, x, y, x, y, nx, ny)
    return _bisector_deg(cx1, cy1, x, y, x, y, cx2, cy2)


def marker_vertex_angle(segs, idx):
    """The orient="auto" angle at vertex `idx` (marker.rs calc_vertex_angle):
    the first vertex follows the first segment, the last the last segment, a
    middle one bisects the incoming and outgoing tangents."""
    f = np.float32
    n = len(segs)
    if idx == 0:
        s1, s2 = segs[0], segs[1]
        if s1[0] == "M" and s2[0] == "L":
            return _line_deg(*s1[1], *s2[1])
        if s1[0] == "M" and s2[0] == "C":
            pm, p1, p = s1[1], s2[1], s2[3]
            if ulps_eq(pm[0], p1[0]) and ulps_eq(pm[1], p1[1]):
                return _line_deg(*pm, *p)
            return _line_deg(*pm, *p1)
        return f(0.0)
    if idx == n - 1:
        s1, s2 = segs[idx - 1], segs[idx]
        if s2[0] == "M":
            return f(0.0)
        if s2[0] == "L":
            return _line_deg(*_prev_vertex(segs, idx), *s2[1])
        if s2[0] == "C":
            p1, p2, p = s2[1], s2[2], s2[3]
            if ulps_eq(p2[0], p[0]) and ulps_eq(p2[1], p[1]):
                return _line_deg(*p1, *p)
            return _line_deg(*p2, *p)
        if s1[0] == "L":
            return _line_deg(*s1[1], *_subpath_start(segs, idx))
        if s1[0] == "C":
            nxt = _subpath_start(segs, idx)
            return _curves_deg(*_prev_vertex(segs, idx), *s1[2], *s1[3], *nxt, *nxt)
        return f(0.0)
    s1, s2 = segs[idx], segs[idx + 1]
    k1, k2 = s1[0], s2[0]
    if k1 == "M" and k2 == "L":
        return _line_deg(*s1[1], *s2[1])
    if k1 == "M" and k2 == "C":
        return _line_deg(*s1[1], *s2[1])
    if k1 == "L" and k2 == "L":
        pv = _prev_vertex(segs, idx)
        return _bisector_deg(*pv, *s1[1], *s1[1], *s2[1])
    if k1 == "C" and k2 == "C":
        return _curves_deg(*_prev_vertex(segs, idx), *s1[2], *s1[3], *s2[1], *s2[3])
    if k1 == "L" and k2 == "C":
        pv = _prev_vertex(segs, idx)
        return _curves_deg(*pv, *pv, *s1[1], *s2[1], *s2[3])
    if k1 == "C" and k2 == "L":
        return _curves_deg(*_prev_vertex(segs, idx), *s1[2], *s1[3], *s2[1], *s2[1])
    if k1 == "L" and k2 == "M":
        return _line_deg(*_prev_vertex(segs, idx), *s1[1])
    if k1 == "C" and k2 == "M":
        p2, p = s1[2], s1[3]
        if ulps_eq(p[0], p2[0]) and ulps_eq(p[1], p2[1]):
            return _line_deg(*_prev_vertex(segs, idx), *p)
        return _line_deg(*p2, *p)
    if k1 == "L" and k2 == "Z":
        pv, nx = _prev_vertex(segs, idx), _subpath_start(segs, idx)
        return _bisector_deg(*pv, *s1[1], *s1[1], *nx)
    if k2 == "Z" and k1 != "Z":
        return _line_deg(*_prev_vertex(segs, idx), *_subpath_start(segs, idx))
    return f(0.0)


def marker_vertices(segs, kind):
    """(point, vertex index) pairs a start / mid / end marker is drawn at
    (marker.rs draw_markers)."""
    if not segs:
        return []
    if kind == "start":
        return [(segs[0][1], 0)] if segs[0][0] == "M" else []
    if kind == "mid":
        return [(segs[i][-1], i) for i in range(1, len(segs) - 1) if segs[i][0] != "Z"]
    last = len(segs) - 1
    s = segs[last]
    if s[0] in ("L", "C"):
        return [(s[-1], last)]
    if s[0] == "Z":
        return [(_subpath_start(segs, last), last)]
    return []


def tight_bounds(verbs, pts):
    xs, ys = [], []
    P = [(pts[2 * k], pts[2 * k + 1]) for k in range(len(pts) // 2)]
    pi = 0
    last = None
    for v in verbs:
        if v == A.MOVE or v == A.LINE:
            last = P[pi]
            pi += 1
            xs.append(last[0])
            ys.append(last[1])
        elif v == A.QUAD:
            c, e = P[pi], P[pi + 1]
            pi += 2
            xs.append(e[0]); ys.append(e[1])
            for k in range(2):
                a, b_, cc = last[k], c[k], e[k]
                den = a - 2 * b_ + cc
                if den != 0:
                    t = (a - b_) / den
                    if 0 < t < 1:
                        m = 1 - t
                        q = (m * m * last[0] + 2 * m * t * c[0] + t * t * e[0], m * m * last[1] + 2 * m * t * c[1] + t * t * e[1])
                        xs.append(q[0]); ys.append(q[1])
            last = e
        elif v == A.CUBIC:
            c1, c2, e = P[pi], P[pi + 1], P[pi + 2]
            pi += 3
            xs.append(e[0]); ys.append(e[1])
            for k in range(2):
                p0, p1, p2, p3 = last[k], c1[k], c2[k], e[k]
                a = -p0 + 3 * p1 - 3 * p2 + p3
                b_ = 2 * (p0 - 2 * p1 + p2)
                cc = p1 - p0
                roots = []
                if abs(a) < 1e-12:
                    if b_ != 0:
                        roots.append(-cc / b_)
                else:
                    disc = b_ * b_ - 4 * a * cc
                    if disc >= 0:
                        sq = math.sqrt(disc)
                        roots += [(-b_ + sq) / (2 * a), (-b_ - sq) / (2 * a)]
                for t in roots:
                    if 0 < t < 1:
                        m = 1 - t
                        q = [m ** 3 * last[j] + 3 * m * m * t * c1[j] + 3 * m * t * t * c2[j] + t ** 3 * e[j] for j in range(2)]
                        xs.append(q[0]); ys.append(q[1])
            last = e
    if not xs:
        return None
    return min(xs), min(ys), max(xs), max(ys)


# ---------------------------------------------------------------- the loader
INHERITED = {"fill", "fill-opacity", "fill-rule", "stroke", "stroke-width", "stroke-opacity", "stroke-linecap",
             "stroke-linejoin", "stroke-miterlimit", "stroke-dasharray", "stroke-dashoffset", "visibility",
             "shape-rendering", "clip-rule", "color", "color-interpolation-filters", "paint-order", "font-size"}
NON_INHERITED = {"opacity", "clip-path", "mask", "filter", "mix-blend-mode", "isolation", "display",
                 "stop-color", "stop-opacity", "flood-color", "flood-opacity", "transform"}
UNSUPPORTED_ELEMS = {"text", "foreignObject", "tspan", "textPath",
                     "animate", "set"}
# usvg's element ids (svgtree/names.rs EId): any other element, or one of
# another namespace, is dropped with its children (svgtree/parse.rs
# parse_tag_name / parse_xml_node)
KNOWN_ELEMS = {
    "a", "circle", "clipPath", "defs", "ellipse", "feBlend", "feColorMatrix", "feComponentTransfer", "feComposite",
    "feConvolveMatrix", "feDiffuseLighting", "feDisplacementMap", "feDistantLight", "feDropShadow", "feFlood",
    "feFuncA", "feFuncB", "feFuncG", "feFuncR", "feGaussianBlur", "feImage", "feMerge", "feMergeNode",
    "feMorphology", "feOffset", "fePointLight", "feSpecularLighting", "feSpotLight", "feTile", "feTurbulence",
    "filter", "g", "image", "line", "linearGradient", "marker", "mask", "path", "pattern", "polygon", "polyline",
    "radialGradient", "rect", "stop", "style", "svg", "switch", "symbol", "text", "textPath", "tref", "tspan", "use"}
BLEND = {"normal": "source-over", "multiply": "multiply", "screen": "screen", "overlay": "overlay",
         "darken": "darken", "lighten": "lighten", "color-dodge": "color-dodge", "color-burn": "color-burn",
         "hard-light": "hard-light", "soft-light": "soft-light", "difference": "difference",
         "exclusion": "exclusion", "hue": "hue", "saturation": "saturation", "color": "color",
         "luminosity": "luminosity"}


F = np.float32


def _tag(e):
    t = e.tag
    return t[len(SVG_NS):] if t.startswith(SVG_NS) else t


class Loader:
    def __init__(self, text: str, tree_cls):
        self.root = ET.fromstring(text)
        self.css = stylesheet_rules(self.root)
        if _tag(self.root) != "svg":
            raise Unsupported("root is not svg")
        self.ids = {}
        for e in self.root.iter():
            i = e.get("id")
            if i is not None and i not in self.ids:
                self.ids[i] = e
        self.parent = {c: p for p in self.root.iter() for c in p}
        self.tree_cls = tree_cls
        # usvg's recursive-link fix for feImage: an element that a filter's
        # feImage links to drops its `filter` attribute when it, or an element
        # inside it, uses that same filter
        self.pattern_active = set()
        # usvg's fix_recursive_links (svgtree/parse.rs:776-810) for clip paths and
        # masks: inside element P (P included), a clip-path / mask linking to P,
        # or to an element with a link back to P inside it, reads as none;
        # repeated, in document order, until none is left
        self.no_link = set()

        def link_of(n, name):
            if (n, name) in self.no_link:
                return None
            v = self.attrs(n).get(name)
            m = re.match(r"\s*url\(\s*['\"]?#([^'\")\s]+)\s*['\"]?\s*\)", v or "")
            return self.ids.get(m.group(1)) if m else None
        for tag, name in (("clipPath", "clip-path"), ("mask", "mask")):
            nodes = [n for n in self.root.iter() if isinstance(n.tag, str) and _tag(n) == tag]
            for _ in range(10000):
                found = None
                for node in nodes:
                    for child in node.iter():
                        if not isinstance(child.tag, str):
                            continue
                        link = link_of(child, name)
                        if link is None:
                            continue
                        if link is node:
                            found = (child, name)
                        else:
                            for n2 in link.iter():
                                if isinstance(n2.tag, str) and link_of(n2, name) is node:
                                    found = (n2, name)
                                    break
                        if found:
                            break
                    if found:
                        break
                if not found:
                    break
                self.no_link.add(found)
        # usvg's recursive-pattern fix, in document order: inside pattern P, a
        # fill or stroke linking to P reads as none; one linking to pattern Q
        # stays, and the paints inside Q that link back to P read as none
        self.no_paint = set()

        def paint_link(n, which):
            if (n, which) in self.no_paint:
                return None
            v = self.attrs(n).get(which)
            m = re.match(r"\s*url\(\s*['\"]?#([^'\")\s]+)\s*['\"]?\s*\)", v or "")
            t = self.ids.get(m.group(1)) if m else None
            return t if t is not None and _tag(t) == "pattern" else None
        for pat in self.root.iter():
            if not isinstance(pat.tag, str) or _tag(pat) != "pattern":
                continue
            for n in pat.iter():
                if n is pat or not isinstance(n.tag, str):
                    continue
                for which in ("fill", "stroke"):
                    link = paint_link(n, which)
                    if link is None:
                        continue
                    if link is pat:
                        self.no_paint.add((n, which))
                        continue
                    for n2 in link.iter():
                        if not isinstance(n2.tag, str):
                            continue
                        for w2 in ("fill", "stroke"):
                            if paint_link(n2, w2) is pat:
                                self.no_paint.add((n2, w2))
        self.no_filter = set()
        for f in self.root.iter():
            if _tag(f) != "filter" or not f.get("id"):
                continue
            for c in f:
                if _tag(c) != "feImage":
                    continue
                href = (c.get(XLINK) or c.get("href") or "").strip()
                target = self.ids.get(href[1:]) if href.startswith("#") else None
                if target is None:
                    continue
                for n in target.iter():
                    if not isinstance(n.tag, str):
                        continue
                    fv = self.attrs(n).get("filter") or ""
                    if re.search(r"url\(\s*['\"]?#" + re.escape(f.get("id")) + r"['\"]?\s*\)", fv):
                        self.no_filter.add(n)
        for e in self.root.iter():
            if _tag(e) in UNSUPPORTED_ELEMS:
                raise Unsupported("element " + _tag(e))
        self.clip_cache, self.mask_cache, self.filter_cache = {}, {}, {}
        # markers being converted (a marker inside its own content is skipped;
        # nodes made for markers carry no id), and the (fill, stroke) that
        # context-fill / context-stroke resolve to: a solid paint index, None,
        # or "server" for a gradient or pattern
        self.marker_stack = []
        self.ctx = None
        self.use_size = (None, None)  # width / height of the <use> instancing an <svg>
        self.solid_ids = set()
        self.ids_out = {}  # SVG id -> the oracle's node id ("<group>" or "p<path>")

    # ---- attributes with style and inheritance
    def attrs(self, e):
        """Attributes with CSS applied, as usvg's svgtree does: presentation
        attributes, then matching <style> rules by specificity and order, then
        the style attribute, then `!important` rules."""
        a = dict(e.attrib)
        st = a.pop("style", None)
        important = {}
        # the `marker` shorthand sets marker-start, -mid and -end, in CSS only
        # (svgtree/parse.rs write_declaration); as an XML attribute it is ignored
        def put(d, k, v):
            for kk in (("marker-start", "marker-mid", "marker-end") if k == "marker" else (k,)):
                d[kk] = v
        for k, v, imp in self.css.get(e, ()):
            if k not in NOT_PRESENTATION:
                put(important if imp else a, k, v)
        if st:
            for part in re.sub(r"/\*.*?\*/", "", st, flags=re.S).split(";"):
                if ":" in part:
                    k, v = part.split(":", 1)
                    if k.strip() not in NOT_PRESENTATION:
                        put(a, k.strip(), v.strip())
        a.update(important)
        return a

    def get(self, e, name, inherited=True):
        a = self.attrs(e)
        if name in a and a[name].strip() != "inherit":
            return a[name]
        if inherited or (name in a and a[name].strip() == "inherit"):
            p = self.parent.get(e)
            hops = 0
            while p is not None and hops < 10000:
                hops += 1
                pa = self.attrs(p)
                if name in pa and pa[name].strip() != "inherit":
                    return pa[name]
                if not inherited:
                    break
                p = self.parent.get(p)
        return None

    def font_size(self, e):
        """The element's font size in user units: `font-size` resolved down its
        ancestors (em and % relative to the parent's size), 12 at the root."""
        chain = []
        n = e
        while n is not None and len(chain) < 10000:
            chain.append(n)
            n = self.parent.get(n)
        fs = 12.0
        for n in reversed(chain):
            v = self.attrs(n).get("font-size")
            if v is None or v.strip() == "inherit":
                continue
            v = v.strip()
            try:
                fs = fs * float(v[:-1]) / 100.0 if v.endswith("%") else parse_length(v, fs, fs)
            except (Unsupported, ValueError):
                pass  # named sizes and invalid values keep the inherited size
        return fs

    def num(self, e, name, default, ref=0.0):
        v = self.attrs(e).get(name)
        if v is None:
            return default
        return parse_length(v, ref, self.font_size(e))

    def href(self, e):
        h = e.get("href") or e.get(XLINK)  # SVG 2: href takes precedence
        if h and h.strip().startswith("#"):
            return self.ids.get(h.strip()[1:])
        return None

    def ref(self, value):
        if not value or value.strip() == "none":
            return None
        m = re.match(r"url\(\s*['\"]?#([^'\")\s]+)\s*['\"]?\s*\)", value.strip())
        if not m:
            return None  # not a link (e.g. a CSS shape function): svgtree reads no link
        return self.ids.get(m.group(1), "missing")



def _map_box(t, b):
    xs = [b[0], b[2], b[2], b[0]]
    ys = [b[1], b[1], b[3], b[3]]
    pts = [(t[0] * x + t[2] * y + t[4], t[1] * x + t[3] * y + t[5]) for x, y in zip(xs, ys)]
    return (min(p[0] for p in pts), min(p[1] for p in pts), max(p[0] for p in pts), max(p[1] for p in pts))


def _group(**kw):
    g = A.Group()
    g.transform = A.Transform.identity()
    g.opacity = 1.0
    g.blend = A.BLEND["source-over"]
    g.clip_path = -1
    g.mask = -1
    for k, v in kw.items():
        setattr(g, k, v)
    return g


def _tf(t):
    return A.Transform(*[float(np.float32(v)) for v in t])


class Builder(Loader):
    """Converts the SVG element tree into render-tree nodes."""

    def load(self):
        svg = self.root
        vb = numbers(svg.get("viewBox"))
        w, h = svg.get("width"), svg.get("height")
        if vb and len(vb) == 4:
            W = parse_length(w, vb[2]) if (w and not w.strip().endswith("%")) else vb[2]
            H = parse_length(h, vb[3]) if (h and not h.strip().endswith("%")) else vb[3]
            par = svg.get("preserveAspectRatio")
            if par in (None, "xMidYMid", "xMidYMid meet"):
                s = min(W / vb[2], H / vb[3])
                root_ts = (s, 0, 0, s, -vb[0] * s + (W - vb[2] * s) / 2, -vb[1] * s + (H - vb[3] * s) / 2)
            else:
                root_ts = view_box_transform(vb, par, W, H)
        else:
            W = parse_length(w, 100) if w else 100.0
            H = parse_length(h, 100) if h else 100.0
            root_ts = IDENT
        self.vbw, self.vbh = (vb[2], vb[3]) if vb and len(vb) == 4 else (W, H)
        self.W, self.H = W, H
        self.tree = self.tree_cls(W, H)
        root = self.tree.add_group(-1, _group())
        if root_ts != IDENT:
            root = self.tree.add_group(root, _group(transform=_tf(root_ts)))
        self.background(svg, root, vb if vb and len(vb) == 4 else (0.0, 0.0, W, H))
        # the root <svg> is a group of its own (opacity, clip-path, mask, filter,
        # display) inside the viewBox transform, as usvg converts it
        # converter.rs convert_doc: a root that is not visible (display:none or
        # failed conditions) leaves the tree empty
        if self.attrs(svg).get("display", "").strip() != "none" and condition_passed(svg):
            g = self.group_for(svg, root, IDENT)
            if g is not None:
                for c in svg:
                    self.node(c, g)
        self.tree.finalize()
        self.tree.ids = self.ids_out
        return self.tree

    def transform_of(self, e, attr="transform", value=None):
        """An element's transform with its transform-origin (converter.rs
        resolve_transform): translate(origin) . transform . translate(-origin),
        the origin's lengths and percentages in user space (percentages of the
        viewBox).  transform-origin is a presentation attribute but not
        inherited; one that does not parse is ignored."""
        ts = parse_transform(value if value is not None else (self.attrs(e).get(attr, "") or ""))
        o = self.own_attr(e, "transform-origin")
        if o is None:
            return ts
        xy = parse_transform_origin(o)
        if xy is None:
            return ts
        fsz = self.font_size(e)
        try:
            dx = parse_length(xy[0], self.vbw, fsz)
            dy = parse_length(xy[1], self.vbh, fsz)
        except (ValueError, Unsupported):
            return ts
        return mat_mul(mat_mul((1.0, 0.0, 0.0, 1.0, dx, dy), ts), (1.0, 0.0, 0.0, 1.0, -dx, -dy))

    def own_attr(self, e, name):
        """A non-inherited presentation attribute: from the element's style or
        attribute, not from its ancestors."""
        v = self.attrs(e).get(name)
        return v.strip() if isinstance(v, str) else None

    def background(self, svg, parent, rect):
        """usvg converter.rs:393-400 and 504-521: the root's non-standard
        background-color (a presentation attribute), when it parses as a plain
        colour, becomes a filled rect of the viewBox drawn before everything
        else, its alpha carried as the fill opacity."""
        v = self.attrs(svg).get("background-color")
        if v is None or v.strip().lower() in ("none", "currentcolor") or v.strip().startswith("url("):
            return
        try:
            c = parse_color(v)
        except InvalidColor:
            return
        if c is None:
            return
        path = A.Path()
        path.fill_paint = self.solid(c)
        path.fill_opacity = float(np.float32(round(c[1] * 255) / 255.0))
        path.fill_rule = A.NONZERO
        path.stroke_paint, path.stroke_width = -1, 1.0
        path.visible, path.anti_alias = 1, 1
        x, y, w, h = rect
        self.tree.add_path(parent, path, [A.MOVE, A.LINE, A.LINE, A.LINE, A.CLOSE],
                           [(x, y), (x + w, y), (x + w, y + h), (x, y + h)])

    def visible(self, e):
        """usvg is_visible_element: not display:none and the conditional
        attributes pass (switch.rs is_condition_passed)."""
        if self.attrs(e).get("display", "").strip() == "none":
            return False
        return condition_passed(e)

    def node(self, e, parent, transform_extra=IDENT):
        tag = _tag(e)
        if tag not in KNOWN_ELEMS:
            return
        if tag in ("defs", "linearGradient", "radialGradient", "clipPath", "mask", "filter", "title", "desc",
                   "metadata", "stop", "pattern", "style", "marker", "symbol"):
            return
        if not self.visible(e):
            return
        if tag not in ("g", "path", "rect", "circle", "ellipse", "line", "polyline", "polygon", "use", "svg", "a",
                       "image", "switch"):
            raise Unsupported("element " + tag)
        ts = self.transform_of(e)
        if transform_extra != IDENT:
            ts = mat_mul(transform_extra, ts)
        if tag == "image":
            self.image(e, parent, ts)
            return
        if tag == "use":
            ref = self.href(e)
            if ref is None or _tag(ref) not in KNOWN_ELEMS:
                return  # svgtree: a use linked to no SVG element is dropped
            x = self.num(e, "x", 0.0, self.vbw)
            y = self.num(e, "y", 0.0, self.vbh)
            if _tag(ref) == "symbol":
                self.use_symbol(e, ref, parent, ts, x, y)
                return
            ts = mat_mul(ts, (1, 0, 0, 1, x, y))
        g = self.group_for(e, parent, ts)
        if g is None:
            return
        if tag in ("g", "a"):
            for c in e:
                self.node(c, g)
        elif tag == "switch":
            # switch.rs: the first child element whose conditions pass
            for c in e:
                # unknown elements are not in usvg's tree, so never the chosen child
                if isinstance(c.tag, str) and _tag(c) in KNOWN_ELEMS and condition_passed(c):
                    self.node(c, g)
                    break
        elif tag == "use":
            # the instanced element inherits from the <use>, not from where it
            # is defined
            n = e
            while n is not None:  # a <use> inside what it references: not rendered
                if n is ref:
                    return
                n = self.parent.get(n)
            # use_node.rs convert: the <use> element's fill and stroke are the
            # context paints of what it instances
            ctx = (self.context_paint(e, "fill"), self.context_paint(e, "stroke"))
            saved, saved_ctx, saved_us = self.parent.get(ref), self.ctx, self.use_size
            if _tag(ref) == "svg":
                # use_node.rs: the <use>'s width / height, when given, replace
                # the referenced <svg>'s (each <use> resets both)
                self.use_size = (self.num(e, "width", None, self.vbw) if e.get("width") is not None else None,
                                 self.num(e, "height", None, self.vbh) if e.get("height") is not None else None)
            self.parent[ref] = e
            self.ctx = ctx
            try:
                self.node(ref, g)
            finally:
                self.ctx = saved_ctx
                self.use_size = saved_us
                if saved is None:
                    self.parent.pop(ref, None)
                else:
                    self.parent[ref] = saved
        elif tag == "svg":
            self.nested_svg(e, g)
        else:
            self.shape(e, g)

    def nested_svg(self, e, g):
        """A nested <svg> as usvg converts it (use_node.rs:163-211, 295-371): its
        content under translate(x, y) and the viewBox transform, in a new
        viewport for percentages, clipped to (x, y, width, height) unless
        overflow is visible / auto or width and height are not both given.
        Inside a <use>, the <use>'s width / height replace the element's, and
        then the clip applies even without the element's own width and height."""
        x, y = self.num(e, "x", 0.0, self.vbw), self.num(e, "y", 0.0, self.vbh)
        w, h = self.num(e, "width", self.vbw, self.vbw), self.num(e, "height", self.vbh, self.vbh)
        us = self.use_size
        w = us[0] if us[0] is not None else w
        h = us[1] if us[1] is not None else h
        vb = numbers(e.get("viewBox")) if e.get("viewBox") is not None else None
        if vb is not None and (len(vb) != 4 or not (vb[2] > 0 and vb[3] > 0)):
            vb = None
        new_ts = (1.0, 0.0, 0.0, 1.0, x, y)
        if vb is not None and w > 0 and h > 0:
            new_ts = mat_mul(new_ts, view_box_transform(vb, e.get("preserveAspectRatio") or "", w, h))
        new_vb = (vb[2], vb[3]) if vb is not None else ((w, h) if w > 0 and h > 0 else (self.vbw, self.vbh))
        ov = (self.attrs(e).get("overflow") or "").strip()
        parent = g
        sized = (e.get("width") is not None and e.get("height") is not None) or us != (None, None)
        if ov not in ("visible", "auto") and sized and w > 0 and h > 0 and math.isfinite(w) and math.isfinite(h):
            root = self.tree.add_group(-1, _group())
            self.rect_path(root, (x, y, w, h), self.solid(((0, 0, 0), 1.0)))
            c = A.Clip()
            c.transform = _tf(IDENT)
            c.clip_path = -1
            c.root = root
            parent = self.tree.add_group(g, _group(clip_path=self.tree.add_clip(c)))
        inner = self.tree.add_group(parent, _group(transform=_tf(new_ts)))
        saved = (self.vbw, self.vbh)
        self.vbw, self.vbh = new_vb
        try:
            for c in e:
                self.node(c, inner)
        finally:
            self.vbw, self.vbh = saved

    def use_symbol(self, e, sym, parent, ts_use, x, y):
        """<use> of a <symbol> as usvg converts it (use_node.rs convert,
        linked_to_symbol): percentages inside the symbol resolve against the
        <use>'s width / height when given; the symbol's content goes under
        translate(x, y) and the fit of the symbol's viewBox into the <use>'s
        size (100% by default); unless the symbol's overflow is visible / auto
        it is clipped to (x, y, width, height) of the <use>, in a group that
        carries the <use>'s transform, the <use>'s own group inside it without
        one; otherwise the <use>'s transform moves onto the symbol's group.
        The symbol's own transform attribute is not used."""
        n = e
        while n is not None:  # a <use> inside what it references: not rendered
            if n is sym:
                return
            n = self.parent.get(n)
        vbw, vbh = self.vbw, self.vbh
        nw = self.num(e, "width", vbw, vbw) if e.get("width") is not None else vbw
        nh = self.num(e, "height", vbh, vbh) if e.get("height") is not None else vbh
        if not (nw > 0 and nh > 0 and math.isfinite(nw) and math.isfinite(nh)):
            nw, nh = vbw, vbh
        ctx = (self.context_paint(e, "fill"), self.context_paint(e, "stroke"))
        saved_parent, saved_ctx = self.parent.get(sym), self.ctx
        self.vbw, self.vbh = nw, nh
        self.parent[sym] = e
        self.ctx = ctx
        try:
            uw, uh = self.num(e, "width", nw, nw), self.num(e, "height", nh, nh)
            new_ts = (1.0, 0.0, 0.0, 1.0, x, y)
            vb = numbers(sym.get("viewBox")) if sym.get("viewBox") is not None else None
            if vb is not None and (len(vb) != 4 or not (vb[2] > 0 and vb[3] > 0)):
                vb = None
            if vb is not None and uw > 0 and uh > 0:
                new_ts = mat_mul(new_ts, view_box_transform(vb, sym.get("preserveAspectRatio") or "", uw, uh))
            ov = (self.attrs(sym).get("overflow") or "").strip()
            if ov not in ("visible", "auto") and uw > 0 and uh > 0 and math.isfinite(uw) and math.isfinite(uh):
                cx, cy = self.num(e, "x", 0.0, nw), self.num(e, "y", 0.0, nh)
                root = self.tree.add_group(-1, _group())
                self.rect_path(root, (cx, cy, uw, uh), self.solid(((0, 0, 0), 1.0)))
                c = A.Clip()
                c.transform = _tf(IDENT)
                c.clip_path = -1
                c.root = root
                cg = self.tree.add_group(parent, _group(transform=_tf(ts_use), clip_path=self.tree.add_clip(c)))
                gu = self.group_for(e, cg, IDENT)
                sym_ts = new_ts
            else:
                gu = self.group_for(e, parent, IDENT)
                sym_ts = mat_mul(ts_use, new_ts)
            if gu is None:
                return
            gs = self.group_for(sym, gu, sym_ts)
            if gs is None:
                return
            for c in sym:
                self.node(c, gs)
        finally:
            self.vbw, self.vbh = vbw, vbh
            self.ctx = saved_ctx
            if saved_parent is None:
                self.parent.pop(sym, None)
            else:
                self.parent[sym] = saved_parent

    def group_for(self, e, parent, ts):
        """Creates the group an element needs (transform, opacity, clip, mask,
        filter, blend); returns the parent to add children to."""
        a = self.attrs(e)
        opacity = opacity_value(a.get("opacity"))
        opacity = max(0.0, min(1.0, opacity))
        clip = self.ref(a.get("clip-path") if (e, "clip-path") not in self.no_link else None)
        mask = self.ref(a.get("mask") if (e, "mask") not in self.no_link else None)
        filt = a.get("filter") if e not in self.no_filter else None
        # mix-blend-mode and isolation count only as CSS properties (style), not as
        # presentation attributes
        css = {}
        for part in re.sub(r"/\*.*?\*/", "", e.get("style") or "", flags=re.S).split(";"):
            if ":" in part:
                k, v = part.split(":", 1)
                css[k.strip()] = v.strip()
        # a value that is not a blend mode reads as normal (the attribute does not parse)
        blend = BLEND.get(css.get("mix-blend-mode", "normal").strip(), BLEND["normal"])
        isolate = css.get("isolation", "auto").strip() == "isolate"
        # svgtree drops a clip-path / mask attribute whose link has no element
        clip = None if clip == "missing" else clip
        mask = None if mask == "missing" else mask
        eid = e.get("id")
        if self.marker_stack:
            eid = None  # nodes made for markers carry no id
        keep_id = eid is not None and _tag(e) in ("g", "use")
        needs = ts != IDENT or opacity != 1.0 or clip is not None or mask is not None or filt or \
            blend != "source-over" or isolate or keep_id
        if not needs:
            return parent
        bbox = None
        has_filter = bool(filt and filt.strip() != "none")
        if clip is not None or mask is not None or has_filter:
            bbox = self.element_bbox(e)
        ci = mi = -1
        if clip is not None:
            ci = self.clip(clip, bbox)
            if ci is None:
                return None
        if mask is not None:
            mi = self.mask(mask, bbox)
            if mi is None:
                return None
        fids = []
        if has_filter:
            # parser/filter.rs convert: a list that does not parse is dropped
            # whole; urls that resolve to no filter only matter when nothing
            # else in the list made one (then the element is not rendered)
            invalid_url = False
            for fn in parse_filter_list(filt) or []:
                if fn[0] == "url":
                    fe = self.ids.get(fn[1])
                    fi = self.filter(fe, bbox) if fe is not None else None
                    if fi is None:
                        invalid_url = True
                    else:
                        fids.append(fi)
                else:
                    fi = self.filter_function(e, fn, bbox)
                    if fi is not None:
                        fids.append(fi)
            if not fids and invalid_url:
                return None
        g = _group(transform=_tf(ts), opacity=float(np.float32(opacity)), blend=A.BLEND[blend],
                   isolate=1 if isolate else 0, clip_path=ci, mask=mi)
        gi = self.tree.add_group(parent, g)
        if fids:
            self.tree.set_group_filters(gi, fids)
        if eid:
            self.ids_out.setdefault(eid, str(gi))
            self.tree.set_node_id(A.NODE_GROUP, gi, eid)
        return gi

    # ---- bounding boxes (object bounding box of an element, its user space)
    def element_bbox(self, e):
        tag = _tag(e)
        if tag in ("g", "a", "svg"):
            boxes = []
            for c in e:
                if _tag(c) in ("defs", "title", "desc") or not self.visible(c):
                    continue
                b = self.element_bbox(c)
                if b is None:
                    continue
                boxes.append(_map_box(self.transform_of(c), b))
            if not boxes:
                return None
            return (min(b[0] for b in boxes), min(b[1] for b in boxes), max(b[2] for b in boxes),
                    max(b[3] for b in boxes))
        if tag == "use":
            ref = self.href(e)
            if ref is None or _tag(ref) not in KNOWN_ELEMS:
                return None  # svgtree: a use linked to no SVG element is dropped
            b = self.element_bbox(ref)
            if b is None:
                return None
            t = self.transform_of(ref)
            t = mat_mul((1, 0, 0, 1, self.num(e, "x", 0.0, self.vbw), self.num(e, "y", 0.0, self.vbh)), t)
            return _map_box(t, b)
        geo = self.geometry(e)
        if geo is None:
            return None
        return tight_bounds(*geo)

    # ---- shapes
    def geometry(self, e):
        tag = _tag(e)
        a = self.attrs(e)
        fsz = self.font_size(e) if any(("em" in v or "ex" in v) for v in a.values()) else 12.0
        def L(n, d, ref):
            # an attribute that does not parse as a length is ignored (the default applies)
            if n not in a:
                return d
            try:
                return parse_length(a[n], ref, fsz)
            except InvalidLength:
                return d
        b = PathB()
        if tag == "path":
            b = parse_path_data(a.get("d", ""))
        elif tag == "rect":
            # usvg shapes.rs convert_rect: lengths and corner arithmetic in f32
            w, h = F(L("width", 0.0, self.vbw)), F(L("height", 0.0, self.vbh))
            if not (w > 0 and h > 0):
                return None
            x, y = F(L("x", 0.0, self.vbw)), F(L("y", 0.0, self.vbh))
            rx = L("rx", None, self.vbw) if "rx" in a else None
            ry = L("ry", None, self.vbh) if "ry" in a else None
            rx = None if (rx is not None and math.copysign(1.0, rx) < 0) else rx
            ry = None if (ry is not None and math.copysign(1.0, ry) < 0) else ry
            if rx is None and ry is None:
                rx = ry = 0.0
            elif rx is None:
                rx = ry
            elif ry is None:
                ry = rx
            rx, ry = F(rx), F(ry)
            two = F(2.0)
            if rx > w / two:
                rx = w / two
            if ry > h / two:
                ry = h / two
            if abs(int(np.float32(rx).view(np.int32))) <= 4:
                b.move_to(x, y); b.line_to(x + w, y); b.line_to(x + w, y + h); b.line_to(x, y + h); b.close()
            else:
                b.move_to(x + rx, y)
                b.line_to(x + w - rx, y)
                b.arc_to(rx, ry, 0, False, True, x + w, y + ry)
                b.line_to(x + w, y + h - ry)
                b.arc_to(rx, ry, 0, False, True, x + w - rx, y + h)
                b.line_to(x + rx, y + h)
                b.arc_to(rx, ry, 0, False, True, x, y + h - ry)
                b.line_to(x, y + ry)
                b.arc_to(rx, ry, 0, False, True, x + rx, y)
                b.close()
        elif tag in ("circle", "ellipse"):
            cx, cy = F(L("cx", 0.0, self.vbw)), F(L("cy", 0.0, self.vbh))
            if tag == "circle":
                r = L("r", 0.0, math.hypot(self.vbw, self.vbh) / math.sqrt(2))
                rx = ry = r
            else:
                rx = L("rx", None, self.vbw) if "rx" in a else None
                ry = L("ry", None, self.vbh) if "ry" in a else None
                rx = None if (rx is not None and math.copysign(1.0, rx) < 0) else rx
                ry = None if (ry is not None and math.copysign(1.0, ry) < 0) else ry
                if rx is None and ry is None:
                    return None
                rx = ry if rx is None else rx
                ry = rx if ry is None else ry
            rx, ry = F(rx), F(ry)
            if not (rx > 0 and ry > 0):
                return None
            b.move_to(cx + rx, cy)
            b.arc_to(rx, ry, 0, False, True, cx, cy + ry)
            b.arc_to(rx, ry, 0, False, True, cx - rx, cy)
            b.arc_to(rx, ry, 0, False, True, cx, cy - ry)
            b.arc_to(rx, ry, 0, False, True, cx + rx, cy)
            b.close()
        elif tag == "line":
            b.move_to(L("x1", 0.0, self.vbw), L("y1", 0.0, self.vbh))
            b.line_to(L("x2", 0.0, self.vbw), L("y2", 0.0, self.vbh))
        elif tag in ("polyline", "polygon"):
            v = numbers(a.get("points", ""))
            if len(v) % 2:
                v = v[:-1]
            if len(v) < 4:
                return None
            b.move_to(v[0], v[1])
            for k in range(2, len(v), 2):
                b.line_to(v[k], v[k + 1])
            if tag == "polygon":
                b.close()
        else:
            return None
        return b.finish()

    def paint(self, e, which, bbox, opacity_attr):
        if (e, which) in self.no_paint:
            return None
        v = self.get(e, which)
        if v is None:
            v = "black" if which == "fill" else "none"
        v = v.strip()
        cur = parse_color(self.get(e, "color") or "black")
        cur = cur[0] if cur else (0, 0, 0)
        op = self.get(e, opacity_attr)
        opacity = 1.0
        if op is not None:
            op = op.strip()
            opacity = float(op[:-1]) / 100 if op.endswith("%") else float(op)
        opacity = max(0.0, min(1.0, opacity))
        # style.rs convert_paint: an unparseable fill is black, an unparseable
        # stroke is none; a paint server that yields nothing uses the fallback
        def fallback_paint(fb):
            if not fb:
                return None
            try:
                c = parse_color(fb, cur)
            except InvalidColor:
                return None
            if c is None:
                return None
            return self.solid(c), opacity * c[1]
        invalid = (self.solid(((0, 0, 0), 1.0)), opacity) if which == "fill" else None
        if v in ("context-fill", "context-stroke"):
            # style.rs convert_paint: the context element's paint; its own
            # opacity is not carried over
            c = None if self.ctx is None else self.ctx[0 if v == "context-fill" else 1]
            if c is None:
                return None
            if c == "server":
                raise Unsupported("context paint server")
            return c, opacity
        if v.startswith("url("):
            m = re.match(r"url\(\s*['\"]?#([^'\")\s]+)\s*['\"]?\s*\)\s*(.*)$", v)
            if not m:
                return invalid
            ref = self.ids.get(m.group(1))
            fallback = m.group(2).strip()
            if fallback:
                try:
                    parse_color(fallback, cur)
                except InvalidColor:
                    return invalid  # the whole paint value fails to parse
            if ref is None:
                return fallback_paint(fallback)
            if _tag(ref) == "pattern":
                g = self.pattern(ref, bbox, opacity)
                if g == "drop":
                    return None  # usvg process_paint: obb units on a zero-sized shape drop the paint
                return g if g is not None else fallback_paint(fallback)
            if _tag(ref) not in ("linearGradient", "radialGradient"):
                return None
            g = self.gradient(ref, bbox, opacity)
            return g if g is not None else fallback_paint(fallback)
        try:
            c = parse_color(v, cur)
        except InvalidColor:
            return invalid
        if c is None:
            return None
        return self.solid(c), opacity * c[1]

    def pattern(self, ref, bbox, opacity):
        """A <pattern> as usvg converts it (parser/paint_server.rs:150-223) and
        resolves it to user space (:1007-1061): attributes through the href
        chain, content from the first pattern in it with children, the tile
        rect in patternUnits, the content under a group carrying the viewBox
        transform, or the bounding-box scale for objectBoundingBox content.
        None when the pattern yields nothing (the fallback applies), "drop"
        when bounding-box units meet a zero-sized shape."""
        chain, g, seen = [], ref, set()
        while g is not None and id(g) not in seen:
            if _tag(g) != "pattern":
                return None
            seen.add(id(g))
            chain.append(g)
            g = self.href(g)
        if id(ref) in self.pattern_active:
            return None  # a pattern drawn inside its own content
        content_src = next((c for c in chain if any(isinstance(k.tag, str) for k in c)), None)
        if content_src is None:
            return None

        def attr(name):
            for n in chain:
                v = n.get(name)
                if v is not None:
                    return v
            return None
        units = (attr("patternUnits") or "objectBoundingBox").strip()
        cunits = (attr("patternContentUnits") or "userSpaceOnUse").strip()
        obb = units != "userSpaceOnUse"
        cobb = cunits == "objectBoundingBox"
        pts = self.transform_of(ref, value=attr("patternTransform") or "")
        if abs(pts[0] * pts[3] - pts[1] * pts[2]) <= 0.0 or not all(math.isfinite(v) for v in pts):
            pts = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)  # a non-invertible patternTransform reads as none

        def num(name, ref_len):
            v = attr(name)
            if v is None:
                return 0.0
            v = v.strip()
            if obb:
                return float(v[:-1]) / 100 if v.endswith("%") else float(v)
            return parse_length(v, ref_len, self.font_size(ref))
        x, y = num("x", self.vbw), num("y", self.vbh)
        w, h = num("width", self.vbw), num("height", self.vbh)
        if not (w > 0 and h > 0):
            return None
        vb = numbers(attr("viewBox")) if attr("viewBox") is not None else None
        if vb is not None and (len(vb) != 4 or not (vb[2] > 0 and vb[3] > 0)):
            vb = None
        if obb or cobb:
            if bbox is None or not (bbox[2] > bbox[0] and bbox[3] > bbox[1]):
                return "drop"
        F32 = np.float32
        if obb:
            bw, bh = F32(bbox[2]) - F32(bbox[0]), F32(bbox[3]) - F32(bbox[1])
            x, y = float(F32(x) * bw + F32(bbox[0])), float(F32(y) * bh + F32(bbox[1]))
            w, h = float(F32(w) * bw), float(F32(h) * bh)
        wrap = None
        if vb is not None:
            wrap = view_box_transform(vb, attr("preserveAspectRatio") or "", w, h)
        elif cobb:
            wrap = (float(F32(bbox[2]) - F32(bbox[0])), 0.0, 0.0, float(F32(bbox[3]) - F32(bbox[1])), 0.0, 0.0)
        root = self.tree.add_group(-1, _group())
        content = self.tree.add_group(root, _group(transform=_tf(wrap))) if wrap is not None else root
        self.pattern_active.add(id(ref))
        try:
            for c in content_src:
                self.node(c, content)
        finally:
            self.pattern_active.discard(id(ref))
        p = A.Paint()
        p.kind = A.PAINT_PATTERN
        p.x1, p.y1, p.x2, p.y2 = x, y, w, h
        p.transform = _tf(pts)
        p.stop_offset = root
        return self.tree.add_paint(p, []), opacity

    def solid(self, c):
        p = A.Paint()
        p.kind = A.PAINT_SOLID
        p.r, p.g, p.b = c[0]
        p.transform = A.Transform.identity()
        i = self.tree.add_paint(p)
        self.solid_ids.add(i)
        return i

    def context_paint(self, e, which, width=None):
        """What an element hands to context-fill / context-stroke: its solid
        paint index, None, or "server" for a gradient or pattern (those are
        resolved against the context element's box, not supported here).  A
        stroke needs a positive stroke-width (style.rs resolve_stroke)."""
        if which == "stroke":
            if width is None:
                sw = self.get(e, "stroke-width")
                width = parse_length(sw, math.hypot(self.vbw, self.vbh) / math.sqrt(2), self.font_size(e)) \
                    if sw else 1.0
            if not width > 0:
                return None
        v = (self.get(e, which) or "").strip()
        if v.startswith("url("):
            m = re.match(r"url\(\s*['\"]?#([^'\")\s]+)\s*['\"]?\s*\)", v)
            ref = self.ids.get(m.group(1)) if m else None
            if ref is not None and _tag(ref) in ("linearGradient", "radialGradient", "pattern"):
                return "server"
        r = self.paint(e, which, None, which + "-opacity")
        if r is None:
            return None
        return r[0] if r[0] in self.solid_ids else "server"

    def grad_attr(self, e, name, chain):
        """usvg resolve_attr: the gradient attributes through the href chain;
        vector / circle attributes only from gradients of the same kind."""
        own = {"x1", "y1", "x2", "y2"} if _tag(e) == "linearGradient" else {"cx", "cy", "r", "fx", "fy", "fr"}
        for g in chain:
            if name in own and _tag(g) != _tag(e):
                continue
            v = g.get(name)
            if v is not None:
                return v
        return None

    def gradient(self, ref, bbox, opacity):
        chain, g = [], ref
        seen = set()
        while g is not None and id(g) not in seen and _tag(g) in ("linearGradient", "radialGradient"):
            seen.add(id(g))
            chain.append(g)
            g = self.href(g)
        stops_src = next((c for c in chain if any(_tag(s) == "stop" for s in c)), None)
        if stops_src is None:
            return None
        stops = []
        prev = 0.0
        for s in stops_src:
            if _tag(s) != "stop":
                continue
            sa = self.attrs(s)
            off = sa.get("offset")
            if off is None:
                o = prev
            else:
                off = off.strip()
                ov = number_strict(off[:-1] if off.endswith("%") else off)
                o = (ov / 100 if off.endswith("%") else ov) if ov is not None else 0.0
            prev = o
            o = max(0.0, min(1.0, o))
            col = sa.get("stop-color", "black")
            sop_v = sa.get("stop-opacity", "1")
            # `inherit` on these non-inherited properties takes the direct
            # parent's value, else the initial one (svgtree resolve_inherit)
            par = self.attrs(self.parent[s]) if self.parent.get(s) is not None else {}
            if col.strip() == "inherit":
                col = par.get("stop-color", "black")
                col = "black" if col.strip() == "inherit" else col
            if sop_v.strip() == "inherit":
                sop_v = par.get("stop-opacity", "1")
                sop_v = "1" if sop_v.strip() == "inherit" else sop_v
            # currentColor: the `color` the stop inherits through its ancestors
            cur_s = self.get(s, "color")
            cur_c = parse_color(cur_s) if cur_s is not None else None
            c = parse_color(col, cur_c[0] if cur_c else (0, 0, 0)) or ((0, 0, 0), 0.0)
            sop = sop_v.strip()
            sop = float(sop[:-1]) / 100 if sop.endswith("%") else float(sop)
            stops.append([float(np.float32(o)), c[0], c[1] * max(0.0, min(1.0, sop))])
        if not stops:
            return None
        # usvg stop normalisation (paint_server.rs:334-404)
        eps = float(np.finfo(np.float32).eps)

        def ulps_eq(a, b):
            return abs(np.float32(a).view(np.int32) - np.float32(b).view(np.int32)) <= 4 or a == b
        if len(stops) >= 3:
            i = 0
            while i < len(stops) - 2:
                if ulps_eq(stops[i][0], stops[i + 1][0]) and ulps_eq(stops[i + 1][0], stops[i + 2][0]):
                    stops.pop(i + 1)
                else:
                    i += 1
        if len(stops) >= 2:
            for i in range(len(stops) - 1):
                if ulps_eq(stops[i][0], 0.0) and ulps_eq(stops[i + 1][0], 0.0):
                    stops[i + 1][0] = float(np.float32(min(1.0, max(0.0, stops[i][0] + eps))))
        for i in range(1, len(stops)):
            o1, o2 = stops[i - 1][0], stops[i][0]
            if o1 > o2 or ulps_eq(o1, o2):
                stops[i - 1][0] = float(np.float32(min(1.0, max(0.0, o1 - eps))))
                stops[i][0] = o1
        units = self.grad_attr(ref, "gradientUnits", chain) or "objectBoundingBox"
        spread = {"pad": 0, "reflect": 1, "repeat": 2}.get((self.grad_attr(ref, "spreadMethod", chain) or "pad").strip(), 0)
        gts = self.transform_of(ref, value=self.grad_attr(ref, "gradientTransform", chain) or "")
        if abs(gts[0] * gts[3] - gts[1] * gts[2]) <= 0.0 or not all(math.isfinite(v) for v in gts):
            gts = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)  # a non-invertible gradientTransform reads as none
        p = A.Paint()
        p.spread = spread
        obb = units.strip() != "userSpaceOnUse"  # anything else is the default, objectBoundingBox
        if obb:
            if bbox is None or bbox[2] - bbox[0] <= 0 or bbox[3] - bbox[1] <= 0:
                return None
            bts = (bbox[2] - bbox[0], 0, 0, bbox[3] - bbox[1], bbox[0], bbox[1])
            gts = mat_mul(bts, gts)

        def ln(name, default, ref_len):
            v = self.grad_attr(ref, name, chain)
            if v is None:
                return default
            v = v.strip()
            if obb:
                return float(v[:-1]) / 100 if v.endswith("%") else float(v)
            return parse_length(v, ref_len)
        if _tag(ref) == "linearGradient":
            p.kind = A.PAINT_LINEAR
            p.x1 = ln("x1", 0.0, self.vbw)
            p.y1 = ln("y1", 0.0, self.vbh)
            p.x2 = ln("x2", 1.0 if obb else self.vbw, self.vbw)
            p.y2 = ln("y2", 0.0, self.vbh)
        else:
            p.kind = A.PAINT_RADIAL
            diag = math.hypot(self.vbw, self.vbh) / math.sqrt(2)
            p.cx = ln("cx", 0.5 if obb else self.vbw / 2, self.vbw)
            p.cy = ln("cy", 0.5 if obb else self.vbh / 2, self.vbh)
            p.r_ = ln("r", 0.5 if obb else diag / 2, diag)
            p.fx = ln("fx", p.cx, self.vbw)
            p.fy = ln("fy", p.cy, self.vbh)
            p.fr = max(ln("fr", 0.0, diag), 0.0)
            if not p.r_ > 0 and len(stops) >= 2:
                # paint_server.rs convert_radial: a non-positive r paints the last stop
                c = stops[-1]
                return self.solid((c[1], 1.0)), opacity * c[2]
            # The two-point conical constructor's concentric cases (Skia's
            # MakeTwoPointConical, kept by tiny-skia's RadialGradient::new): with
            # focus and centre within 2^-15 of each other, equal radii leave an
            # infinitely thin ring at r (Pad: the first colour inside it, the last
            # outside; a tiny r: the last colour), and a zero focal radius is a
            # plain radial gradient.
            tol = 1.0 / 32768.0
            f32 = np.float32
            if len(stops) >= 2 and abs(f32(p.fx) - f32(p.cx)) <= tol and abs(f32(p.fy) - f32(p.cy)) <= tol:
                if abs(f32(p.fr) - f32(p.r_)) <= tol:
                    if spread != 0:
                        raise Unsupported("degenerate concentric gradient with repeat/reflect")
                    if not f32(p.r_) > tol:
                        c = stops[-1]
                        return self.solid((c[1], 1.0)), opacity * c[2]
                    first, last = stops[0], stops[-1]
                    stops = [[0.0, first[1], first[2]], [1.0, first[1], first[2]], [1.0, last[1], last[2]]]
                    p.cx, p.cy, p.fr = p.fx, p.fy, 0.0
                elif abs(f32(p.fr)) <= tol:
                    p.cx, p.cy, p.fr = p.fx, p.fy, 0.0
        p.transform = _tf(gts)
        if len(stops) == 1:
            c = stops[0]
            return self.solid((c[1], 1.0)), opacity * c[2]
        st = []
        for o, c, a in stops:
            s = A.Stop()
            s.offset = o
            s.r, s.g, s.b = c
            s.opacity = float(np.float32(a))
            st.append(s)
        return self.tree.add_paint(p, st), opacity

    def shape(self, e, parent):
        geo = self.geometry(e)
        if geo is None:
            return
        verbs, pts = geo
        bbox = tight_bounds(verbs, pts)
        vis = (self.get(e, "visibility") or "visible").strip()
        path = A.Path()
        path.fill_paint = -1
        path.stroke_paint = -1
        path.visible = 1 if vis == "visible" else 0
        sr = (self.get(e, "shape-rendering") or "geometricPrecision").strip()
        path.anti_alias = 0 if sr in ("crispEdges", "optimizeSpeed") else 1
        order = paint_order(self.get(e, "paint-order"))
        # converter.rs svg_paint_order_to_usvg
        path.stroke_first = 1 if order[0] == "stroke" or order[:2] == ["markers", "stroke"] else 0
        fill = self.paint(e, "fill", bbox, "fill-opacity")
        if fill is not None:
            path.fill_paint, path.fill_opacity = fill[0], float(np.float32(fill[1]))
        path.fill_rule = A.EVENODD if (self.get(e, "fill-rule") or "nonzero").strip() == "evenodd" else A.NONZERO
        sw = self.get(e, "stroke-width")
        fsz = self.font_size(e)
        width = parse_length(sw, math.hypot(self.vbw, self.vbh) / math.sqrt(2), fsz) if sw else 1.0
        dashes = []
        if width > 0:
            stroke = self.paint(e, "stroke", bbox, "stroke-opacity")
            if stroke is not None:
                path.stroke_paint, path.stroke_opacity = stroke[0], float(np.float32(stroke[1]))
                path.stroke_width = float(np.float32(width))
                ml = self.get(e, "stroke-miterlimit")
                mlv = number_strict(ml) if ml else None
                path.miter_limit = max(mlv, 1.0) if mlv is not None else 4.0  # style.rs: below 1 reads as 1
                path.line_cap = {"butt": 0, "round": 1, "square": 2}.get((self.get(e, "stroke-linecap") or "butt").strip(), 0)
                path.line_join = {"miter": 0, "miter-clip": 1, "round": 2, "bevel": 3, "arcs": 0}.get(
                    (self.get(e, "stroke-linejoin") or "miter").strip(), 0)
                da = self.get(e, "stroke-dasharray")
                if da and da.strip() != "none":
                    dashes = [parse_length(x, self.vbw, fsz) for x in re.split(r"[\s,]+", da.strip()) if x]
                    if any(d < 0 for d in dashes) or sum(dashes) <= 0:
                        dashes = []
                    elif len(dashes) % 2:
                        dashes = dashes * 2
                    do = self.get(e, "stroke-dashoffset")
                    path.dash_phase = float(parse_length(do, self.vbw, fsz)) if do else 0.0
        links = self.marker_links(e) if vis == "visible" else []
        if path.fill_paint < 0 and path.stroke_paint < 0 and not links:
            return
        if path.stroke_paint < 0:
            path.stroke_width = 1.0

        def add(p, d, with_id):
            if p.fill_paint < 0 and p.stroke_paint < 0:
                return
            pi = self.tree.add_path(parent, p, verbs, pts, d)
            if with_id and e.get("id") and not self.marker_stack:
                self.ids_out.setdefault(e.get("id"), "p%d" % pi)
                self.tree.set_node_id(A.NODE_PATH, pi, e.get("id"))
        if not links:
            add(path, dashes, True)
            return

        def single(which):
            # converter.rs append_single_paint_path: one paint, no id
            p = A.Path.from_buffer_copy(path)
            if which == "fill":
                p.stroke_paint, p.stroke_width = -1, 1.0
                add(p, [], False)
            elif which == "stroke":
                p.fill_paint = -1
                add(p, dashes, False)

        def ctx_of(i):
            return None if i < 0 else (i if i in self.solid_ids else "server")
        ctx = (ctx_of(path.fill_paint), ctx_of(path.stroke_paint))

        def markers():
            mg = self.tree.add_group(parent, _group())
            segs = marker_segments(verbs, pts)
            for kind, m in links:
                self.marker(e, segs, m, kind, mg, ctx)
        # converter.rs convert_path: the marker group before, between or
        # after the painted path by paint-order
        if order[0] == "markers":
            markers()
            add(path, dashes, True)
        elif order[1] == "markers":
            single(order[0])
            markers()
            single(order[2])
        else:
            add(path, dashes, True)
            markers()

    def marker_links(self, e):
        """[(kind, <marker> element)] for marker-start, -mid and -end, skipping
        links to anything but a marker and markers already being drawn
        (marker.rs convert)."""
        out = []
        for kind in ("start", "mid", "end"):
            v = self.get(e, "marker-" + kind)
            if not v or v.strip() == "none":
                continue
            m = re.match(r"\s*url\(\s*['\"]?#([^'\")\s]+)\s*['\"]?\s*\)", v)
            ref = self.ids.get(m.group(1)) if m else None
            if ref is None or _tag(ref) != "marker" or any(ref is x for x in self.marker_stack):
                continue
            out.append((kind, ref))
        return out

    def marker(self, e, segs, m, kind, mg, ctx):
        """One marker-start / -mid / -end of a shape as usvg resolves it
        (marker.rs resolve): at every vertex of its kind a group under `mg`
        holding the marker's content, transformed by translate(vertex) .
        rotate(orient) . scale(the viewBox scale of the marker box, or the
        stroke scale) . translate(-refX, -refY), and clipped to the viewBox
        or marker box unless overflow is visible or auto."""
        f = np.float32
        a = self.attrs(m)
        if (m.get("markerUnits") or "").strip() == "userSpaceOnUse":
            scale = 1.0
        else:
            sw = self.get(e, "stroke-width")
            scale = parse_length(sw, math.hypot(self.vbw, self.vbh) / math.sqrt(2), self.font_size(e)) if sw else 1.0
        scale = _f32(scale)
        if not (scale > 0 and math.isfinite(scale)):
            return
        rx, ry = _f32(self.num(m, "refX", 0.0, self.vbw)), _f32(self.num(m, "refY", 0.0, self.vbh))
        mw, mh = _f32(self.num(m, "markerWidth", 3.0, self.vbw)), _f32(self.num(m, "markerHeight", 3.0, self.vbh))
        if not (mw > 0 and mh > 0 and math.isfinite(mw) and math.isfinite(mh)):
            return
        vb = numbers(m.get("viewBox")) if m.get("viewBox") is not None else None
        if vb is not None and (len(vb) != 4 or not (vb[2] > 0 and vb[3] > 0)):
            vb = None
        ov = a.get("overflow")
        ci = -1
        if ov is None or ov.strip() in ("hidden", "scroll"):
            root = self.tree.add_group(-1, _group())
            rect = tuple(_f32(v) for v in vb) if vb is not None else (0.0, 0.0, mw, mh)
            self.rect_path(root, rect, self.solid(((0, 0, 0), 1.0)))
            c = A.Clip()
            c.transform = _tf(IDENT)
            c.clip_path = -1
            c.root = root
            ci = self.tree.add_clip(c)
        orient = (m.get("orient") or "").strip()
        for p, idx in marker_vertices(segs, kind):
            ts = (1.0, 0.0, 0.0, 1.0, _f32(p[0]), _f32(p[1]))
            if orient == "auto-start-reverse" and idx == 0:
                ang = f(np.fmod(f(marker_vertex_angle(segs, idx) + f(180.0)), f(360.0)))
            elif orient in ("auto", "auto-start-reverse"):
                ang = marker_vertex_angle(segs, idx)
            else:
                d = parse_angle_deg(orient)
                ang = f(d) if d is not None else f(0.0)
            if not ulps_eq(ang, 0.0):
                ts = sk_concat(ts, sk_rotate(ang))
            if vb is not None:
                vt = view_box_transform(vb, m.get("preserveAspectRatio") or "", float(f(mw) * f(scale)),
                                        float(f(mh) * f(scale)))
                ts = sk_concat(ts, (abs(vt[0]), 0.0, 0.0, abs(vt[3]), 0.0, 0.0))
            else:
                ts = sk_concat(ts, (scale, 0.0, 0.0, scale, 0.0, 0.0))
            ts = sk_concat(ts, (1.0, 0.0, 0.0, 1.0, -rx, -ry))
            gi = self.tree.add_group(mg, _group(transform=_tf(ts), clip_path=ci))
            saved = self.ctx
            self.marker_stack.append(m)
            self.ctx = ctx
            try:
                for c in m:
                    self.node(c, gi)
            finally:
                self.marker_stack.pop()
                self.ctx = saved

    # ---- raster images
    def image(self, e, parent, ts):
        """<image> of a PNG data URL, as usvg converts it (parser/image.rs:110-264)
        and resvg draws it (image.rs:167-201): the decoded pixels, premultiplied
        like tiny-skia's decoder, fill the rect (0, 0, width, height) of a group
        whose transform fits that rect into the element's viewport by
        preserveAspectRatio (a clip to the viewport for `slice`); padded, and
        sampled nearest, bilinear or bicubic by image-rendering.  JPEG, GIF,
        WebP, SVG images and file references are not supported."""
        import base64
        from . import png
        href = (e.get(XLINK) or e.get("href") or "").strip()
        if not href.startswith("data:"):
            raise Unsupported("image file reference")
        head, _, payload = href.partition(",")
        if ";base64" not in head:
            raise Unsupported("image data URL encoding")
        try:
            data = base64.b64decode("".join(payload.split()))
        except ValueError:
            return
        mime = head[5:].split(";")[0].strip().lower()
        if mime in ("image/jpg", "image/jpeg", "image/gif", "image/webp", "image/svg+xml"):
            raise Unsupported("image " + mime)
        if mime != "image/png" and data[:8] != b"\x89PNG\r\n\x1a\n":
            raise Unsupported("image of an unknown type")
        try:
            rgba = png.decode_png(data)
        except (ValueError, KeyError, IndexError, struct_error(), zlib_error()):
            return
        if (self.get(e, "visibility") or "visible").strip() != "visible":
            return
        a = rgba[..., 3:4].astype(np.uint32)
        prod = rgba[..., :3].astype(np.uint32) * a + 128  # tiny-skia premultiply_u8
        rgba = np.concatenate([((prod + (prod >> 8)) >> 8).astype(np.uint8), rgba[..., 3:4]], axis=2)
        F = np.float32
        ah, aw = F(rgba.shape[0]), F(rgba.shape[1])
        x, y = F(self.num(e, "x", 0.0, self.vbw)), F(self.num(e, "y", 0.0, self.vbh))
        w, h = F(self.num(e, "width", float(aw), self.vbw)), F(self.num(e, "height", float(ah), self.vbh))
        has_w, has_h = e.get("width") is not None, e.get("height") is not None
        if has_w and not has_h:
            h = F(ah * F(w / aw))
        elif has_h and not has_w:
            w = F(aw * F(h / ah))
        if not (w > 0 and h > 0):
            return
        parts = (e.get("preserveAspectRatio") or "").split()
        if parts and parts[0] == "defer":
            parts = parts[1:]
        align = parts[0] if parts else "xMidYMid"
        slice_ = len(parts) > 1 and parts[1] == "slice"
        if align == "none":
            sw, sh = w, h
        else:
            # tiny-skia-path Size::scale_to / expand_to
            rw = F(F(h * aw) / ah)
            with_h = (rw <= w) if slice_ else (rw >= w)
            sw, sh = (rw, h) if not with_h else (w, F(F(w * ah) / aw))
        ox, oy = x, y
        if align != "none":
            ax, ay = align[1:4], align[5:8]
            dx, dy = F(w - sw), F(h - sh)
            ox = x + (F(dx / F(2)) if ax == "Mid" else (dx if ax == "Max" else F(0)))
            oy = y + (F(dy / F(2)) if ay == "Mid" else (dy if ay == "Max" else F(0)))
        image_ts = (float(F(sw / aw)), 0.0, 0.0, float(F(sh / ah)), float(F(ox)), float(F(oy)))
        mode = (self.get(e, "image-rendering") or "optimizeQuality").strip()
        quality = {"optimizeSpeed": A.IMAGE_NEAREST, "crisp-edges": A.IMAGE_NEAREST, "pixelated": A.IMAGE_NEAREST,
                   "smooth": A.IMAGE_BILINEAR}.get(mode, A.IMAGE_BICUBIC)
        g = self.group_for(e, parent, ts)
        if g is None:
            return
        if slice_ and align != "none":
            root = self.tree.add_group(-1, _group())
            self.rect_path(root, (float(x), float(y), float(w), float(h)), self.solid(((0, 0, 0), 1.0)))
            c = A.Clip()
            c.transform = _tf(IDENT)
            c.clip_path = -1
            c.root = root
            g = self.tree.add_group(g, _group(clip_path=self.tree.add_clip(c)))
        gi = self.tree.add_group(g, _group(transform=_tf(image_ts)))
        p = A.Paint()
        p.kind = A.PAINT_IMAGE
        p.stop_offset = self.tree.add_image(rgba)
        p.spread = quality
        p.transform = A.Transform.identity()
        self.rect_path(gi, (0.0, 0.0, float(aw), float(ah)), self.tree.add_paint(p, []))

    def rect_path(self, parent, r, paint):
        """A filled rect path (PathBuilder::from_rect) under `parent`."""
        x, y, w, h = r
        path = A.Path()
        path.fill_paint, path.fill_opacity, path.fill_rule = paint, 1.0, A.NONZERO
        path.stroke_paint, path.stroke_width = -1, 1.0
        path.visible, path.anti_alias = 1, 1
        self.tree.add_path(parent, path, [A.MOVE, A.LINE, A.LINE, A.LINE, A.CLOSE],
                           [(x, y), (x + w, y), (x + w, y + h), (x, y + h)])

    # ---- clip paths
    def clip(self, ce, bbox):
        if _tag(ce) != "clipPath":
            return None
        units = (ce.get("clipPathUnits") or "userSpaceOnUse").strip()
        ts = self.transform_of(ce, value=ce.get("transform", ""))
        if units == "objectBoundingBox":
            if bbox is None or bbox[2] <= bbox[0] or bbox[3] <= bbox[1]:
                return None
            ts = mat_mul(ts, (bbox[2] - bbox[0], 0, 0, bbox[3] - bbox[1], bbox[0], bbox[1]))
        root = self.tree.add_group(-1, _group())
        for c in ce:
            tag = _tag(c)
            if tag in ("title", "desc"):
                continue
            if tag == "text":
                raise Unsupported("clip child text")
            # converter.rs convert_clip_path_elements: only shapes and <use>
            # (of a shape) draw; <g>, <image>, <switch> and the rest are skipped
            if tag not in ("path", "rect", "circle", "ellipse", "line", "polyline", "polygon", "use"):
                continue
            self.clip_child(c, root)
        c = A.Clip()
        c.transform = _tf(ts)
        c.clip_path = -1
        c.root = root
        nested = self.ref(self.attrs(ce).get("clip-path") if (ce, "clip-path") not in self.no_link else None)
        if nested == "missing":
            return None
        if nested is not None:
            ni = self.clip(nested, bbox)
            if ni is None:
                return None
            c.clip_path = ni
        return self.tree.add_clip(c)

    def clip_child(self, e, root):
        if not self.visible(e):
            return
        a = self.attrs(e)
        ts = self.transform_of(e)
        target = e
        if _tag(e) == "use":
            target = self.href(e)
            if target is None or _tag(target) not in ("path", "rect", "circle", "ellipse", "line", "polyline",
                                                      "polygon"):
                if target is not None and _tag(target) == "text":
                    raise Unsupported("clip use of text")
                return  # a <use> of anything but a shape draws nothing in a clip path
            ts = mat_mul(ts, (1, 0, 0, 1, self.num(e, "x", 0.0, self.vbw), self.num(e, "y", 0.0, self.vbh)))
        parent = root
        cp = self.ref(a.get("clip-path") if (e, "clip-path") not in self.no_link else None)
        ci = -1
        if cp is not None:
            if cp == "missing":
                return
            ci = self.clip(cp, self.element_bbox(target))
            if ci is None:
                return
        if ts != IDENT or ci >= 0:
            parent = self.tree.add_group(root, _group(transform=_tf(ts), clip_path=ci))
        geo = self.geometry(target)
        if geo is None:
            return
        path = A.Path()
        path.fill_paint = self.solid(((0, 0, 0), 1.0))
        path.fill_opacity = 1.0
        path.stroke_paint = -1
        path.stroke_width = 1.0
        path.visible = 1 if (self.get(e, "visibility") or "visible").strip() == "visible" else 0
        sr = (self.get(target, "shape-rendering") or "geometricPrecision").strip()
        path.anti_alias = 0 if sr in ("crispEdges", "optimizeSpeed") else 1
        path.fill_rule = A.EVENODD if (self.get(e, "clip-rule") or "nonzero").strip() == "evenodd" else A.NONZERO
        self.tree.add_path(parent, path, geo[0], geo[1])

    # ---- masks
    def mask(self, me, bbox):
        if _tag(me) != "mask":
            return None
        units = (me.get("maskUnits") or "objectBoundingBox").strip()
        cunits = (me.get("maskContentUnits") or "userSpaceOnUse").strip()

        def fr(name, default):
            v = me.get(name)
            if v is None:
                return default
            v = v.strip()
            return float(v[:-1]) / 100 if v.endswith("%") else float(v)
        if units == "objectBoundingBox":
            if bbox is None or bbox[2] <= bbox[0] or bbox[3] <= bbox[1]:
                return None
            bw, bh = bbox[2] - bbox[0], bbox[3] - bbox[1]
            x = bbox[0] + fr("x", -0.1) * bw
            y = bbox[1] + fr("y", -0.1) * bh
            w = fr("width", 1.2) * bw
            h = fr("height", 1.2) * bh
        else:
            x = self.num(me, "x", -0.1 * self.vbw, self.vbw)
            y = self.num(me, "y", -0.1 * self.vbh, self.vbh)
            w = self.num(me, "width", 1.2 * self.vbw, self.vbw)
            h = self.num(me, "height", 1.2 * self.vbh, self.vbh)
        if not (w > 0 and h > 0):
            return None
        root = self.tree.add_group(-1, _group())
        content = root
        if cunits == "objectBoundingBox":
            if bbox is None:
                return None
            content = self.tree.add_group(root, _group(transform=_tf(
                (bbox[2] - bbox[0], 0, 0, bbox[3] - bbox[1], bbox[0], bbox[1]))))
        for c in me:
            self.node(c, content)
        m = A.Mask()
        m.x, m.y, m.w, m.h = x, y, w, h
        mt = (self.attrs(me).get("mask-type") or "luminance").strip()
        m.kind = A.MASK_ALPHA if mt == "alpha" else A.MASK_LUMINANCE
        m.mask = -1
        m.root = root
        nested = self.ref(self.attrs(me).get("mask") if (me, "mask") not in self.no_link else None)
        if nested == "missing":
            return None
        if nested is not None:
            ni = self.mask(nested, bbox)
            if ni is None:
                return None
            m.mask = ni
        return self.tree.add_mask(m)

    # ---- filters
    def convolve(self, c, p):
        """feConvolveMatrix as usvg converts it (parser/filter.rs:648-714);
        False where usvg substitutes a transparent flood."""
        ox, oy = 3, 3
        if c.get("order") is not None:
            v = numbers(c.get("order"))
            x = int(v[0]) if v else 3
            y = int(v[1]) if len(v) > 1 else x
            if x > 0 and y > 0:
                ox, oy = x, y
        m = [F(v) for v in numbers(c.get("kernelMatrix"))] if c.get("kernelMatrix") is not None else []
        if len(m) != ox * oy:
            m = []
        ksum = F(0)
        for v in m:
            ksum = F(ksum + v)
        r = F(ksum * F(1000000.0))
        r = F(np.sign(r) * np.floor(np.abs(r) + F(0.5))) if np.isfinite(r) else r
        ksum = F(r / F(1000000.0))
        if _approx_zero_ulps(ksum):
            ksum = F(1.0)
        divisor = F(float(c.get("divisor"))) if c.get("divisor") is not None else ksum
        if _approx_zero_ulps(divisor):
            return False
        bias = F(float(c.get("bias"))) if c.get("bias") is not None else F(0.0)

        def target(name, order):
            t = c.get(name)
            t = int(float(t)) if t is not None else int(np.floor(F(order) / F(2.0)))
            return t if 0 <= t < order else None
        tx, ty = target("targetX", ox), target("targetY", oy)
        if tx is None or ty is None or not m:
            return False
        if len(m) > len(p.f) - 2:
            raise Unsupported("convolve kernel larger than the primitive record")
        p.kind = A.FE_CONVOLVE
        edge = (c.get("edgeMode") or "duplicate").strip()
        p.i[0], p.i[1], p.i[2], p.i[3] = ox, oy, tx, ty
        p.i[4] = {"none": A.EDGE_NONE, "wrap": A.EDGE_WRAP}.get(edge, A.EDGE_DUPLICATE)
        p.i[5] = 1 if (c.get("preserveAlpha") or "false").strip() == "true" else 0
        p.f[0], p.f[1] = divisor, bias
        for k, v in enumerate(m):
            p.f[2 + k] = v
        return True

    def lighting(self, c, p, specular):
        """feDiffuseLighting / feSpecularLighting with their light source
        (parser/filter.rs:882-981); False where usvg substitutes a transparent flood."""
        light = None
        for n in c:
            if _tag(n) in ("feDistantLight", "fePointLight", "feSpotLight"):
                light = n
                break
        if light is None:
            return False

        def fa(e, name, default):
            v = e.get(name)
            return F(float(v)) if v is not None else F(default)
        if specular:
            se = fa(c, "specularExponent", 1.0)
            if not (1.0 <= se <= 128.0):
                return False
            p.kind = A.FE_SPECULAR
            p.f[0], p.f[1], p.f[2] = fa(c, "surfaceScale", 1.0), fa(c, "specularConstant", 1.0), se
        else:
            p.kind = A.FE_DIFFUSE
            p.f[0], p.f[1] = fa(c, "surfaceScale", 1.0), fa(c, "diffuseConstant", 1.0)
        lc = self.get(c, "lighting-color", inherited=False)
        col = (255, 255, 255)
        if lc is not None:
            if lc.strip().lower() == "currentcolor":
                cur = self.get(c, "color")
                pc = parse_color(cur) if cur is not None else None
                col = pc[0] if pc else (0, 0, 0)
            else:
                try:
                    pc = parse_color(lc)
                    col = pc[0] if pc else (255, 255, 255)
                except Exception:
                    col = (255, 255, 255)
        p.i[1], p.i[2], p.i[3] = col
        lt = _tag(light)
        if lt == "feDistantLight":
            p.i[0] = A.LIGHT_DISTANT
            p.f[4], p.f[5] = fa(light, "azimuth", 0.0), fa(light, "elevation", 0.0)
        elif lt == "fePointLight":
            p.i[0] = A.LIGHT_POINT
            p.f[4], p.f[5], p.f[6] = fa(light, "x", 0.0), fa(light, "y", 0.0), fa(light, "z", 0.0)
        else:
            p.i[0] = A.LIGHT_SPOT
            p.f[4], p.f[5], p.f[6] = fa(light, "x", 0.0), fa(light, "y", 0.0), fa(light, "z", 0.0)
            p.f[7], p.f[8], p.f[9] = fa(light, "pointsAtX", 0.0), fa(light, "pointsAtY", 0.0), fa(light, "pointsAtZ", 0.0)
            sx = fa(light, "specularExponent", 1.0)
            p.f[10] = sx if sx >= 0.0 else F(1.0)
            p.f[11] = fa(light, "limitingConeAngle", np.nan)
        return True

    def own_value(self, e, name):
        """A non-inherited attribute's value; `inherit` takes the direct
        parent's (svgtree/parse.rs resolve_inherit), None when it has none."""
        v = self.attrs(e).get(name)
        if v is not None and v.strip() == "inherit":
            p = self.parent.get(e)
            v = self.attrs(p).get(name) if p is not None else None
            if v is not None and v.strip() == "inherit":
                v = None
        return v

    def attr_color(self, e, name):
        """An element's own colour attribute as svgtypes parses it and usvg splits
        it: ((r, g, b), alpha) with the alpha stored as u8; black when absent or
        invalid."""
        v = self.own_value(e, name)
        try:
            c = parse_color(v) if v is not None and v.strip().lower() != "currentcolor" else None
        except (InvalidColor, Unsupported):
            c = None
        if c is None:
            return (0, 0, 0), 1.0
        return c[0], float(F(round(c[1] * 255.0)) / F(255.0))

    def component_transfer(self, c, p):
        """feComponentTransfer as usvg converts it (parser/filter.rs:570-622): per
        channel the last feFunc child with a known type; `tableValues` that do
        not parse give an empty table, which leaves the channel unchanged."""
        p.kind = A.FE_COMPONENT_TRANSFER
        chans = {"feFuncR": 0, "feFuncG": 1, "feFuncB": 2, "feFuncA": 3}
        for n in c:
            ch = chans.get(_tag(n))
            if ch is None:
                continue
            t = n.get("type")
            t = t.strip() if t is not None else None
            vals = []
            if t == "identity":
                kind = A.TF_IDENTITY
            elif t in ("table", "discrete"):
                kind = A.TF_TABLE if t == "table" else A.TF_DISCRETE
                vals = number_list_strict(n.get("tableValues")) if n.get("tableValues") is not None else []
                vals = vals or []
                if len(vals) > A.TF_MAX_VALUES:
                    raise Unsupported("component transfer table longer than the primitive record")
            elif t == "linear":
                kind = A.TF_LINEAR
                sl, ic = number_strict(n.get("slope")), number_strict(n.get("intercept"))
                vals = [sl if sl is not None else 1.0, ic if ic is not None else 0.0]
            elif t == "gamma":
                kind = A.TF_GAMMA
                am, ex, of = (number_strict(n.get(k)) for k in ("amplitude", "exponent", "offset"))
                vals = [am if am is not None else 1.0, ex if ex is not None else 1.0, of if of is not None else 0.0]
            else:
                continue
            p.i[ch] = kind
            p.i[4 + ch] = len(vals) if kind in (A.TF_TABLE, A.TF_DISCRETE) else 0
            for k in range(16):
                p.f[16 * ch + k] = vals[k] if k < len(vals) else 0.0

    def fe_image(self, c, p, fe, dummy):
        """feImage of an element (parser/filter.rs:821-852): the element converted
        under a detached group whose children the primitive renders.  No href
        or a missing element gives usvg's transparent stand-in; an image file
        or data URL is not supported.  Recursive links are cut when the
        document is read (no_filter)."""
        href = (c.get(XLINK) or c.get("href") or "").strip()
        if not href:
            dummy(p)
            return
        if not href.startswith("#"):
            raise Unsupported("feImage of an image")
        ref = self.ids.get(href[1:])
        if ref is None:
            dummy(p)
            return
        root = self.tree.add_group(-1, _group())
        self.node(ref, root)
        p.kind = A.FE_IMAGE
        p.i[0] = root

    def filter_function(self, e, fn, bbox):
        """One CSS filter function as usvg lowers it (parser/filter.rs:36-84 and
        :1088-1290): a filter of one sRGB primitive on SourceGraphic whose
        region is the element's bounding box grown to (-50%, -50%, 200%, 200%)
        for blur and drop-shadow, (-10%, -10%, 120%, 120%) for the others.
        None for an element without a bounding box."""
        if bbox is None or not (bbox[2] > bbox[0] and bbox[3] > bbox[1]):
            return None
        name, arg = fn
        p = A.Primitive()
        p.linear_rgb = 0
        p.in1, p.in2 = A.IN_SOURCE_GRAPHIC, A.IN_SOURCE_GRAPHIC
        one = F(1.0)

        def length(ln, horizontal):
            # units.rs convert_user_length with AId::Dx / AId::Dy
            v, u = F(ln[0]), ln[1]
            if u in ("", "px"):
                return v
            if u == "%":
                return F(F(F(self.vbw if horizontal else self.vbh) * v) / F(100.0))
            if u in ("em", "ex"):
                r = F(v * F(self.font_size(e)))
                return F(r / F(2.0)) if u == "ex" else r
            return F(F(v * F(96.0)) / F({"in": 1.0, "cm": 2.54, "mm": 25.4, "pt": 72.0, "pc": 6.0}[u]))

        def table(ch, vals):
            p.i[ch], p.i[4 + ch] = A.TF_TABLE, len(vals)
            for k, v in enumerate(vals):
                p.f[16 * ch + k] = float(v)

        def matrix(rows):
            p.kind = A.FE_COLOR_MATRIX
            p.i[0] = A.CM_MATRIX
            for k, v in enumerate(rows):
                p.f[k] = float(v)
        if name == "blur":
            p.kind = A.FE_BLUR
            sd = length(arg, True)
            p.f[0] = p.f[1] = float(sd) if sd >= 0 else 0.0
        elif name == "drop-shadow":
            p.kind = A.FE_DROP_SHADOW
            col, dx, dy, sd = arg
            if col is None:
                try:
                    col = parse_color(self.get(e, "color") or "black")
                except (InvalidColor, Unsupported):
                    col = None
                col = col or ((0, 0, 0), 1.0)
            p.i[0], p.i[1], p.i[2] = col[0]
            sd = length(sd, True)
            p.f[0] = p.f[1] = float(sd) if sd >= 0 else 0.0
            p.f[2], p.f[3] = float(length(dx, True)), float(length(dy, False))
            p.f[4] = float(F(round(col[1] * 255.0)) / F(255.0))
        elif name in ("brightness", "contrast"):
            p.kind = A.FE_COMPONENT_TRANSFER
            a = F(arg)
            icpt = F(0.0) if name == "brightness" else F(F(-F(F(0.5) * a)) + F(0.5))
            for ch in range(3):
                p.i[ch] = A.TF_LINEAR
                p.f[16 * ch], p.f[16 * ch + 1] = float(a), float(icpt)
        elif name == "invert":
            p.kind = A.FE_COMPONENT_TRANSFER
            a = F(min(arg, 1.0))
            for ch in range(3):
                table(ch, [a, F(one - a)])
        elif name == "opacity":
            p.kind = A.FE_COMPONENT_TRANSFER
            table(3, [F(0.0), F(min(arg, 1.0))])
        elif name in ("grayscale", "sepia"):
            a = F(min(arg, 1.0))
            r = F(one - a)
            if name == "grayscale":
                base = [(0.2126, 0.7874), (0.7152, -0.7152), (0.0722, -0.0722),
                        (0.2126, -0.2126), (0.7152, 0.2848), (0.0722, -0.0722),
                        (0.2126, -0.2126), (0.7152, -0.7152), (0.0722, 0.9278)]
            else:
                base = [(0.393, 0.607), (0.769, -0.769), (0.189, -0.189),
                        (0.349, -0.349), (0.686, 0.314), (0.168, -0.168),
                        (0.272, -0.272), (0.534, -0.534), (0.131, 0.869)]
            m = []
            for k, (b0, b1) in enumerate(base):
                t = F(F(abs(b1)) * r)
                m.append(F(F(b0) + t) if b1 > 0 else F(F(b0) - t))
                if k % 3 == 2:
                    m += [F(0.0), F(0.0)]
            matrix(m + [0.0, 0.0, 0.0, 1.0, 0.0])
        elif name == "saturate":
            p.kind = A.FE_COLOR_MATRIX
            p.i[0] = A.CM_SATURATE
            p.f[0] = float(max(F(arg), F(0.0)))
        elif name == "hue-rotate":
            p.kind = A.FE_COLOR_MATRIX
            p.i[0] = A.CM_HUE_ROTATE
            p.f[0] = float(F(arg))
        big = name in ("blur", "drop-shadow")
        rx, rw = (F(-0.5), F(2.0)) if big else (F(-0.1), F(1.2))
        bx, by = F(bbox[0]), F(bbox[1])
        bw, bh = F(F(bbox[2]) - bx), F(F(bbox[3]) - by)
        f = A.Filter()
        f.x, f.y = float(F(F(rx * bw) + bx)), float(F(F(rx * bh) + by))
        f.w, f.h = float(F(rw * bw)), float(F(rw * bh))
        p.x, p.y, p.w, p.h = f.x, f.y, f.w, f.h
        return self.tree.add_filter(f, [p], [])

    def filter(self, fe, bbox):
        if _tag(fe) != "filter":
            return None
        # parser/filter.rs convert_url: region attributes and units through the
        # xlink:href chain, primitives from the first filter in it with children
        chain, g, seen = [], fe, set()
        while g is not None and id(g) not in seen and _tag(g) == "filter":  # links to other elements end it
            seen.add(id(g))
            chain.append(g)
            g = self.href(g)
        if len(chain) > 1:
            merged = ET.Element(fe.tag, dict(fe.attrib))
            for name in ("x", "y", "width", "height", "filterUnits", "primitiveUnits"):
                if merged.get(name) is None:
                    v = next((n.get(name) for n in chain[1:] if n.get(name) is not None), None)
                    if v is not None:
                        merged.set(name, v)
            src = next((n for n in chain if any(isinstance(k.tag, str) for k in n)), None)
            if src is None:
                return None
            merged.extend(list(src))
            fe = merged
        units = (fe.get("filterUnits") or "objectBoundingBox").strip()
        punits = (fe.get("primitiveUnits") or "userSpaceOnUse").strip()
        pobb = punits == "objectBoundingBox"
        F32 = np.float32
        if pobb and (bbox is None or not (bbox[2] > bbox[0] and bbox[3] > bbox[1])):
            return None  # parser/filter.rs: primitive units on a zero-sized shape
        # parser/filter.rs:307-320: objectBoundingBox primitive units scale
        # lengths (std deviations, offsets, radii, displacement) by the bbox size
        sw, sh = (F32(F32(bbox[2]) - F32(bbox[0])), F32(F32(bbox[3]) - F32(bbox[1]))) if pobb else (F32(1), F32(1))

        def frac(v, default):
            if v is None:
                return F32(default)
            v = v.strip()
            return F32(float(v[:-1]) / 100) if v.endswith("%") else F32(float(v))

        def fr(e, name, default):
            v = e.get(name)
            if v is None:
                return default
            v = v.strip()
            return float(v[:-1]) / 100 if v.endswith("%") else float(v)
        if units == "objectBoundingBox":
            if bbox is None or bbox[2] <= bbox[0] or bbox[3] <= bbox[1]:
                return None
            bw, bh = bbox[2] - bbox[0], bbox[3] - bbox[1]
            x, y = bbox[0] + fr(fe, "x", -0.1) * bw, bbox[1] + fr(fe, "y", -0.1) * bh
            w, h = fr(fe, "width", 1.2) * bw, fr(fe, "height", 1.2) * bh
        else:
            x = self.num(fe, "x", -0.1 * self.vbw, self.vbw)
            y = self.num(fe, "y", -0.1 * self.vbh, self.vbh)
            w = self.num(fe, "width", 1.2 * self.vbw, self.vbw)
            h = self.num(fe, "height", 1.2 * self.vbh, self.vbh)
        if not (w > 0 and h > 0):
            return None
        prims, names, merge = [], {}, []
        for c in fe:
            tag = _tag(c)
            if tag in ("title", "desc"):
                continue
            p = A.Primitive()
            if pobb:
                # parser/filter.rs resolve_primitive_region: flood / image
                # subregions are fractions of the element's bbox; the others map
                # the filter region through the fractions (as usvg does)
                fx, fy = frac(c.get("x"), 0.0), frac(c.get("y"), 0.0)
                fw, fh = frac(c.get("width"), 1.0), frac(c.get("height"), 1.0)
                if not (fw > 0 and fh > 0):
                    break
                if tag in ("feFlood", "feImage"):
                    p.x, p.y = float(F32(fx * sw) + F32(bbox[0])), float(F32(fy * sh) + F32(bbox[1]))
                    p.w, p.h = float(F32(fw * sw)), float(F32(fh * sh))
                else:
                    p.x, p.y = float(F32(F32(x) * fw) + fx), float(F32(F32(y) * fh) + fy)
                    p.w, p.h = float(F32(F32(w) * fw)), float(F32(F32(h) * fh))
            else:
                p.x = self.num(c, "x", x, self.vbw) if c.get("x") is not None else x
                p.y = self.num(c, "y", y, self.vbh) if c.get("y") is not None else y
                p.w = self.num(c, "width", w, self.vbw) if c.get("width") is not None else w
                p.h = self.num(c, "height", h, self.vbh) if c.get("height") is not None else h
            cif = (self.get(c, "color-interpolation-filters") or "linearRGB").strip()
            p.linear_rgb = 0 if cif == "sRGB" else 1

            def inp(name, node=c):
                v = node.get(name)
                if v is None:
                    return len(prims) - 1 if prims else A.IN_SOURCE_GRAPHIC
                v = v.strip()
                if v == "SourceGraphic":
                    return A.IN_SOURCE_GRAPHIC
                if v == "SourceAlpha":
                    return A.IN_SOURCE_ALPHA
                if v in names:
                    return names[v]
                if v in ("BackgroundImage", "BackgroundAlpha", "FillPaint", "StrokePaint"):
                    return A.IN_SOURCE_GRAPHIC  # parser/filter.rs parse_in: not supported, SourceGraphic
                return len(prims) - 1 if prims else A.IN_SOURCE_GRAPHIC
            p.in1 = inp("in")

            def dummy(q):
                # usvg's stand-in for an invalid primitive: a transparent black flood
                q.kind = A.FE_FLOOD
                q.i[0] = q.i[1] = q.i[2] = 0
                q.f[0] = 0.0
            if tag == "feGaussianBlur":
                # parser/filter.rs convert_std_dev_attr: one or two numbers, else
                # 0 0; a negative component becomes 0
                p.kind = A.FE_BLUR
                sdx, sdy = std_dev_attr(c.get("stdDeviation", "0 0"))
                p.f[0], p.f[1] = float(F32(sdx) * sw), float(F32(sdy) * sh)
            elif tag == "feColorMatrix":
                p.kind = A.FE_COLOR_MATRIX
                t = (c.get("type") or "matrix").strip()
                vals = numbers(c.get("values", ""))
                has_vals = c.get("values") is not None
                identity = [1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0]
                # parser/filter.rs convert_color_matrix_kind: saturate and hueRotate
                # without `values` fall back to the identity matrix
                if t == "saturate" and has_vals:
                    p.i[0] = A.CM_SATURATE
                    p.f[0] = min(max(vals[0], 0.0), 1.0) if vals else 1.0
                elif t == "hueRotate" and has_vals:
                    p.i[0] = A.CM_HUE_ROTATE
                    p.f[0] = vals[0] if vals else 0.0
                elif t in ("saturate", "hueRotate"):
                    p.i[0] = A.CM_MATRIX
                    for k in range(20):
                        p.f[k] = identity[k]
                elif t == "luminanceToAlpha":
                    p.i[0] = A.CM_LUM_TO_ALPHA
                else:
                    p.i[0] = A.CM_MATRIX
                    if len(vals) != 20:
                        vals = [1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0]
                    for k in range(20):
                        p.f[k] = vals[k]
            elif tag == "feMorphology":
                p.kind = A.FE_MORPHOLOGY
                p.i[0] = 1 if (c.get("operator") or "erode").strip() == "dilate" else 0
                # parser/filter.rs convert_morphology: default 1 1; one or two
                # numbers (else 0 0); a zero component becomes 1; a negative one
                # keeps the default
                rx, ry = 1.0, 1.0
                if c.get("radius") is not None:
                    r = numbers(c.get("radius"))
                    a, b = (r[0], r[1]) if len(r) == 2 else ((r[0], r[0]) if len(r) == 1 else (0.0, 0.0))
                    if a == 0 and b == 0:
                        a = b = 1.0
                    if a == 0:
                        a = 1.0
                    if b == 0:
                        b = 1.0
                    if math.copysign(1.0, a) > 0 and math.copysign(1.0, b) > 0:
                        rx, ry = a, b
                p.f[0], p.f[1] = float(F32(rx) * sw), float(F32(ry) * sh)
            elif tag == "feComposite":
                p.kind = A.FE_COMPOSITE
                p.in2 = inp("in2")
                op = (c.get("operator") or "over").strip()
                p.i[0] = {"over": A.OP_OVER, "in": A.OP_IN, "out": A.OP_OUT, "atop": A.OP_ATOP, "xor": A.OP_XOR,
                          "arithmetic": A.OP_ARITHMETIC}.get(op, A.OP_OVER)
                for k, n in enumerate(("k1", "k2", "k3", "k4")):
                    p.f[k] = float(c.get(n, "0"))
            elif tag == "feFlood":
                p.kind = A.FE_FLOOD
                col = parse_color(self.own_value(c, "flood-color") or "black") or ((0, 0, 0), 0.0)
                p.i[0], p.i[1], p.i[2] = col[0]
                fo = (self.own_value(c, "flood-opacity") or "1").strip()
                fo = float(fo[:-1]) / 100 if fo.endswith("%") else float(fo)
                p.f[0] = max(0.0, min(1.0, fo)) * col[1]
            elif tag == "feOffset":
                p.kind = A.FE_OFFSET
                dx, dy = number_strict(c.get("dx")), number_strict(c.get("dy"))
                p.f[0] = float(F32(dx if dx is not None else 0.0) * sw)
                p.f[1] = float(F32(dy if dy is not None else 0.0) * sh)
            elif tag == "feComponentTransfer":
                self.component_transfer(c, p)
            elif tag == "feImage":
                self.fe_image(c, p, fe, dummy)
            elif tag == "feTile":
                p.kind = A.FE_TILE
            elif tag == "feDisplacementMap":
                # parser/filter.rs convert_displacement_map
                p.kind = A.FE_DISPLACEMENT_MAP
                p.in2 = inp("in2")
                ch = {"R": 0, "G": 1, "B": 2}
                p.i[0] = ch.get(c.get("xChannelSelector"), 3)
                p.i[1] = ch.get(c.get("yChannelSelector"), 3)
                sc = number_strict(c.get("scale"))
                p.f[0] = float(F32(sc if sc is not None else 0.0) * F32(F32(sw + sh) / F32(2)))
            elif tag == "feTurbulence":
                # parser/filter.rs convert_turbulence
                p.kind = A.FE_TURBULENCE
                bf = number_list_strict(c.get("baseFrequency")) if c.get("baseFrequency") is not None else None
                fx = fy = 0.0
                if bf is not None and len(bf) in (1, 2):
                    bx, by = F(bf[0]), F(bf[-1])
                    if math.copysign(1.0, bx) > 0 and math.copysign(1.0, by) > 0:
                        fx, fy = float(bx), float(by)
                p.f[0], p.f[1] = fx, fy
                no = number_strict(c.get("numOctaves"))
                no = F(no) if no is not None else F(1.0)
                if math.copysign(1.0, no) < 0:
                    no = F(0.0)
                no = math.floor(no + 0.5)  # f32::round (half away from zero), non-negative here
                if no > A.TURB_MAX_OCTAVES:
                    raise Unsupported("numOctaves above the device limit")
                p.i[0] = int(no)
                sd = number_strict(c.get("seed"))
                sd = math.trunc(float(F(sd))) if sd is not None and math.isfinite(F(sd)) else 0
                p.i[1] = max(-2 ** 31, min(2 ** 31 - 1, sd))
                p.i[2] = 1 if c.get("stitchTiles") == "stitch" else 0
                p.i[3] = 1 if c.get("type") == "fractalNoise" else 0
            elif tag == "feDropShadow":
                # parser/filter.rs convert_drop_shadow: stdDeviation "2 2", dx and dy
                # numbers (default 2), flood colour and opacity as feFlood
                p.kind = A.FE_DROP_SHADOW
                sdx, sdy = std_dev_attr(c.get("stdDeviation", "2 2"))
                p.f[0], p.f[1] = float(F32(sdx) * sw), float(F32(sdy) * sh)
                dx, dy = number_strict(c.get("dx")), number_strict(c.get("dy"))
                p.f[2] = float(F32(dx if dx is not None else 2.0) * sw)
                p.f[3] = float(F32(dy if dy is not None else 2.0) * sh)
                rgb, alpha = self.attr_color(c, "flood-color")
                p.i[0], p.i[1], p.i[2] = rgb
                p.f[4] = float(F(alpha) * F(opacity_value(self.attrs(c).get("flood-opacity"))))
            elif tag == "feMerge":
                p.kind = A.FE_MERGE
                ins = []
                for n in c:
                    if _tag(n) == "feMergeNode":
                        ins.append(inp("in", n))
                p.i[0], p.i[1] = len(merge), len(ins)
                merge += ins
            elif tag == "feBlend":
                p.kind = A.FE_BLEND
                p.in2 = inp("in2")
                p.i[0] = A.BLEND[BLEND.get((c.get("mode") or "normal").strip(), "source-over")]
            elif tag == "feConvolveMatrix":
                if not self.convolve(c, p):
                    dummy(p)
            elif tag in ("feDiffuseLighting", "feSpecularLighting"):
                if not self.lighting(c, p, tag == "feSpecularLighting"):
                    dummy(p)
            else:
                raise Unsupported("filter primitive " + tag)
            res = c.get("result")
            if res:
                names[res] = len(prims)
            prims.append(p)
        if not prims:
            return None
        f = A.Filter()
        f.x, f.y, f.w, f.h = x, y, w, h
        return self.tree.add_filter(f, prims, merge)


def load_svg(text: str, tree_cls=None):
    """Parses SVG text into a render tree (resvg_gb300.Tree)."""
    if tree_cls is None:
        from . import Tree as tree_cls
    return Builder(text, tree_cls).load()
