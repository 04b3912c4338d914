"""Pins the oracle against resvg's own golden images.

For every test of resvg's integration suite (crates/resvg/tests/tests/**.svg
with its .png) in the categories this backend covers, the SVG is loaded with
the SVG-subset front end (resvg_gb300.svg), rendered by the oracle exactly the
way the suite renders it (crates/resvg/tests/integration/main.rs:52-110:
the tree size rounded, scaled to width 300, a scale transform, demultiplied in
f64), and compared with the golden PNG using the suite's own rule
(main.rs:148-220: a pixel differs when any channel differs by more than 1,
pixels transparent in both images never differ).  A test passes when no
pixel differs.

Usage:  python tests/golden/pin_oracle.py <resvg checkout> [--write] [--verbose] [--only=<substring>]
  --write  rewrites tests/golden/oracle_pin.json (the committed summary) and
           tests/golden/fixtures.npz: for up to FIXTURES_PER_DIR passing tests
           per test directory, the SVG text and the golden image (demultiplied
           RGBA8), both zlib-compressed.  tests/test_oracle_golden.py replays
           them on the oracle (CPU) and tests/test_gpu_golden.py on the GPU.
  --extra-nodes  writes tests/golden/extra_nodes.npz: the render_node cases of
           crates/resvg/tests/integration/extra.rs (an SVG, the SVG id rendered,
           the golden image), replayed by id through the C ABI in
           tests/test_gpu_render_node.py.
"""
from __future__ import annotations

import json
import math
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from resvg_gb300 import png, svg  # noqa: E402

CATEGORIES = [
    "shapes", "painting/fill", "painting/fill-opacity", "painting/fill-rule", "painting/stroke",
    "painting/stroke-dasharray", "painting/stroke-dashoffset", "painting/stroke-linecap",
    "painting/stroke-linejoin", "painting/stroke-miterlimit", "painting/stroke-opacity",
    "painting/stroke-width", "painting/opacity", "painting/mix-blend-mode", "painting/isolation",
    "painting/paint-order", "painting/shape-rendering", "painting/visibility", "painting/display",
    "painting/color", "paint-servers/linearGradient", "paint-servers/radialGradient",
    "paint-servers/stop", "paint-servers/stop-color", "paint-servers/stop-opacity",
    "masking/clipPath", "masking/clip-rule", "masking/mask", "structure/g", "structure/use",
    "structure/transform", "structure/style", "structure/svg",
    "filters/feGaussianBlur", "filters/feColorMatrix", "filters/feMorphology", "filters/feComposite",
    "filters/feFlood", "filters/feOffset", "filters/feMerge", "filters/feBlend", "filters/filter",
    "filters/feConvolveMatrix", "filters/feDiffuseLighting", "filters/feSpecularLighting",
    "filters/feDistantLight", "filters/fePointLight", "filters/feSpotLight",
    "filters/filter-functions", "filters/feComponentTransfer", "filters/feDropShadow",
    "filters/feTurbulence", "filters/feTile", "filters/feDisplacementMap", "filters/feImage",
    "paint-servers/pattern", "structure/image", "painting/marker", "painting/context", "structure/symbol",
    "structure/transform-origin", "filters/enable-background", "structure/switch", "structure/systemLanguage",
    "filters/flood-color", "filters/flood-opacity", "structure/defs", "painting/overflow", "structure/a",
    "painting/image-rendering", "structure/style-attribute", "masking/clip",
]
IMAGE_SIZE = 300
FIXTURES_PER_DIR = 4


def render_size(tw, th):
    """tiny-skia Size::to_int_size then IntSize::scale_to_width(300)."""
    iw = max(1, int(round_half_away(tw)))
    ih = max(1, int(round_half_away(th)))
    nh = math.ceil(np.float32(IMAGE_SIZE) * np.float32(ih) / np.float32(iw))
    return IMAGE_SIZE, int(nh)


def round_half_away(v):
    return math.floor(v + 0.5) if v >= 0 else -math.floor(-v + 0.5)


def pixel_diff(expected, actual):
    """The suite's diff count (images of equal size)."""
    if expected.shape != actual.shape:
        return max(expected.shape[0], actual.shape[0]) * max(expected.shape[1], actual.shape[1])
    both_clear = (expected[..., 3] == 0) & (actual[..., 3] == 0)
    d = np.abs(expected.astype(np.int16) - actual.astype(np.int16)).max(axis=2) > 1
    return int((d & ~both_clear).sum())


def collect(root):
    """The suite's tests in CATEGORIES: an SVG with its golden PNG that
    crates/resvg/tests/integration/render.rs runs (a few files in the tree,
    e.g. structure/svg/no-size, have no test there and are left out)."""
    import re
    base = os.path.join(root, "crates", "resvg", "tests", "tests")
    listed = None
    rs = os.path.join(root, "crates", "resvg", "tests", "integration", "render.rs")
    if os.path.exists(rs):
        listed = set(re.findall(r'render\("tests/([^"]+)"\)', open(rs).read()))
    out = []
    for cat in CATEGORIES:
        top = os.path.join(base, cat)
        for d, _, files in sorted(os.walk(top)):
            sub = os.path.relpath(d, base)
            for name in sorted(files):
                if name.endswith(".svg") and os.path.exists(os.path.join(d, name[:-4] + ".png")):
                    if listed is not None and f"{sub}/{name[:-4]}" not in listed:
                        continue
                    out.append((sub, name[:-4], os.path.join(d, name)))
    return out


def collect_extra(root):
    """crates/resvg/tests/integration/extra.rs: (name, path, mode, arg) with
    mode "scale" (render_extra_with_scale) or "node" (render_node by id)."""
    d = os.path.join(root, "crates", "resvg", "tests", "extra")
    src = os.path.join(root, "crates", "resvg", "tests", "integration", "extra.rs")
    out = []
    if not os.path.exists(src):
        return out
    import re
    text = open(src).read()
    for m in re.finditer(r'render_extra\("extra/([^"]+)"\)', text):
        out.append((m.group(1), os.path.join(d, m.group(1) + ".svg"), "scale", 1.0))
    for m in re.finditer(r'render_extra_with_scale\(\s*"extra/([^"]+)",\s*([0-9.]+)\)', text):
        out.append((m.group(1), os.path.join(d, m.group(1) + ".svg"), "scale", float(m.group(2))))
    for m in re.finditer(r'render_node\("extra/([^"]+)",\s*"([^"]+)"\)', text):
        out.append((m.group(1), os.path.join(d, m.group(1) + ".svg"), "node", m.group(2)))
    return out


def render_extra(tree, mode, arg):
    """The pixmap size, transform (or node id) of main.rs:96-108 for extra tests."""
    tw, th = tree.size
    if mode == "scale":
        iw = max(1, int(round_half_away(tw)))
        ih = max(1, int(round_half_away(th)))
        w = int(math.ceil(np.float32(iw) * np.float32(arg)))
        h = int(math.ceil(np.float32(ih) * np.float32(arg)))
        return w, h, (float(arg), 0.0, 0.0, float(arg), 0.0, 0.0), None
    from resvg_gb300 import node_abs_bbox
    nid = tree.ids.get(arg)
    b = node_abs_bbox(tree, arg) if nid else None
    if b is None:
        return None
    return max(1, int(round_half_away(b[2]))), max(1, int(round_half_away(b[3]))), (1, 0, 0, 1, 0, 0), nid


def run(root, verbose=False, only=None):
    oracle.build()
    results, fixtures = {}, {}
    for cat, name, path in collect(root):
        key = cat + "/" + name
        if only and only not in key:
            continue
        try:
            text = open(path, encoding="utf-8").read()
            tree = svg.load_svg(text)
        except svg.Unsupported as e:
            results[key] = {"status": "unsupported", "why": str(e)[:80]}
            continue
        except Exception as e:  # malformed or exotic input the subset loader rejects
            results[key] = {"status": "unsupported", "why": type(e).__name__}
            continue
        tw, th = tree.size
        w, h = render_size(tw, th)
        ts = (np.float32(w) / np.float32(tw), 0.0, 0.0, np.float32(h) / np.float32(th), 0.0, 0.0)
        pm = oracle.render(tree.view(), ts, w, h)
        actual = png.demultiply(pm)
        expected = png.read_png(path[:-4] + ".png")
        n = pixel_diff(expected, actual)
        results[key] = {"status": "pass" if n == 0 else "fail", "pixels": n}
        if n == 0:
            fixtures[key] = (text, expected)
        if verbose:
            print("%-60s %s" % (key, results[key]))
    for name, path, mode, arg in collect_extra(root):
        key = "extra/" + name
        if only and only not in key:
            continue
        if not os.path.exists(path[:-4] + ".png"):
            continue
        try:
            tree = svg.load_svg(open(path, encoding="utf-8").read())
        except svg.Unsupported as e:
            results[key] = {"status": "unsupported", "why": str(e)[:80]}
            continue
        except Exception as e:
            results[key] = {"status": "unsupported", "why": type(e).__name__}
            continue
        spec = render_extra(tree, mode, arg)
        if spec is None:
            results[key] = {"status": "fail", "pixels": -1}
            continue
        w, h, ts, nid = spec
        pm = oracle.render(tree.view(), ts, w, h) if nid is None else oracle.render_node(tree.view(), nid, ts, w, h)
        expected = png.read_png(path[:-4] + ".png")
        n = pixel_diff(expected, png.demultiply(pm)) if pm is not None else -1
        results[key] = {"status": "pass" if n == 0 else "fail", "pixels": n, "mode": mode}
        if verbose:
            print("%-60s %s" % (key, results[key]))
    return results, fixtures


def write_extra_node_fixtures(root):
    """The render_node cases of extra.rs: name, SVG text, node id, golden image."""
    names, blob = [], {}
    for name, path, mode, arg in collect_extra(root):
        if mode != "node" or not os.path.exists(path[:-4] + ".png"):
            continue
        i = len(names)
        text = open(path, encoding="utf-8").read()
        img = png.read_png(path[:-4] + ".png")
        blob["svg_%d" % i] = np.frombuffer(zlib.compress(text.encode(), 9), dtype=np.uint8)
        blob["png_%d" % i] = np.frombuffer(zlib.compress(np.ascontiguousarray(img).tobytes(), 9), dtype=np.uint8)
        blob["shape_%d" % i] = np.array(img.shape, dtype=np.int32)
        blob["id_%d" % i] = np.array(arg)
        names.append("extra/" + name)
    blob["names"] = np.array(names)
    np.savez(os.path.join(HERE, "extra_nodes.npz"), **blob)
    return names


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else None
    if root is None or not os.path.isdir(root):
        print(__doc__)
        return 2
    if "--extra-nodes" in sys.argv:
        print(write_extra_node_fixtures(root))
        return 0
    only = None
    for a in sys.argv[1:]:
        if a.startswith("--only="):
            only = a[len("--only="):]
    results, fixtures = run(root, verbose="--verbose" in sys.argv, only=only)
    tot = {}
    for r in results.values():
        tot[r["status"]] = tot.get(r["status"], 0) + 1
    print(json.dumps(tot))
    if "--write" in sys.argv:
        with open(os.path.join(HERE, "oracle_pin.json"), "w") as f:
            json.dump({"rule": "resvg integration suite: width 300, demultiplied, channel threshold 1, "
                               "pass = 0 differing pixels", "totals": tot, "tests": results}, f, indent=0,
                      sort_keys=True)
        # a bounded subset travels with the repository: the first
        # FIXTURES_PER_DIR passing tests of every test directory
        by_dir = {}
        for k in sorted(fixtures):
            by_dir.setdefault(k.rsplit("/", 1)[0], []).append(k)
        names = [k for v in by_dir.values() for k in v[:FIXTURES_PER_DIR]]
        blob = {}
        for i, k in enumerate(names):
            text, img = fixtures[k]
            blob["svg_%d" % i] = np.frombuffer(zlib.compress(text.encode(), 9), dtype=np.uint8)
            blob["png_%d" % i] = np.frombuffer(zlib.compress(np.ascontiguousarray(img).tobytes(), 9),
                                               dtype=np.uint8)
            blob["shape_%d" % i] = np.array(img.shape, dtype=np.int32)
        blob["names"] = np.array(names)
        np.savez(os.path.join(HERE, "fixtures.npz"), **blob)
    return 0


if __name__ == "__main__":
    sys.exit(main())
