"""The oracle against resvg's golden images (CPU).

`test_fixtures_match` replays the committed fixtures (a subset of resvg's
integration suite, tests/golden/fixtures.npz) through the SVG-subset front
end and the oracle and requires zero differing pixels under the suite's rule.
`test_full_suite_summary` reruns the whole comparison only when the
environment variable RESVG_REFERENCE names a resvg checkout (it is skipped
otherwise) and checks that no test that passed in the committed summary
(tests/golden/oracle_pin.json) regressed.
"""
import json
import os

import numpy as np
import pytest

from tests import golden_fixtures as G

FIXTURES = G.load()


@pytest.fixture(scope="module")
def svg_mod(native):
    from resvg_gb300 import svg
    return svg


@pytest.mark.parametrize("idx", range(len(FIXTURES)), ids=[f[0] for f in FIXTURES])
def test_fixtures_match(svg_mod, oracle_mod, idx):
    from resvg_gb300 import png
    name, text, expected = FIXTURES[idx]
    tree = svg_mod.load_svg(text)
    w, h, ts = G.render_transform(tree)
    actual = png.demultiply(oracle_mod.render(tree.view(), ts, w, h))
    assert G.pixel_diff(expected, actual) == 0, name


def _reference_root():
    root = os.environ.get("RESVG_REFERENCE")  # a resvg checkout, when one is available
    return root if root and os.path.isdir(os.path.join(root, "crates", "resvg", "tests", "tests")) else None


@pytest.mark.skipif(_reference_root() is None, reason="no resvg checkout available")
def test_full_suite_summary(native, oracle_mod):
    from tests.golden import pin_oracle
    results, _ = pin_oracle.run(_reference_root())
    with open(os.path.join(G.HERE, "oracle_pin.json")) as f:
        pinned = json.load(f)["tests"]
    regressed = [k for k, v in pinned.items() if v["status"] == "pass" and results.get(k, {}).get("status") != "pass"]
    assert not regressed, regressed[:10]
