"""The FP64 reference of the differentiable renderer on its own (CPU): its
forward-mode gradients against central finite differences of its own FP64
loss (h = 1e-6), on a small scene."""
import numpy as np
import pytest

from resvg_gb300 import soft


@pytest.fixture(scope="module")
def small():
    a = soft.make_scenes(seed=5, scenes=1, size=32, paths=4, min_segs=2, max_segs=4)
    t = soft.perturb(a, seed=6)
    return a, t


def _target(oracle_mod, t):
    return oracle_mod.soft_forward(t)[1].astype(np.float32)


def _loss(oracle_mod, arrays, target):
    _, bl = oracle_mod.soft_forward(arrays)
    return float(np.mean((bl - target.astype(np.float64)) ** 2))


@pytest.mark.parametrize("group", ["points", "colors", "stop_offsets", "stop_colors", "sigma", "opacity"])
def test_forward_mode_matches_fd(oracle_mod, small, group):
    a, t = small
    target = _target(oracle_mod, t)
    rng = np.random.default_rng(7)
    v = rng.normal(size=a[group].shape)
    _, dl = oracle_mod.soft_dloss(a, target, {group: v})
    h = 1e-6
    ap, am = dict(a), dict(a)
    ap[group] = (a[group] + h * v).astype(np.float32)
    am[group] = (a[group] - h * v).astype(np.float32)
    # the perturbation is rounded to f32 in the arrays: use the actual step
    step = (ap[group].astype(np.float64) - am[group].astype(np.float64))
    fd = (_loss(oracle_mod, ap, target) - _loss(oracle_mod, am, target))
    _, dl_actual = oracle_mod.soft_dloss(a, target, {group: step})
    assert fd == pytest.approx(dl_actual, rel=1e-4, abs=1e-12)
    assert dl != 0.0
