"""The differentiable soft-coverage renderer on the GPU against its FP64
reference (oracle/soft.cpp) and against central finite differences.

Tolerances: the FP32 forward image within 2e-4 of the FP64 one (absolute, on
values in [0, 1]); adjoint directional derivatives within 1e-3 relative of
the FP64 forward-mode ones and of central finite differences (step 1e-3) of
the FP64 forward; within 1e-2 of central differences (step 1e-2) of the FP32
GPU forward."""
import numpy as np
import pytest

from resvg_gb300 import soft

pytestmark = pytest.mark.gpu

GROUPS = ["points", "colors", "stop_offsets", "stop_colors", "sigma", "opacity"]


@pytest.fixture(scope="module")
def case(gpu):
    import torch
    a = soft.make_scenes(seed=21, scenes=2, size=48, paths=6, min_segs=2, max_segs=6)
    t = soft.perturb(a, seed=22)
    sc = soft.Scenes(a)
    tgt = soft.Scenes(t)
    _, target = soft.forward(tgt)
    torch.cuda.synchronize()
    return a, sc, target


def test_forward_matches_fp64(case, oracle_mod):
    a, sc, _ = case
    image, blurred = soft.forward(sc)
    im64, bl64 = oracle_mod.soft_forward(a)
    assert np.abs(image.cpu().numpy() - im64).max() <= 2e-4
    assert np.abs(blurred.cpu().numpy() - bl64).max() <= 2e-4


def _adjoint(sc, target):
    image, blurred = soft.forward(sc)
    loss, g = soft.mse(blurred, target)
    return loss, soft.backward(sc, image, g)


@pytest.mark.parametrize("group", GROUPS + ["all"])
def test_adjoint_matches_fp64_forward_mode(case, oracle_mod, group):
    a, sc, target = case
    loss, grads = _adjoint(sc, target)
    rng = np.random.default_rng(5)
    groups = GROUPS if group == "all" else [group]
    v = {k: rng.normal(size=a[k].shape) for k in groups}
    adj = sum(float((grads[k].double().cpu().numpy() * v[k]).sum()) for k in groups)
    loss64, ref = oracle_mod.soft_dloss(a, target.cpu().numpy(), v)
    assert loss == pytest.approx(loss64, rel=1e-4)
    assert adj == pytest.approx(ref, rel=1e-3), (adj, ref)


@pytest.mark.parametrize("group", GROUPS)
def test_adjoint_matches_central_fd(case, oracle_mod, group):
    """Central differences with step 1e-3 of the FP64 forward (the FP32
    forward's rounding, ~1e-7 per pixel, would swamp a 1e-3 step).  Stop
    offsets use 1e-6: gradients are sampled at pixel centres, so the loss is
    only piecewise smooth in an offset, with a kink wherever a pixel's t
    crosses it (about every 1/48 of t here); a 1e-3 step crosses several."""
    a, sc, target = case
    _, grads = _adjoint(sc, target)
    rng = np.random.default_rng(9)
    v = rng.normal(size=a[group].shape)
    h = 1e-6 if group == "stop_offsets" else 1e-3
    tgt = target.double().cpu().numpy()

    def L(sign):
        p = dict(a)
        p[group] = (a[group].astype(np.float64) + sign * h * v).astype(np.float32)
        return float(((oracle_mod.soft_forward(p)[1] - tgt) ** 2).mean()), p[group]
    lp, xp = L(+1)
    lm, xm = L(-1)
    # the perturbed parameters are f32: divide by the step actually taken
    step = xp.astype(np.float64) - xm.astype(np.float64)
    fd = lp - lm
    adj = float((grads[group].double().cpu().numpy() * step).sum())
    assert fd == pytest.approx(adj, rel=1e-3)


@pytest.mark.parametrize("group", [g for g in GROUPS if g != "stop_offsets"])
def test_adjoint_matches_fp32_fd_loosely(case, group):
    """The same check on the FP32 GPU forward itself, at 1e-2 relative (not
    for stop offsets: see above; FP32 cannot take a step small enough)."""
    import torch
    a, sc, target = case
    _, grads = _adjoint(sc, target)
    rng = np.random.default_rng(9)
    v = torch.from_numpy(rng.normal(size=a[group].shape).astype(np.float32)).cuda()
    h = 1e-2

    def L(sign):
        p = dict(sc.params)
        p[group] = (sc.params[group] + sign * h * v).contiguous()
        _, bl = soft.forward(sc, p)
        return float(((bl.double() - target.double()) ** 2).mean())
    fd = (L(+1) - L(-1)) / (2 * h)
    adj = float((grads[group] * v).double().sum())
    assert fd == pytest.approx(adj, rel=1e-2)


def test_autograd_function_matches_direct_call(case):
    import torch
    a, sc, target = case
    _, grads = _adjoint(sc, target)
    ps = {k: sc.params[k].clone().requires_grad_(True) for k in GROUPS}
    out = soft.render(sc, ps["points"], ps["colors"], ps["stop_offsets"], ps["stop_colors"], ps["sigma"],
                      ps["opacity"])
    loss = ((out - target) ** 2).mean()
    loss.backward()
    for k in GROUPS:
        torch.testing.assert_close(ps[k].grad, grads[k], rtol=1e-4, atol=1e-9)


def test_config4_shape_runs(gpu):
    """One full-size config-4 batch (256 scenes x 256^2 x 64 paths) forward + adjoint."""
    a = soft.make_scenes(seed=4, scenes=256, size=256, paths=64)
    t = soft.perturb(a, seed=5)
    sc, tgt = soft.Scenes(a), soft.Scenes(t)
    _, target = soft.forward(tgt)
    loss, grads = _adjoint(sc, target)
    assert np.isfinite(loss) and loss > 0
    for k in GROUPS:
        assert bool(grads[k].isfinite().all())
    assert float(grads["points"].abs().sum()) > 0


@pytest.fixture(scope="module")
def slice_case(gpu):
    """Four scenes of the config-4 shape (256^2, 64 paths of 2-8 cubic
    segments, four-stop gradients, per-scene blur): the same generator and
    sizes as the 256-scene batch, a slice the FP64 reference finishes in
    seconds."""
    import torch
    a = soft.make_scenes(seed=4, scenes=4, size=256, paths=64)
    t = soft.perturb(a, seed=5)
    sc, tgt = soft.Scenes(a), soft.Scenes(t)
    _, target = soft.forward(tgt)
    torch.cuda.synchronize()
    return a, sc, target


def test_config4_slice_forward_matches_fp64(slice_case, oracle_mod):
    a, sc, _ = slice_case
    image, blurred = soft.forward(sc)
    im64, bl64 = oracle_mod.soft_forward(a)
    assert np.abs(image.cpu().numpy() - im64).max() <= 2e-4
    assert np.abs(blurred.cpu().numpy() - bl64).max() <= 2e-4


@pytest.mark.parametrize("group", GROUPS + ["all"])
def test_config4_slice_adjoint_matches_fp64_forward_mode(slice_case, oracle_mod, group):
    """Directional derivatives of the loss at full scene size: the GPU
    adjoint against the FP64 forward-mode derivative, 1e-3 relative."""
    a, sc, target = slice_case
    loss, grads = _adjoint(sc, target)
    rng = np.random.default_rng(17)
    groups = GROUPS if group == "all" else [group]
    v = {k: rng.normal(size=a[k].shape) for k in groups}
    adj = sum(float((grads[k].double().cpu().numpy() * v[k]).sum()) for k in groups)
    loss64, ref = oracle_mod.soft_dloss(a, target.cpu().numpy(), v)
    assert loss == pytest.approx(loss64, rel=1e-4)
    assert adj == pytest.approx(ref, rel=1e-3), (adj, ref)


@pytest.mark.parametrize("group", ["points", "colors", "sigma", "opacity"])
def test_config4_slice_adjoint_matches_central_fd(slice_case, oracle_mod, group):
    """Central differences (step 1e-3) of the FP64 forward at full scene
    size, 1e-3 relative."""
    a, sc, target = slice_case
    _, grads = _adjoint(sc, target)
    rng = np.random.default_rng(23)
    v = rng.normal(size=a[group].shape)
    tgt = target.double().cpu().numpy()

    def L(sign):
        p = dict(a)
        p[group] = (a[group].astype(np.float64) + sign * 1e-3 * v).astype(np.float32)
        return float(((oracle_mod.soft_forward(p)[1] - tgt) ** 2).mean()), p[group]
    lp, xp = L(+1)
    lm, xm = L(-1)
    adj = float((grads[group].double().cpu().numpy() * (xp.astype(np.float64) - xm.astype(np.float64))).sum())
    assert lp - lm == pytest.approx(adj, rel=1e-3)
