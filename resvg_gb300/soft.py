"""Differentiable soft-coverage rendering on the GPU (host-side API).

A batch of scenes of closed cubic paths with solid or 4-stop linear-gradient
paints and one Gaussian blur per scene is rendered by the FP32 analytic-area
soft rasteriser (csrc/kernels/soft.cu); the hand-written adjoint returns the
gradients of any pixel loss with respect to control points, colours, stop
colours, stop offsets and blur sigma.  `SoftRender` wraps the C ABI as a
torch.autograd.Function (the gradient harness); the kernels run through the
library either way.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi, check, lib

PARAMS = ("points", "colors", "stop_offsets", "stop_colors", "sigma", "opacity")


def make_scenes(seed=0, scenes=256, size=256, paths=64, min_segs=4, max_segs=16):
    """Seeded synthetic scenes (host numpy arrays): closed cubic loops with
    control points uniform over the canvas, alternating solid and linear
    gradient paints (4 stops), alpha in [0.3, 1], blur sigma in [0.5, 4]."""
    rng = np.random.default_rng(seed)
    npaths = scenes * paths
    segs = rng.integers(min_segs, max_segs + 1, size=npaths)
    seg_offset = np.concatenate([[0], np.cumsum(segs)]).astype(np.uint32)
    total = int(seg_offset[-1])
    # 3 points per cubic: loops are closed by construction (the last cubic
    # ends at the path's start point)
    points = rng.uniform(0.0, float(size), size=(3 * total, 2)).astype(np.float32)
    paint_kind = (np.arange(npaths) % 2).astype(np.uint32)
    colors = rng.uniform(0.0, 1.0, size=(npaths, 4)).astype(np.float32)
    colors[:, 3] = rng.uniform(0.3, 1.0, size=npaths)
    stop_offsets = np.sort(rng.uniform(0.0, 1.0, size=(npaths, 4)), axis=1).astype(np.float32)
    stop_colors = rng.uniform(0.0, 1.0, size=(npaths, 4, 4)).astype(np.float32)
    stop_colors[:, :, 3] = rng.uniform(0.3, 1.0, size=(npaths, 4))
    grad_line = rng.uniform(0.0, float(size), size=(npaths, 4)).astype(np.float32)
    sigma = rng.uniform(0.5, 4.0, size=scenes).astype(np.float32)
    # drawn last so the other parameters keep the values earlier seeds gave them
    opacity = rng.uniform(0.3, 1.0, size=npaths).astype(np.float32)
    return {"scenes": scenes, "width": size, "height": size, "paths": paths, "seg_offset": seg_offset,
            "points": points, "paint_kind": paint_kind, "colors": colors, "stop_offsets": stop_offsets,
            "stop_colors": stop_colors, "grad_line": grad_line, "sigma": sigma, "opacity": opacity}


def perturb(arrays, seed=1, point_sd=2.0, color_sd=0.05):
    """The target scene: control points + N(0, point_sd), colours + N(0, color_sd)."""
    rng = np.random.default_rng(seed)
    out = dict(arrays)
    pts = arrays["points"] + rng.normal(0.0, point_sd, size=arrays["points"].shape).astype(np.float32)
    out["points"] = pts.astype(np.float32)
    out["colors"] = np.clip(arrays["colors"] + rng.normal(0.0, color_sd, size=arrays["colors"].shape), 0, 1).astype(np.float32)
    out["stop_colors"] = np.clip(arrays["stop_colors"] + rng.normal(0.0, color_sd, size=arrays["stop_colors"].shape),
                                 0, 1).astype(np.float32)
    return out


def _declare(L):
    if getattr(L, "_soft_declared", False):
        return
    L.rgpu_soft_forward.restype = C.c_int
    L.rgpu_soft_forward.argtypes = [C.POINTER(_abi.SoftBatch), C.c_void_p, C.c_void_p, C.c_void_p]
    L.rgpu_soft_backward.restype = C.c_int
    L.rgpu_soft_backward.argtypes = [C.POINTER(_abi.SoftBatch), C.c_void_p, C.c_void_p, C.POINTER(_abi.SoftGrads),
                                     C.c_void_p]
    L.rgpu_soft_mse.restype = C.c_int
    L.rgpu_soft_mse.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p]
    L._soft_declared = True


class Scenes:
    """A batch resident on the GPU: static structure (segment offsets, paint
    kinds, gradient lines) plus the learnable parameters as torch tensors."""

    def __init__(self, arrays, device="cuda"):
        import torch
        self.S, self.W, self.H, self.P = (int(arrays[k]) for k in ("scenes", "width", "height", "paths"))
        self.total_segments = int(arrays["seg_offset"][-1])
        self.seg_offset = torch.from_numpy(arrays["seg_offset"].astype(np.int32)).to(device)
        self.paint_kind = torch.from_numpy(arrays["paint_kind"].astype(np.int32)).to(device)
        self.grad_line = torch.from_numpy(arrays["grad_line"]).to(device).contiguous()
        self.params = {k: torch.from_numpy(np.ascontiguousarray(arrays[k])).to(device).contiguous() for k in PARAMS}

    def batch(self, params=None):
        p = params or self.params
        b = _abi.SoftBatch()
        b.scenes, b.width, b.height, b.paths_per_scene = self.S, self.W, self.H, self.P
        b.total_segments = self.total_segments
        b.seg_offset = self.seg_offset.data_ptr()
        b.paint_kind = self.paint_kind.data_ptr()
        b.grad_line = self.grad_line.data_ptr()
        for k in PARAMS:
            t = p[k]
            assert t.is_cuda and t.dtype.is_floating_point and t.is_contiguous()
            setattr(b, k, t.data_ptr())
        return b

    def image_shape(self):
        return (self.S, self.H, self.W, 4)


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def forward(scenes, params=None):
    """(image, blurred): composite and blurred composite, (S, H, W, 4) float32."""
    import torch
    L = lib()
    _declare(L)
    dev = scenes.seg_offset.device
    image = torch.empty(scenes.image_shape(), dtype=torch.float32, device=dev)
    blurred = torch.empty_like(image)
    b = scenes.batch(params)
    check(L.rgpu_soft_forward(C.byref(b), image.data_ptr(), blurred.data_ptr(), _stream()), "rgpu_soft_forward")
    return image, blurred


def backward(scenes, image, grad_blurred, params=None):
    """Gradients of <grad_blurred, blurred(params)> with respect to every parameter."""
    import torch
    L = lib()
    _declare(L)
    p = params or scenes.params
    grads = {k: torch.empty_like(p[k]) for k in PARAMS}
    g = _abi.SoftGrads(*[grads[k].data_ptr() for k in PARAMS])
    b = scenes.batch(params)
    gb = grad_blurred.contiguous()
    check(L.rgpu_soft_backward(C.byref(b), image.data_ptr(), gb.data_ptr(), C.byref(g), _stream()),
          "rgpu_soft_backward")
    return grads


def mse(blurred, target):
    """(loss as a float, dloss/dblurred) for the mean squared error."""
    import torch
    L = lib()
    _declare(L)
    loss = torch.zeros(1, dtype=torch.float32, device=blurred.device)
    grad = torch.empty_like(blurred)
    check(L.rgpu_soft_mse(blurred.data_ptr(), target.data_ptr(), blurred.numel(), loss.data_ptr(), grad.data_ptr(),
                          _stream()), "rgpu_soft_mse")
    return float(loss.item()), grad


def _autograd():
    import torch

    class SoftRender(torch.autograd.Function):
        """blurred = render(points, colors, stop_offsets, stop_colors, sigma, opacity)."""

        @staticmethod
        def forward(ctx, scenes, points, colors, stop_offsets, stop_colors, sigma, opacity):
            params = {"points": points.contiguous(), "colors": colors.contiguous(),
                      "stop_offsets": stop_offsets.contiguous(), "stop_colors": stop_colors.contiguous(),
                      "sigma": sigma.contiguous(), "opacity": opacity.contiguous()}
            image, blurred = forward(scenes, params)
            ctx.scenes = scenes
            ctx.params = params
            ctx.save_for_backward(image)
            return blurred

        @staticmethod
        def backward(ctx, grad_blurred):
            (image,) = ctx.saved_tensors
            g = backward(ctx.scenes, image, grad_blurred, ctx.params)
            return None, g["points"], g["colors"], g["stop_offsets"], g["stop_colors"], g["sigma"], g["opacity"]

    return SoftRender


_SoftRender = None


def render(scenes, points, colors, stop_offsets, stop_colors, sigma, opacity):
    """Differentiable render (torch autograd) of the blurred composite."""
    global _SoftRender
    if _SoftRender is None:
        _SoftRender = _autograd()
    return _SoftRender.apply(scenes, points, colors, stop_offsets, stop_colors, sigma, opacity)
