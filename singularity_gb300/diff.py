"""Differentiable Kerr render and its adjoint, over the C ABI (sgx_diff_*).

The form (include/sgx.h, "differentiable render and its adjoint") keeps the
reference's fixed-step Kerr RK4, termination and disc shading
(geodesic_kernel.cu:300-401, kerr_hamilton.h:97-178) and makes the image
differentiable in four parameters: spin a/M, inclination (rad), disc inner
radius (M) and a temperature scale.  No counterpart in the reference.

``DiffRenderer`` runs the forward pass (image) and the adjoint (gradient of a
loss with respect to the four parameters, given dLoss/dImage).  ``render``
wraps both in a ``torch.autograd.Function`` so that an image loss written in
PyTorch back-propagates into a parameter tensor; ``fit`` is the parameter
recovery loop (Adam on an image loss).
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .backend import Renderer, SgxError

PARAM_NAMES = ("spin", "incl", "r_in", "t_scale")


@dataclass
class DiffOptions:
    """Options of the form (sgx_diff_opts): FP32 or FP64, disc model (emitting
    slab or equatorial crossings), soft edge width (M), winding fade (rad),
    slab half-thickness (M) and optical depth across, adjoint form, steps
    between the forward's checkpoints."""
    precision: int = N.PRECISION_FP32
    edge_width: float = 0.1
    fade_start: float = 0.625 * math.pi
    fade_width: float = 0.125 * math.pi
    model: int = N.DIFF_MODEL_SLAB
    half_thickness: float = 0.3
    tau_perp: float = 4.0
    adjoint_form: int = N.DIFF_ADJOINT_REVERSE
    checkpoint_interval: int = 0  # 0: automatic (10 for FP32 reverse-pass adjoints that fit, else 64)

    def to_c(self) -> N.DiffOpts:
        o = N.DiffOpts()
        o.struct_size = C.sizeof(N.DiffOpts)
        o.precision = self.precision
        o.edge_width = self.edge_width
        o.fade_start = self.fade_start
        o.fade_width = self.fade_width
        o.model = self.model
        o.half_thickness = self.half_thickness
        o.tau_perp = self.tau_perp
        o.adjoint_form = self.adjoint_form
        o.checkpoint_interval = self.checkpoint_interval
        return o

    def oracle_form(self) -> dict:
        """The same form as keyword arguments of the oracle's diff_render."""
        return dict(eps=self.edge_width, fade=(self.fade_start, self.fade_width), model=self.model,
                    half_thickness=self.half_thickness, tau_perp=self.tau_perp)


def _params_c(p: Sequence[float]) -> N.DiffParams:
    if len(p) != 4:
        raise ValueError("params are (spin, incl, r_in, t_scale)")
    return N.DiffParams(*(float(x) for x in p))


class DiffRenderer:
    """Forward and adjoint passes on one device context.

    ``forward`` returns the image as a CUDA tensor (H, W, 3) float32; the
    context keeps the forward's records, which ``backward`` consumes.  Each
    forward bumps ``generation`` so callers can tell whether the records still
    belong to their forward.
    """

    def __init__(self, renderer: Optional[Renderer] = None, device: int = -1):
        self._r = renderer if renderer is not None else Renderer(device)
        self._lib = self._r._lib
        self.generation = 0
        self.last_params: Optional[tuple] = None

    @property
    def renderer(self) -> Renderer:
        return self._r

    def forward(self, u: N.Uniforms, params: Sequence[float], opts: Optional[DiffOptions] = None):
        import torch
        o = (opts or DiffOptions()).to_c()
        img = torch.empty((u.height, u.width, 3), dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        self._r._check(self._lib.sgx_diff_forward(self._r.handle, C.byref(u), C.byref(_params_c(params)),
                                                  C.byref(o), C.c_void_p(img.data_ptr()), C.c_void_p(stream)))
        self.generation += 1
        self.last_params = tuple(float(x) for x in params)
        return img

    def backward(self, grad_image) -> np.ndarray:
        """dLoss/d(spin, incl, r_in, t_scale) for dLoss/dImage of the last forward."""
        import torch
        g = grad_image.detach().to(device="cuda", dtype=torch.float32).contiguous()
        out = (C.c_double * 4)()
        stream = torch.cuda.current_stream().cuda_stream
        self._r._check(self._lib.sgx_diff_backward(self._r.handle, C.c_void_p(g.data_ptr()), out,
                                                   C.c_void_p(stream)))
        return np.array(out[:], dtype=np.float64)

    def stats(self):
        rays, steps, over = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._r._check(self._lib.sgx_diff_stats(self._r.handle, C.byref(rays), C.byref(steps), C.byref(over)))
        return {"rays": rays.value, "steps": steps.value, "crossing_overflow": over.value,
                "checkpoint_steps": int(self._lib.sgx_diff_checkpoint_steps(self._r.handle))}


def _autograd_fn():
    import torch

    class KerrRender(torch.autograd.Function):
        @staticmethod
        def forward(ctx, params, dr, u, opts):
            p = [float(x) for x in params.detach().double().cpu().tolist()]
            img = dr.forward(u, p, opts)
            ctx.dr, ctx.u, ctx.opts, ctx.p = dr, u, opts, p
            ctx.gen = dr.generation
            ctx.p_dtype, ctx.p_device = params.dtype, params.device
            return img

        @staticmethod
        def backward(ctx, g):
            dr = ctx.dr
            if dr.generation != ctx.gen:  # another forward ran since: recompute the records
                dr.forward(ctx.u, ctx.p, ctx.opts)
                ctx.gen = dr.generation
            grad = dr.backward(g)
            return torch.as_tensor(grad, dtype=ctx.p_dtype, device=ctx.p_device), None, None, None

    return KerrRender


_FN = None


def render(params, dr: DiffRenderer, u: N.Uniforms, opts: Optional[DiffOptions] = None):
    """Differentiable image (H, W, 3) of params = tensor([spin, incl, r_in, t_scale])."""
    global _FN
    if _FN is None:
        _FN = _autograd_fn()
    return _FN.apply(params, dr, u, opts)


@dataclass
class FitResult:
    params: np.ndarray        # (steps + 1, 4): the start and every step's parameters
    loss: np.ndarray          # (steps,) loss before each step
    grad: np.ndarray          # (steps, 4)
    seconds: float


def fit(dr: DiffRenderer, u: N.Uniforms, target, init: Sequence[float], steps: int = 200,
        lr: Sequence[float] = (0.02, 0.02, 0.1, 0.02), opts: Optional[DiffOptions] = None,
        bounds: Sequence[tuple] = ((0.0, 0.998), (0.05, math.pi - 0.05), (2.0, 20.0), (0.2, 5.0)),
        cosine: bool = False) -> FitResult:
    """Adam on the mean-squared image error to `target` (a CUDA tensor of the
    form's image), one learning rate per parameter (constant, or decayed along
    a half cosine to 5 % by the last step when `cosine`); parameters are
    clamped to `bounds` after every step.  On the 512x512x4 recovery scene the
    constant rates reach the target to < 1e-4 in 200 steps; the cosine decay
    stops short (t_scale off by 5e-2)."""
    import time

    import torch
    p = torch.tensor(list(init), dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([{"params": [p], "lr": 1.0}])
    lr_t = torch.tensor(list(lr), dtype=torch.float64)
    lo = torch.tensor([b[0] for b in bounds], dtype=torch.float64)
    hi = torch.tensor([b[1] for b in bounds], dtype=torch.float64)
    hist_p = [p.detach().clone().numpy()]
    hist_l, hist_g = [], []
    t0 = time.perf_counter()
    for it in range(steps):
        scale = 0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * it / max(1, steps))) if cosine else 1.0
        opt.zero_grad()
        img = render(p, dr, u, opts)
        loss = torch.mean((img - target) ** 2)
        loss.backward()
        hist_l.append(float(loss.detach()))
        hist_g.append(p.grad.detach().clone().numpy())
        # per-parameter learning rates: Adam's update is scale-free in the
        # gradient, so scaling the update by lr_t gives each parameter its own rate
        with torch.no_grad():
            before = p.detach().clone()
        opt.step()
        with torch.no_grad():
            p.copy_(torch.minimum(torch.maximum(before + (p - before) * lr_t * scale, lo), hi))
        hist_p.append(p.detach().clone().numpy())
    torch.cuda.synchronize()
    return FitResult(np.array(hist_p), np.array(hist_l), np.array(hist_g), time.perf_counter() - t0)


__all__ = ["DiffOptions", "DiffRenderer", "render", "fit", "FitResult", "PARAM_NAMES", "SgxError"]
