"""torch.autograd bindings of the DTS and HFBS solves and their adjoints.

The reference has no gradients; these are thin bindings over
dtsgb_batch_dts_backward_device and dtsgb_hfbs_backward_device
(include/dtsgb.h) that let a PyTorch graph differentiate through the
fixed-iteration solves with respect to the target and the confidence.  DTS
window bounds and HFBS bins, counts and normalisation come from the guide
and are held fixed: the guide gets no gradient.  The soft-window DTS solve
(soft_dts_solve, over dtsgb_soft_*) also differentiates with respect to the
edge weights dH, dV that edge_weights derives from the guide.

Tensors stay on the GPU: the solve reads the caller's device buffers and
writes its result into a tensor allocated by PyTorch.  The library's launch
sequence is replayed from a CUDA graph, which cannot be captured on the
legacy default stream, so the work runs on a side stream ordered after, and
before, PyTorch's current stream.  Each forward holds its own batch
(checkpoints and window bounds) until its backward has run.
"""
from __future__ import annotations

import threading

import numpy as np
import torch

from .solvers import (COLOR_SPACE, HFBS, Batch, DomainFilterParams, DomainOptimizeParams,
                      HFBSGridParams, ImageDim, ImageType, SoftDTS)

__all__ = ["DtsSolveFunction", "dts_solve", "HfbsSolveFunction", "hfbs_solve",
           "SoftDtsSolveFunction", "soft_dts_solve", "edge_weights"]

_pool: dict = {}
_pool_lock = threading.Lock()


def _take_batch(key):
    with _pool_lock:
        free = _pool.get(key)
        if free:
            return free.pop()
    b, h, w, flags = key
    return Batch([(w, h)] * b, flags=flags)


def _give_back(key, batch):
    with _pool_lock:
        _pool.setdefault(key, []).append(batch)


_side: dict = {}


def _side_stream(device) -> torch.cuda.Stream:
    with _pool_lock:
        s = _side.get(device)
        if s is None:
            s = _side[device] = torch.cuda.Stream(device)
        return s


def _ptrs(t: torch.Tensor):
    return [t[i].data_ptr() for i in range(t.shape[0])]


class DtsSolveFunction(torch.autograd.Function):
    """v = DTS(guide; target, confidence) for a batch of equal-size images.

    forward(target [B,H,W] f32, confidence [B,H,W] f32, rgba [B,H,W,4] u8,
    filter_params, optimize_params, color_space, segment, flags) -> [B,H,W] f32
    """

    @staticmethod
    def forward(ctx, target, confidence, rgba, filter_params, optimize_params,
                color_space=COLOR_SPACE.YCbCr, segment=0, flags=0):
        if not (target.is_cuda and confidence.is_cuda and rgba.is_cuda):
            raise ValueError("DtsSolveFunction wants CUDA tensors")
        if target.dtype != torch.float32 or confidence.dtype != torch.float32:
            raise ValueError("target and confidence must be float32")
        if rgba.dtype != torch.uint8 or rgba.shape[-1] != 4:
            raise ValueError("rgba must be uint8 [B,H,W,4]")
        B, H, W = target.shape
        if confidence.shape != target.shape or tuple(rgba.shape[:3]) != (B, H, W):
            raise ValueError("target, confidence and rgba shapes differ")
        t = target.contiguous()
        c = confidence.contiguous()
        g = rgba.contiguous()
        key = (B, H, W, int(flags))
        batch = _take_batch(key)
        out = torch.empty_like(t)
        cur = torch.cuda.current_stream(t.device)
        side = _side_stream(t.device)
        side.wait_stream(cur)
        batch.set_stream(side.cuda_stream)
        batch.enable_grad(True, int(segment))
        batch.upload_device(color_space, _ptrs(g), _ptrs(t), _ptrs(c))
        batch.solve_dts(filter_params, optimize_params)
        batch.download_device(0, _ptrs(out))
        cur.wait_stream(side)
        ctx.batch, ctx.key = batch, key
        return out

    @staticmethod
    def backward(ctx, grad_out):
        batch = ctx.batch
        go = grad_out.contiguous().float()
        gt = torch.empty_like(go)
        gc = torch.empty_like(go)
        cur = torch.cuda.current_stream(go.device)
        side = _side_stream(go.device)
        side.wait_stream(cur)
        batch.set_stream(side.cuda_stream)
        batch.backward_device(_ptrs(go), _ptrs(gt), _ptrs(gc))
        cur.wait_stream(side)
        ctx.batch = None
        _give_back(ctx.key, batch)
        need_t, need_c = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        return (gt if need_t else None, gc if need_c else None,
                None, None, None, None, None, None)


def dts_solve(rgba: torch.Tensor, target: torch.Tensor, confidence: torch.Tensor,
              filter_params: DomainFilterParams | None = None,
              optimize_params: DomainOptimizeParams | None = None,
              color_space: COLOR_SPACE = COLOR_SPACE.YCbCr, segment: int = 0,
              flags: int = 0) -> torch.Tensor:
    """Differentiable batched DTS solve (ComputeColorSpaceDifferential +
    IntegrateColorDifferentials + Optimize on every image)."""
    fp = filter_params or DomainFilterParams()
    op = optimize_params or DomainOptimizeParams()
    return DtsSolveFunction.apply(target, confidence, rgba, fp, op, color_space, segment,
                                  flags)


def _hfbs_max_grid(w, h, p: HFBSGridParams):
    """The grid of Optimize for (w, h, p) (src/hfbs.cu:589-591)."""
    import math
    return (int(math.ceil(np.float32(w) / np.float32(p.sigma_x))),
            int(math.ceil(np.float32(h) / np.float32(p.sigma_y))),
            int(math.ceil(255.0 / float(np.float32(p.sigma_l)))))


def _take_hfbs(key):
    with _pool_lock:
        free = _pool.get(key)
        if free:
            return free.pop()
    _, h, w, gx, gy, gl = key
    return HFBS(ImageDim(w, h), gx, gy, gl)


class HfbsSolveFunction(torch.autograd.Function):
    """out = HFBS(guide; target, confidence) for a batch of equal-size images,
    each solved by its own HFBS handle.

    forward(target [B,H,W] f32, confidence [B,H,W] f32, rgba [B,H,W,4] u8,
    grid_params, color_space, segment, max_grid) -> [B,H,W] f32
    """

    @staticmethod
    def forward(ctx, target, confidence, rgba, grid_params, color_space=COLOR_SPACE.YCbCr,
                segment=0, max_grid=None):
        if not (target.is_cuda and confidence.is_cuda and rgba.is_cuda):
            raise ValueError("HfbsSolveFunction wants CUDA tensors")
        if target.dtype != torch.float32 or confidence.dtype != torch.float32:
            raise ValueError("target and confidence must be float32")
        if rgba.dtype != torch.uint8 or rgba.shape[-1] != 4:
            raise ValueError("rgba must be uint8 [B,H,W,4]")
        B, H, W = target.shape
        if confidence.shape != target.shape or tuple(rgba.shape[:3]) != (B, H, W):
            raise ValueError("target, confidence and rgba shapes differ")
        t = target.contiguous()
        c = confidence.contiguous()
        g = rgba.contiguous()
        gx, gy, gl = max_grid or _hfbs_max_grid(W, H, grid_params)
        key = ("hfbs", H, W, gx, gy, gl)
        out = torch.empty_like(t)
        cur = torch.cuda.current_stream(t.device)
        side = _side_stream(t.device)
        side.wait_stream(cur)
        solvers = []
        for i in range(B):
            s = _take_hfbs(key)
            s.SetStream(side.cuda_stream)
            s.EnableGrad(True, int(segment))
            s.InitFrameDevice(color_space, g[i].data_ptr(), t[i].data_ptr(), c[i].data_ptr())
            s.SetFilterParams(grid_params)
            s.Optimize()
            s.DownloadDevice(ImageType.OPTIMIZED_QUANTITY, out[i].data_ptr())
            solvers.append(s)
        cur.wait_stream(side)
        ctx.solvers, ctx.key = solvers, key
        return out

    @staticmethod
    def backward(ctx, grad_out):
        go = grad_out.contiguous().float()
        need_t, need_c = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        gt = torch.empty_like(go)
        gc = torch.empty_like(go)
        cur = torch.cuda.current_stream(go.device)
        side = _side_stream(go.device)
        side.wait_stream(cur)
        for i, s in enumerate(ctx.solvers):
            s.SetStream(side.cuda_stream)
            s.BackwardDevice(go[i].data_ptr(), gt[i].data_ptr() if need_t else None,
                             gc[i].data_ptr() if need_c else None)
        cur.wait_stream(side)
        with _pool_lock:
            _pool.setdefault(ctx.key, []).extend(ctx.solvers)
        ctx.solvers = None
        return (gt if need_t else None, gc if need_c else None, None, None, None, None, None)


def hfbs_solve(rgba: torch.Tensor, target: torch.Tensor, confidence: torch.Tensor,
               grid_params: HFBSGridParams | None = None,
               color_space: COLOR_SPACE = COLOR_SPACE.YCbCr, segment: int = 0,
               max_grid=None) -> torch.Tensor:
    """Differentiable HFBS solve (InitFrame + SetFilterParams + Optimize on
    every image).  max_grid: the handles' (max_grid_x, max_grid_y,
    max_grid_l), by default the solve's own grid."""
    gp = grid_params or HFBSGridParams()
    return HfbsSolveFunction.apply(target, confidence, rgba, gp, color_space, segment,
                                   max_grid)


def edge_weights(rgba: torch.Tensor, filter_params: DomainFilterParams | None = None,
                 color_space: COLOR_SPACE = COLOR_SPACE.YCbCr):
    """The guide-derived edge weights (dH, dV), each [B,H,W] float32, as
    ComputeColorSpaceDifferential computes them (not differentiable: the
    guide is integer)."""
    if not rgba.is_cuda or rgba.dtype != torch.uint8 or rgba.shape[-1] != 4:
        raise ValueError("rgba must be a CUDA uint8 [B,H,W,4] tensor")
    B, H, W = rgba.shape[:3]
    g = rgba.contiguous()
    dh = torch.empty((B, H, W), dtype=torch.float32, device=rgba.device)
    dv = torch.empty_like(dh)
    s = SoftDTS([(W, H)] * B)
    cur = torch.cuda.current_stream(rgba.device)
    s.set_stream(cur.cuda_stream)
    s.edge_weights(color_space, _ptrs(g), filter_params or DomainFilterParams(), _ptrs(dh),
                   _ptrs(dv))
    s.close()
    return dh, dv


class SoftDtsSolveFunction(torch.autograd.Function):
    """v = soft-window DTS(dH, dV; target, confidence) for a batch of
    equal-size images, differentiable in all four inputs.

    forward(dH, dV, target, confidence [B,H,W] f32, optimize_params, tau)
    -> [B,H,W] f32
    """

    @staticmethod
    def forward(ctx, dh, dv, target, confidence, optimize_params, tau=1.0):
        ts = (dh, dv, target, confidence)
        if not all(x.is_cuda and x.dtype == torch.float32 for x in ts):
            raise ValueError("SoftDtsSolveFunction wants CUDA float32 tensors")
        if not all(x.shape == target.shape for x in ts) or target.dim() != 3:
            raise ValueError("dH, dV, target and confidence must share one [B,H,W] shape")
        B, H, W = target.shape
        dh, dv, t, c = (x.contiguous() for x in ts)
        s = SoftDTS([(W, H)] * B)
        cur = torch.cuda.current_stream(t.device)
        s.set_stream(cur.cuda_stream)
        out = torch.empty_like(t)
        s.solve(_ptrs(dh), _ptrs(dv), _ptrs(t), _ptrs(c), optimize_params, float(tau),
                _ptrs(out))
        ctx.soft = s
        ctx.keep = (dh, dv, t, c)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        s = ctx.soft
        go = grad_out.contiguous().float()
        grads = [torch.empty_like(go) if need else None for need in ctx.needs_input_grad[:4]]
        s.set_stream(torch.cuda.current_stream(go.device).cuda_stream)
        s.backward(_ptrs(go), *[None if g is None else _ptrs(g) for g in grads[2:]],
                   *[None if g is None else _ptrs(g) for g in grads[:2]])
        s.close()
        ctx.soft = ctx.keep = None
        return (*grads, None, None)


def soft_dts_solve(dh: torch.Tensor, dv: torch.Tensor, target: torch.Tensor,
                   confidence: torch.Tensor,
                   optimize_params: DomainOptimizeParams | None = None,
                   tau: float = 1.0) -> torch.Tensor:
    """Differentiable soft-window DTS Optimize: windows with fractional ends
    of width tau (transformed-domain units) around the reference's
    threshold sigma_z, so that the result has gradients with respect to the
    edge weights dH, dV as well as the target and the confidence."""
    op = optimize_params or DomainOptimizeParams()
    return SoftDtsSolveFunction.apply(dh, dv, target, confidence, op, tau)
