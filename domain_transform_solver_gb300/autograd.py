"""torch.autograd binding of the batched DTS solve and its adjoint.

The reference has no gradients; this is the thin binding over
dtsgb_batch_dts_backward_device (include/dtsgb.h) that lets a PyTorch graph
differentiate through the fixed-iteration DTS solve with respect to the
target and the confidence.  The window bounds come from the guide and are
held fixed: the guide gets no gradient.

Tensors stay on the GPU: the solve reads the caller's device buffers and
writes its result into a tensor allocated by PyTorch.  The library's launch
sequence is replayed from a CUDA graph, which cannot be captured on the
legacy default stream, so the work runs on a side stream ordered after, and
before, PyTorch's current stream.  Each forward holds its own batch
(checkpoints and window bounds) until its backward has run.
"""
from __future__ import annotations

import threading

import torch

from .solvers import (COLOR_SPACE, Batch, DomainFilterParams, DomainOptimizeParams)

__all__ = ["DtsSolveFunction", "dts_solve"]

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
