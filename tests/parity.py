"""Helpers shared by the GPU parity tests: run the CUDA path through the C
ABI (via the package's mirror classes) and the FP64 oracle on the same
inputs, and compare them the way the parity bar is defined:

* window bounds (integers): bit-exact, except where the FP64 domain
  transform puts a bound decision within TIE_REL*(sigma+1) of the threshold
  (a near-tie that FP32 and FP64 may resolve differently; counted);
* float outputs: max-abs <= 1e-4 * (target range), evaluated against the
  FP64 oracle run on the same windows the GPU chose.
"""
from __future__ import annotations

import math

import numpy as np

TOL_REL = 1e-4   # max-abs error relative to the target range
TIE_REL = 1e-4   # near-tie margin, relative to (sigma + 1)


def target_range(t) -> float:
    r = float(np.max(t) - np.min(t))
    return r if r > 0 else 1.0


def check_bounds(gpu_lu, ora_lum, sigma):
    """Return (#mismatch, #mismatch that is not a near-tie)."""
    gl, gu = gpu_lu
    ol, ou, om = ora_lum
    mism = (gl != ol) | (gu != ou)
    tie = np.abs(om) <= TIE_REL * (sigma + 1.0)
    return int(mism.sum()), int((mism & ~tie).sum())


def filter_sigmas(sx, sy, num_iter):
    out = []
    for it in range(num_iter):
        m = np.float32(1.0) if it == 0 else np.float32(
            3 * 2.0 ** (num_iter - (it + 1)) / math.sqrt(4.0 ** num_iter - 1))
        out.append((float(np.float32(np.float32(sx) * m)),
                    float(np.float32(np.float32(sy) * m))))
    return out


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 to bfloat16 (round to nearest even) and back."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)
