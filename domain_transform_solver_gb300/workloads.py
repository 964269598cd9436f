"""Seeded synthetic inputs for the five benchmark configurations.

The reference benchmarks on Middlebury-derived depth super-resolution,
colorization and stereo data; none of that is shipped or reproduced here.
These generators make inputs of the same roles, sizes and value ranges:

  cfg 0  DTS depth super-resolution 640x480: polygon RGB guide + N(0,3),
         piecewise-planar depth in [0.5,10] sampled every 8 px (+N(0,0.01)),
         confidence 1 at the samples.
  cfg 1  HFBS colorization 640x480: grey guide of 30 linearly shaded
         polygons; U/V targets at a random 2% of pixels, polygon-constant in
         [-0.5,0.5], confidence 1 there.
  cfg 2  DTS stereo refinement 1280x384: polygon guide, disparity planes in
         [0,128] + N(0,0.5), 20% uniform outliers, confidence exp(-|err|).
  cfg 3  64 ragged instances, W~U[256,1920], H~U[256,1080], cfg-0 guides,
         5% sparse targets with confidence 1.
  cfg 4  16 x 1024x768 cfg-0-style inputs plus an N(0,1) upstream gradient.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEED_BASE = 1000


@dataclass
class Instance:
    rgba: np.ndarray        # (H, W, 4) uint8
    target: np.ndarray      # (H, W) float32
    confidence: np.ndarray  # (H, W) float32
    labels: np.ndarray      # (H, W) int32 polygon id (0 = background)

    @property
    def width(self) -> int:
        return self.rgba.shape[1]

    @property
    def height(self) -> int:
        return self.rgba.shape[0]


def _convex_polygon(rng, w, h):
    k = int(rng.integers(3, 9))
    cx, cy = rng.uniform(0, w), rng.uniform(0, h)
    r = rng.uniform(0.05, 0.35) * min(w, h)
    pts = np.stack([cx + rng.uniform(-r, r, k), cy + rng.uniform(-r, r, k)], 1)
    # convex hull (monotone chain)
    pts = pts[np.lexsort((pts[:, 1], pts[:, 0]))]

    def cross(o, a, b):
        return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0])

    lower, upper = [], []
    for p in pts:
        while len(lower) >= 2 and cross(lower[-2], lower[-1], p) <= 0:
            lower.pop()
        lower.append(p)
    for p in pts[::-1]:
        while len(upper) >= 2 and cross(upper[-2], upper[-1], p) <= 0:
            upper.pop()
        upper.append(p)
    return np.array(lower[:-1] + upper[:-1])


def _poly_mask(hull, w, h):
    x0 = max(int(np.floor(hull[:, 0].min())), 0)
    x1 = min(int(np.ceil(hull[:, 0].max())) + 1, w)
    y0 = max(int(np.floor(hull[:, 1].min())), 0)
    y1 = min(int(np.ceil(hull[:, 1].max())) + 1, h)
    mask = np.zeros((h, w), bool)
    if x1 <= x0 or y1 <= y0 or len(hull) < 3:
        return mask
    yy, xx = np.mgrid[y0:y1, x0:x1]
    px, py = xx + 0.5, yy + 0.5
    inside = np.ones(px.shape, bool)
    n = len(hull)
    for i in range(n):
        ax, ay = hull[i]
        bx, by = hull[(i + 1) % n]
        inside &= (bx - ax) * (py - ay) - (by - ay) * (px - ax) >= 0
    mask[y0:y1, x0:x1] = inside
    return mask


def polygon_labels(rng, w, h, n_poly):
    labels = np.zeros((h, w), np.int32)
    for i in range(1, n_poly + 1):
        labels[_poly_mask(_convex_polygon(rng, w, h), w, h)] = i
    return labels


def _rgb_guide(rng, labels, n_poly, noise=3.0):
    colours = rng.integers(0, 256, (n_poly + 1, 3)).astype(np.float64)
    img = colours[labels] + rng.normal(0, noise, labels.shape + (3,))
    rgb = np.clip(np.rint(img), 0, 255).astype(np.uint8)
    a = np.full(labels.shape + (1,), 255, np.uint8)
    return np.ascontiguousarray(np.concatenate([rgb, a], axis=2))


def _planes(rng, labels, n_poly, lo, hi):
    h, w = labels.shape
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    a = rng.uniform(lo, hi, n_poly + 1)
    span = (hi - lo) / max(w, h)
    b = rng.uniform(-span, span, n_poly + 1)
    c = rng.uniform(-span, span, n_poly + 1)
    cx, cy = w / 2.0, h / 2.0
    z = a[labels] + b[labels] * (xx - cx) + c[labels] * (yy - cy)
    return np.clip(z, lo, hi)


def depth_sr_instance(seed: int, w: int = 640, h: int = 480, n_poly: int = 40,
                      stride: int = 8, sample_frac: float | None = None) -> Instance:
    """cfg 0 (and cfg 3 / cfg 4 instances).  stride: regular samples every
    `stride` px; sample_frac instead picks that fraction of pixels at random."""
    rng = np.random.default_rng(seed)
    labels = polygon_labels(rng, w, h, n_poly)
    rgba = _rgb_guide(rng, labels, n_poly)
    depth = _planes(rng, labels, n_poly, 0.5, 10.0)
    conf = np.zeros((h, w), np.float32)
    if sample_frac is None:
        conf[::stride, ::stride] = 1.0
    else:
        conf[rng.random((h, w)) < sample_frac] = 1.0
    noisy = depth + rng.normal(0, 0.01, depth.shape)
    target = np.where(conf > 0, noisy, 0.0).astype(np.float32)
    return Instance(rgba, target, conf, labels)


def colorization_instance(seed: int = SEED_BASE + 1, w: int = 640, h: int = 480,
                          n_poly: int = 30, frac: float = 0.02):
    """cfg 1: returns (instance with U target, V target)."""
    rng = np.random.default_rng(seed)
    labels = polygon_labels(rng, w, h, n_poly)
    h_, w_ = labels.shape
    yy, xx = np.mgrid[0:h_, 0:w_].astype(np.float64)
    base = rng.uniform(30, 225, n_poly + 1)
    gx = rng.uniform(-0.15, 0.15, n_poly + 1)
    gy = rng.uniform(-0.15, 0.15, n_poly + 1)
    grey = base[labels] + gx[labels] * (xx - w / 2) + gy[labels] * (yy - h / 2)
    grey = np.clip(np.rint(grey), 0, 255).astype(np.uint8)
    rgba = np.ascontiguousarray(
        np.stack([grey, grey, grey, np.full_like(grey, 255)], axis=2))
    u_val = rng.uniform(-0.5, 0.5, n_poly + 1)
    v_val = rng.uniform(-0.5, 0.5, n_poly + 1)
    mask = rng.random((h, w)) < frac
    conf = mask.astype(np.float32)
    u = np.where(mask, u_val[labels], 0.0).astype(np.float32)
    v = np.where(mask, v_val[labels], 0.0).astype(np.float32)
    return Instance(rgba, u, conf, labels), v


def stereo_instance(seed: int = SEED_BASE + 2, w: int = 1280, h: int = 384,
                    n_poly: int = 40) -> Instance:
    """cfg 2: initial disparity with noise and 20% outliers."""
    rng = np.random.default_rng(seed)
    labels = polygon_labels(rng, w, h, n_poly)
    rgba = _rgb_guide(rng, labels, n_poly)
    disp = _planes(rng, labels, n_poly, 0.0, 128.0)
    init = disp + rng.normal(0, 0.5, disp.shape)
    out = rng.random(disp.shape) < 0.2
    init = np.where(out, rng.uniform(0, 128, disp.shape), init)
    conf = np.exp(-np.abs(init - disp)).astype(np.float32)
    return Instance(rgba, init.astype(np.float32), conf, labels)


def batched_sizes(seed: int = SEED_BASE + 3, n: int = 64):
    rng = np.random.default_rng(seed)
    ws = rng.integers(256, 1921, n)
    hs = rng.integers(256, 1081, n)
    return [(int(a), int(b)) for a, b in zip(ws, hs)]


def batched_instances(seed: int = SEED_BASE + 3, n: int = 64, scale: float = 1.0,
                      indices=None):
    """cfg 3: n ragged instances (scale < 1 shrinks them for quick tests);
    indices: generate only these instances of the n (one rank's share)."""
    out = []
    for i, (w, h) in enumerate(batched_sizes(seed, n)):
        if indices is not None and i not in indices:
            continue
        w2, h2 = scaled_size(w, h, scale)
        out.append(depth_sr_instance(seed * 1000 + i, w2, h2, sample_frac=0.05))
    return out


def scaled_size(w: int, h: int, scale: float):
    return max(16, int(w * scale)), max(16, int(h * scale))


def grad_instances(seed: int = SEED_BASE + 4, n: int = 16, w: int = 1024, h: int = 768,
                   indices=None):
    """cfg 4: n cfg-0-style instances of w x h (samples every 8 px) and one
    N(0,1) upstream gradient dL/dv per instance; indices: only these."""
    keep = range(n) if indices is None else sorted(indices)
    insts = [depth_sr_instance(seed * 1000 + i, w, h) for i in keep]
    rng = np.random.default_rng(seed)
    grads = [rng.standard_normal((h, w)).astype(np.float32) for _ in range(n)]
    return insts, [grads[i] for i in keep]


# ---- solver parameters of each configuration -------------------------------
CFG0_FILTER = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.1)
CFG0_OPT = dict(num_iterations=10, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
CFG1_HFBS = dict(sigma_x=8.0, sigma_y=8.0, sigma_l=16.0, lambda_=8.0, alpha=1.0,
                 beta=0.9, bistoch_iter_max=20, optim_iter_max=64, neg_exp_beta=0.9)
CFG2_FILTER = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.1)
CFG2_OPT = dict(num_iterations=15, loss=2, lambda_=0.99, sigma_z=30.0, step_size=0.99)
