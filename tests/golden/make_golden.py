"""Writes the golden fixtures of tests/test_golden.py: seeded inputs and the
FP64 oracle's outputs for one small case of each part of the path.

    python tests/golden/make_golden.py

The reference publishes no numeric vectors (its tests only smoke-run the
solvers), so these pin the oracle against later changes and give the GPU
tests fixed expected outputs.  The DTS case uses the first seed whose window
decisions all lie at least 3e-4 from their thresholds, so that the GPU's
window search must match the oracle's exactly.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle as O  # noqa: E402
from domain_transform_solver_gb300 import workloads as W  # noqa: E402

DTS_FILTER = dict(W.CFG0_FILTER)
DTS_OPT = dict(W.CFG0_OPT, num_iterations=5)
HFBS = dict(W.CFG1_HFBS, optim_iter_max=24)
HFBS_GRID = (12, 8, 32)  # max grid: the overflow bin stored, pad faces covered
MARGIN = 3e-4


def dts_case():
    sz = DTS_OPT["sigma_z"]
    for seed in range(100, 200):
        inst = W.depth_sr_instance(seed, 96, 64, n_poly=6, stride=4)
        o = O.OracleDTS(96, 64)
        o.init_frame(1, inst.rgba, inst.target, inst.confidence)
        o.differential(DTS_FILTER["sigma_x"], DTS_FILTER["sigma_y"], DTS_FILTER["sigma_r"])
        o.integrate()
        b = [o.bounds(a, sz) for a in (0, 1)]
        # the GPU's fixed-point window sums are within ~2e-5 of FP64: keep
        # every window decision at least 3e-4 from its threshold
        if min(float(np.abs(m).min()) for _, _, m in b) <= MARGIN:
            continue
        o.optimize(DTS_OPT["num_iterations"], DTS_OPT["loss"], DTS_OPT["lambda_"], sz,
                   DTS_OPT["step_size"])
        v = o.download(5)
        return dict(seed=seed, rgba=inst.rgba, target=inst.target,
                    confidence=inst.confidence, lx=b[0][0], ux=b[0][1], ly=b[1][0],
                    uy=b[1][1], v=v)
    raise RuntimeError("no seed without near-ties")


def hfbs_case():
    u, _ = W.colorization_instance(31, 96, 64, n_poly=5, frac=0.05)
    rng = np.random.default_rng(32)
    c = rng.random(u.target.shape).astype(np.float32)
    g = rng.standard_normal(u.target.shape).astype(np.float32)
    o = O.OracleHFBS(96, 64, *HFBS_GRID)
    o.clear_all()
    o.init_frame(0, u.rgba, u.target, c)
    o.set_params(**HFBS)
    assert o.optimize() == 0
    out = o.download(5)
    gt, gc = o.backward(g.astype(np.float64))
    return dict(rgba=u.rgba, target=u.target, confidence=c, out=out,
                count=o.grid("splat_sum"), grad_out=g, grad_target=gt, grad_confidence=gc)


def color_case():
    rng = np.random.default_rng(33)
    rgba = rng.integers(0, 256, (64, 64, 4)).astype(np.uint8)
    rgba[0, :8] = [[0, 0, 0, 0], [255, 255, 255, 255], [255, 0, 0, 7], [0, 255, 0, 9],
                   [0, 0, 255, 11], [128, 128, 128, 128], [1, 2, 3, 4], [254, 253, 252, 251]]
    return dict(rgba=rgba, ycbcr=O.color_convert(1, rgba), yyy=O.color_convert(2, rgba))


def main():
    O.build()
    np.savez_compressed(HERE / "dts_depth_sr_96x64.npz", **dts_case())
    np.savez_compressed(HERE / "hfbs_colorization_96x64.npz", **hfbs_case())
    np.savez_compressed(HERE / "color_64x64.npz", **color_case())


if __name__ == "__main__":
    main()
