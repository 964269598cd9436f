"""Writes the reference-output fixtures tests/golden/ref_*.npz: seeded inputs
and what the reference's own DTS / HFBS sources compute for them, built for
the CPU by oracle/refemu/build_ref.py from the reference checkout.

    python tests/golden/make_ref_golden.py

These pin the oracle (tests/test_ref_pin.py, CPU) and the GPU path
(tests/test_gpu_ref_pin.py) to the reference's code rather than to a
restatement of it.  Image sizes avoid the reads the reference makes outside
its images whose values depend on allocation padding (both sides at least
128 -- its row scan's minimum -- neither a multiple of 128 floats, and the
width within the padded height); HFBS grids are allocated larger than the
grid in use, as the reference's CLIs allocate them.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import ref as R  # noqa: E402
from domain_transform_solver_gb300 import workloads as W  # noqa: E402

CONF_PARAMS = (8.0, 8.0, 0.1, 1.0)  # sigma_x, sigma_y, sigma_r, sigmas[0]


def _dts_case(name, inst_rgba, target, conf, cs, filt, opt, overwrite=-1.0, planes=False):
    r = R.dts_solve(inst_rgba, target, conf, cs, filt, opt, overwrite, CONF_PARAMS)
    one = R.dts_solve(inst_rgba, target, conf, cs, filt, dict(opt, num_iterations=1),
                      overwrite, CONF_PARAMS)
    meta = dict(kind="dts", color_space=cs, filter=filt, optimize=opt, overwrite=overwrite,
                conf_params=CONF_PARAMS, auto_confidence=conf is None)
    out = dict(rgba=inst_rgba, target=target, result=r["result"],
               result_1iter=one["result"], color=r["color"],
               bounds=r["bounds"].astype(np.int16), meta=json.dumps(meta))
    if planes:  # the integrands, for one case
        out["dH"], out["dV"] = r["dH"], r["dV"]
    if conf is not None:
        out["confidence"] = conf
    else:
        out["conf_used"] = r["conf"]
    return name, out


def dts_cases():
    a = W.depth_sr_instance(2001, 200, 150, n_poly=10, sample_frac=0.2)
    yield _dts_case("dts_l2_ycbcr_200x150", a.rgba, a.target, a.confidence, 1,
                    W.CFG0_FILTER, W.CFG0_OPT, planes=True)
    b = W.stereo_instance(2002, 150, 200, n_poly=8)
    yield _dts_case("dts_charbonnier_rgb_overwrite_150x200", b.rgba, b.target, b.confidence, 0,
                    dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.2),
                    dict(num_iterations=5, loss=2, lambda_=0.99, sigma_z=20.0,
                         step_size=0.99), overwrite=0.5)
    c = W.depth_sr_instance(2003, 220, 140, n_poly=8, sample_frac=0.3)
    yield _dts_case("dts_auto_confidence_yyy_220x140", c.rgba, c.target, None, 2,
                    W.CFG0_FILTER, dict(W.CFG0_OPT, num_iterations=4))


def filter_case():
    a = W.depth_sr_instance(2004, 180, 130, n_poly=8)
    x = np.random.default_rng(2004).random((130, 180)).astype(np.float32)
    out, b = R.filter(a.rgba, 1, 6.0, 6.0, 0.15, x, 3, with_bounds=True)
    meta = dict(kind="filter", color_space=1, sigma_x=6.0, sigma_y=6.0, sigma_r=0.15,
                num_iter=3)
    return "filter_ycbcr_180x130", dict(rgba=a.rgba, input=x, output=out,
                                        bounds=b.astype(np.int16), meta=json.dumps(meta))


def stereo_case():
    inst = W.stereo_instance(2005, 190, 130, n_poly=10)
    rng = np.random.default_rng(2005)
    left = inst.rgba
    right = np.roll(left, -6, axis=1).copy()
    right[..., :3] = np.clip(right[..., :3].astype(int) + rng.integers(-3, 4, right[..., :3].shape),
                             0, 255).astype(np.uint8)
    t = (rng.integers(3, 10, (130, 190)) + 0.5 + rng.uniform(-0.2, 0.2, (130, 190))).astype(np.float32)
    c = (rng.integers(0, 256, (130, 190)) / 255.0).astype(np.float32)
    filt = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.2)
    d = dict(left=left, right=right, target=t, confidence=c)
    opts = []
    for loss in (1, 2):
        opt = dict(num_iterations=1, loss=loss, lambda_=0.99, sigma_z=12.0, step_size=0.99,
                   photo_consis_lambda=0.5, DT_lambda=0.2)
        d[f"result_loss{loss}"] = R.stereo_solve(left, right, 2.0, t, c, 1, filt, opt)
        opts.append(opt)
    d["meta"] = json.dumps(dict(kind="stereo", color_space=1, center_offset=2.0, filter=filt,
                                optimize=opts))
    return "stereo_190x130", d


def _hfbs_case(name, rgba, target, conf, cs, params, max_grid):
    out, grids, dims = R.hfbs_solve(rgba, target, conf, cs, params, max_grid)
    gx, gy, gl = dims
    meta = dict(kind="hfbs", color_space=cs, params=params, max_grid=list(max_grid),
                grid=list(dims))
    d = dict(rgba=rgba, target=target, result=out, meta=json.dumps(meta))
    if conf is not None:
        d["confidence"] = conf
    for k in ("splat_sum", "splat_norm", "inv_diag_A", "z"):
        d[k] = grids[k][:gl, :gy, :gx].copy()
    return name, d


def hfbs_cases():
    u, v = W.colorization_instance(2006, 200, 150, n_poly=6, frac=0.05)
    yield _hfbs_case("hfbs_colorization_u_200x150", u.rgba, u.target, u.confidence, 2,
                     dict(W.CFG1_HFBS), (200, 150, 64))
    yield _hfbs_case("hfbs_overflow_bin_200x150", u.rgba, v, u.confidence, 2,
                     dict(W.CFG1_HFBS, sigma_l=5.0, optim_iter_max=30), (200, 150, 64))
    d = W.depth_sr_instance(2007, 240, 180, n_poly=12)
    yield _hfbs_case("hfbs_depth_clamp_default_conf_240x180", d.rgba,
                     ((d.target - 5) * 12.8).astype(np.float32), None, 1,
                     dict(W.CFG1_HFBS, optim_iter_max=40), (240, 180, 64))
    rng = np.random.default_rng(2008)
    g = rng.integers(0, 256, (30, 70, 4)).astype(np.uint8)
    g[..., 3] = 255
    g[0, :5, 0] = 255
    t = rng.uniform(-0.5, 0.5, (30, 70)).astype(np.float32)
    c = (rng.random((30, 70)) < 0.4).astype(np.float32)
    yield _hfbs_case("hfbs_pad_faces_70x30", g, t, c, 0,
                     dict(W.CFG1_HFBS, sigma_l=40.0, bistoch_iter_max=9, optim_iter_max=17),
                     (64, 64, 64))


def color_case():
    rng = np.random.default_rng(2009)
    rgba = rng.integers(0, 256, (128, 128, 4)).astype(np.uint8)
    return "color_128x128", dict(rgba=rgba, ycbcr=R.color_convert(1, rgba),
                                 yyy=R.color_convert(2, rgba), meta=json.dumps(dict(kind="color")))


def all_cases():
    yield from dts_cases()
    yield filter_case()
    yield stereo_case()
    yield from hfbs_cases()
    yield color_case()


def main():
    for name, d in all_cases():
        path = HERE / f"ref_{name}.npz"
        np.savez_compressed(path, **d)
        print(f"{path.name}: {path.stat().st_size // 1024} KB")


if __name__ == "__main__":
    main()
