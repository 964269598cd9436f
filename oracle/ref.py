"""ctypes binding of the reference's own DTS / HFBS sources compiled for the
CPU (oracle/refemu/build_ref.py) -- TEST INFRASTRUCTURE ONLY.

It exists where the reference checkout exists (the build reads its
sources in place); tests/golden/make_ref_golden.py runs it to write the
golden vectors that pin the oracle and the GPU path, and the CPU tests
re-run it against those vectors when the checkout is present.
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "refemu"))
import build_ref  # noqa: E402

_lib = None


def available() -> bool:
    return build_ref.DEFAULT_SRC.is_dir()


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = build_ref.build()
        L = ctypes.CDLL(str(path))
        vp, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.dtsref_dts_solve.argtypes = [i, i, i, vp, vp, vp, f, f, f, vp, i, i, f, f, f, f,
                                       vp, vp, vp, vp, vp, vp, vp, vp]
        L.dtsref_filter.argtypes = [i, i, i, vp, f, f, f, vp, i, vp, vp]
        L.dtsref_stereo_solve.argtypes = [i, i, i, vp, vp, f, vp, vp, f, f, f, i, i, f, f,
                                          f, f, f, vp]
        L.dtsref_hfbs_solve.argtypes = [i, i, i, vp, vp, vp, vp, vp, i, i, i, vp, vp, vp]
        L.dtsref_color_convert.argtypes = [i, i, i, vp]
        for fn in ("dtsref_dts_solve", "dtsref_filter", "dtsref_stereo_solve",
                   "dtsref_hfbs_solve", "dtsref_color_convert"):
            getattr(L, fn).restype = i
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def dts_solve(rgba, target, conf, color_space, filt, opt, overwrite=-1.0,
              conf_params=(8.0, 8.0, 0.1, 1.0)):
    """The reference's Solve<DtsOptions> (conf None: its confidence
    estimate runs first).  Returns a dict of result, color, dH, dV, ctH,
    ctV, conf and bounds (h, w, 4: X lower/upper, Y lower/upper)."""
    h, w = target.shape
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    t, c = _f32(target), _f32(conf)
    out = {k: np.zeros((h, w), np.float32) for k in ("result", "dH", "dV", "ctH", "ctV", "conf")}
    out["color"] = np.zeros((h, w, 4), np.uint8)
    out["bounds"] = np.zeros((h, w, 4), np.int32)
    cp = np.asarray(conf_params, np.float32)
    rc = lib().dtsref_dts_solve(
        w, h, int(color_space), _p(rgba), _p(t), _p(c), filt["sigma_x"], filt["sigma_y"],
        filt["sigma_r"], _p(cp), opt["num_iterations"], int(opt["loss"]), opt["lambda_"],
        opt["sigma_z"], opt["step_size"], overwrite, _p(out["result"]), _p(out["color"]),
        _p(out["dH"]), _p(out["dV"]), _p(out["ctH"]), _p(out["ctV"]), _p(out["conf"]),
        _p(out["bounds"]))
    if rc != 0:
        raise ValueError("the reference needs images of at least 128x128")
    return out


def color_convert(color_space, rgba):
    """The reference's colour conversion kernel on an (h, w, 4) image."""
    out = np.array(rgba, dtype=np.uint8, order="C", copy=True)
    h, w = out.shape[:2]
    lib().dtsref_color_convert(w, h, int(color_space), _p(out))
    return out


def filter(rgba, color_space, sx, sy, sr, inp, num_iter=3, with_bounds=False):
    """DomainTransformFilter::Filter; with_bounds: also each pass's windows
    as (num_iter, h, w, 4) (X lower/upper, Y lower/upper)."""
    h, w = inp.shape
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    x = _f32(inp)
    out = np.zeros((h, w), np.float32)
    b = np.zeros((num_iter, h, w, 4), np.int32) if with_bounds else None
    if lib().dtsref_filter(w, h, int(color_space), _p(rgba), sx, sy, sr, _p(x), num_iter,
                           _p(out), _p(b)) != 0:
        raise ValueError("the reference needs images of at least 128x128")
    return (out, b) if with_bounds else out


def stereo_solve(left, right, center_offset, target, conf, color_space, filt, opt):
    h, w = target.shape
    left = np.ascontiguousarray(left, dtype=np.uint8)
    right = np.ascontiguousarray(right, dtype=np.uint8)
    t, c = _f32(target), _f32(conf)
    out = np.zeros((h, w), np.float32)
    if lib().dtsref_stereo_solve(
            w, h, int(color_space), _p(left), _p(right), center_offset, _p(t), _p(c),
            filt["sigma_x"], filt["sigma_y"], filt["sigma_r"], opt["num_iterations"],
            int(opt["loss"]), opt["lambda_"], opt["sigma_z"], opt["step_size"],
            opt["photo_consis_lambda"], opt["DT_lambda"], _p(out)) != 0:
        raise ValueError("the reference needs images of at least 128x128")
    return out


def hfbs_solve(rgba, target, conf, color_space, params, max_grid):
    """HFBS::Optimize.  params: sigma_x, sigma_y, sigma_l, lambda_, alpha,
    beta, neg_exp_beta, bistoch_iter_max, optim_iter_max.  Returns (result,
    grids dict of splat_sum / splat_norm / inv_diag_A / b / z as
    (max_gl, max_gy, max_gx) arrays or None if the grid was too large,
    (grid_x, grid_y, grid_l))."""
    h, w = target.shape
    gx, gy, gl = max_grid
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    t, c = _f32(target), _f32(conf)
    pf = np.asarray([params[k] for k in ("sigma_x", "sigma_y", "sigma_l", "lambda_", "alpha",
                                         "beta", "neg_exp_beta")], np.float32)
    pi = np.asarray([params["bistoch_iter_max"], params["optim_iter_max"]], np.int32)
    out = np.zeros((h, w), np.float32)
    grids = np.zeros((5, gl, gy, gx), np.float32)
    dims = np.zeros(3, np.int32)
    rc = lib().dtsref_hfbs_solve(w, h, int(color_space), _p(rgba), _p(t), _p(c), _p(pf),
                                 _p(pi), gx, gy, gl, _p(out), _p(grids), _p(dims))
    names = ("splat_sum", "splat_norm", "inv_diag_A", "b", "z")
    g = None if rc == 1 else {n: grids[k] for k, n in enumerate(names)}
    return out, g, tuple(int(v) for v in dims)
