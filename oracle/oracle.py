"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() (as the checker) and bench.py's
cpu_baseline leg.  The product library never imports it.  See oracle.h.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"


def build(force: bool = False) -> None:
    libs = [BUILD / "liboracle_f64.so", BUILD / "liboracle_f32.so"]
    srcs = [HERE / "oracle.c", HERE / "oracle.h", HERE / "Makefile"]
    newest = max(p.stat().st_mtime for p in srcs)
    if not force and all(p.exists() and p.stat().st_mtime >= newest for p in libs):
        return
    r = subprocess.run(["make", "-C", str(HERE), "-B" if force else "-s"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


_libs: dict[str, ctypes.CDLL] = {}


class HfbsParams(ctypes.Structure):
    _fields_ = [("sigma_x", ctypes.c_float), ("sigma_y", ctypes.c_float),
                ("sigma_l", ctypes.c_float), ("lambda_", ctypes.c_float),
                ("alpha", ctypes.c_float), ("beta", ctypes.c_float),
                ("bistoch_iter_max", ctypes.c_int),
                ("optim_iter_max", ctypes.c_int),
                ("neg_exp_beta", ctypes.c_float), ("grid_x", ctypes.c_int),
                ("grid_y", ctypes.c_int), ("grid_l", ctypes.c_int)]


def lib(real: str = "f64") -> ctypes.CDLL:
    if real not in _libs:
        build()
        L = ctypes.CDLL(str(BUILD / f"liboracle_{real}.so"))
        vp, i, f, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_int64
        sigs = {
            "ora_real_bytes": ([], i),
            "ora_set_threads": ([i], None),
            "ora_get_threads": ([], i),
            "ora_color_convert": ([i, i, vp, vp, ll], None),
            "ora_dts_create": ([i, i], vp),
            "ora_dts_destroy": ([vp], None),
            "ora_dts_set_compat": ([vp, i, i], None),
            "ora_dts_set_image_dim": ([vp, i, i], i),
            "ora_dts_clear_all": ([vp], None),
            "ora_dts_init_frame": ([vp, i, vp, vp, vp], None),
            "ora_dts_set_target_conf": ([vp, vp, vp], None),
            "ora_dts_differential": ([vp, f, f, f], None),
            "ora_dts_integrate": ([vp], None),
            "ora_dts_filter": ([vp, f, f, f, vp, vp, i], None),
            "ora_dts_compute_confidence": ([vp, f, f, f, f, i], None),
            "ora_dts_optimize": ([vp, i, i, f, f, f, f], None),
            "ora_dts_init_right_frame": ([vp, f, i, vp], None),
            "ora_dts_process_right_frame": ([vp], None),
            "ora_dts_optimize_stereo": ([vp, i, i, f, f, f, f, f], None),
            "ora_dts_backward": ([vp, i, i, f, f, f, vp, vp, vp], i),
            "ora_dts_download": ([vp, i, vp], None),
            "ora_dts_bounds": ([vp, i, f, vp, vp, vp], None),
            "ora_dts_add_bounds_override": ([vp, i, f, vp, vp], None),
            "ora_dts_clear_bounds_override": ([vp], None),
            "ora_soft_solve": ([i, i, vp, vp, vp, vp, i, i, f, f, f, f, vp], None),
            "ora_soft_backward": ([i, i, vp, vp, vp, vp, i, i, f, f, f, f, vp, vp, vp, vp,
                                   vp], None),
            "ora_hfbs_create": ([i, i, i, i, i], vp),
            "ora_hfbs_destroy": ([vp], None),
            "ora_hfbs_set_compat": ([vp, i], None),
            "ora_hfbs_set_image_dim": ([vp, i, i], i),
            "ora_hfbs_set_params": ([vp, ctypes.POINTER(HfbsParams)], None),
            "ora_hfbs_clear_all": ([vp], None),
            "ora_hfbs_init_frame": ([vp, i, vp, vp, vp], None),
            "ora_hfbs_optimize": ([vp], i),
            "ora_hfbs_set_target_conf": ([vp, vp, vp], None),
            "ora_hfbs_backward": ([vp, vp, vp, vp], i),
            "ora_hfbs_download": ([vp, i, vp], None),
            "ora_hfbs_grid_dims": ([vp, ctypes.POINTER(i), ctypes.POINTER(i),
                                    ctypes.POINTER(i)], None),
            "ora_hfbs_grid": ([vp, i, vp], None),
        }
        for name, (args, res) in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _libs[real] = L
    return _libs[real]


def set_threads(n: int) -> int:
    """OpenMP worker threads of both builds (n <= 0: all host threads);
    returns the count now in effect."""
    for real in ("f64", "f32"):
        lib(real).ora_set_threads(int(n))
    return lib("f32").ora_get_threads()


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _dtype(real):
    return np.float64 if real == "f64" else np.float32


# Colour-conversion evaluation orders (oracle.c, a1).
CONTRACT_NONE, CONTRACT_NVCC, CONTRACT_NVCC_ALT = 0, 1, 2
DEFAULT_CONTRACT = CONTRACT_NVCC


def color_convert(color_space: int, rgba: np.ndarray, contract: int = DEFAULT_CONTRACT,
                  real: str = "f64") -> np.ndarray:
    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    out = np.empty_like(a)
    lib(real).ora_color_convert(int(color_space), int(contract), _p(a), _p(out),
                                a.size // 4)
    return out


class OracleDTS:
    """Mirror of DomainTransformFilter + DomainTransformSolver."""

    def __init__(self, max_w: int, max_h: int, real: str = "f64",
                 ref_y_limit: bool = True, contract: int = DEFAULT_CONTRACT):
        self.L = lib(real)
        self.real = real
        self.dt = _dtype(real)
        self.h = self.L.ora_dts_create(max_w, max_h)
        self.L.ora_dts_set_compat(self.h, int(ref_y_limit), int(contract))
        self.w, self.hh = max_w, max_h

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ora_dts_destroy(self.h)
            self.h = None

    def set_image_dim(self, w, h):
        if self.L.ora_dts_set_image_dim(self.h, w, h) == 0:
            self.w, self.hh = w, h

    def clear_all(self):
        self.L.ora_dts_clear_all(self.h)

    def init_frame(self, cs, rgba, target=None, conf=None):
        rgba = np.ascontiguousarray(rgba, np.uint8)
        t = None if target is None else np.ascontiguousarray(target, np.float32)
        c = None if conf is None else np.ascontiguousarray(conf, np.float32)
        self.L.ora_dts_init_frame(self.h, int(cs), _p(rgba), _p(t), _p(c))

    def set_target_conf(self, target=None, conf=None):
        """target / confidence at the oracle's precision (FP64 for "f64")."""
        t = None if target is None else np.ascontiguousarray(target, self.dt)
        c = None if conf is None else np.ascontiguousarray(conf, self.dt)
        self.L.ora_dts_set_target_conf(self.h, _p(t), _p(c))

    def differential(self, sx, sy, sr):
        self.L.ora_dts_differential(self.h, sx, sy, sr)

    def integrate(self):
        self.L.ora_dts_integrate(self.h)

    def filter(self, sx, sy, sr, inp, num_iter=3):
        inp = np.ascontiguousarray(inp, np.float32)
        out = np.empty((self.hh, self.w), self.dt)
        self.L.ora_dts_filter(self.h, sx, sy, sr, _p(inp), _p(out), num_iter)
        return out

    def compute_confidence(self, sx, sy, sr, sigma0, left_clear):
        self.L.ora_dts_compute_confidence(self.h, sx, sy, sr, sigma0, left_clear)

    def optimize(self, num_iterations, loss, lam, sigma_z, step, overwrite=-1.0):
        self.L.ora_dts_optimize(self.h, num_iterations, int(loss), lam, sigma_z,
                                step, overwrite)

    def init_right_frame(self, center_offset, cs, rgba):
        rgba = np.ascontiguousarray(rgba, np.uint8)
        self.L.ora_dts_init_right_frame(self.h, center_offset, int(cs), _p(rgba))

    def process_right_frame(self):
        self.L.ora_dts_process_right_frame(self.h)

    def optimize_stereo(self, num_iterations, loss, lam, sigma_z, step, photo_lambda,
                        overwrite=-1.0):
        self.L.ora_dts_optimize_stereo(self.h, num_iterations, int(loss), lam, sigma_z,
                                       step, photo_lambda, overwrite)

    def backward(self, num_iterations, loss, lam, sigma_z, step, grad_out):
        g = np.ascontiguousarray(grad_out, self.dt)
        gt = np.empty((self.hh, self.w), self.dt)
        gc = np.empty((self.hh, self.w), self.dt)
        st = self.L.ora_dts_backward(self.h, num_iterations, int(loss), lam, sigma_z, step,
                                     _p(g), _p(gt), _p(gc))
        if st != 0:
            raise ValueError("unsupported loss for the adjoint")
        return gt, gc

    def download(self, image_type):
        if image_type == 0:
            out = np.empty((self.hh, self.w, 4), np.uint8)
        else:
            out = np.empty((self.hh, self.w), self.dt)
        self.L.ora_dts_download(self.h, int(image_type), _p(out))
        return out

    def bounds(self, axis, sigma):
        l = np.empty((self.hh, self.w), np.int32)
        u = np.empty((self.hh, self.w), np.int32)
        m = np.empty((self.hh, self.w), self.dt)
        self.L.ora_dts_bounds(self.h, axis, sigma, _p(l), _p(u), _p(m))
        return l, u, m

    def add_bounds_override(self, axis, sigma, l, u):
        l = np.ascontiguousarray(l, np.int32)
        u = np.ascontiguousarray(u, np.int32)
        self.L.ora_dts_add_bounds_override(self.h, axis, sigma, _p(l), _p(u))

    def clear_bounds_override(self):
        self.L.ora_dts_clear_bounds_override(self.h)


GRID_NAMES = ["splat_sum", "splat_c", "b", "splat_norm", "inv_diag_A",
              "blur_c", "z_init", "z_final"]


class OracleHFBS:
    """Mirror of class HFBS."""

    def __init__(self, max_w, max_h, max_gx, max_gy, max_gl, real="f64",
                 contract: int = DEFAULT_CONTRACT):
        self.L = lib(real)
        self.dt = _dtype(real)
        self.h = self.L.ora_hfbs_create(max_w, max_h, max_gx, max_gy, max_gl)
        self.L.ora_hfbs_set_compat(self.h, int(contract))
        self.w, self.hh = max_w, max_h

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ora_hfbs_destroy(self.h)
            self.h = None

    def set_image_dim(self, w, h):
        if self.L.ora_hfbs_set_image_dim(self.h, w, h) == 0:
            self.w, self.hh = w, h

    def set_params(self, **kw):
        p = HfbsParams(8.0, 8.0, 4.0, 8.0, 1.0, 0.9, 20, 140, 0.9, 1, 1, 1)
        for k, v in kw.items():
            setattr(p, k, v)
        self.L.ora_hfbs_set_params(self.h, ctypes.byref(p))

    def clear_all(self):
        self.L.ora_hfbs_clear_all(self.h)

    def init_frame(self, cs, rgba, target, conf=None):
        rgba = np.ascontiguousarray(rgba, np.uint8)
        t = np.ascontiguousarray(target, np.float32)
        c = None if conf is None else np.ascontiguousarray(conf, np.float32)
        self.L.ora_hfbs_init_frame(self.h, int(cs), _p(rgba), _p(t), _p(c))

    def optimize(self) -> int:
        return self.L.ora_hfbs_optimize(self.h)

    def set_target_conf(self, target=None, conf=None):
        t = None if target is None else np.ascontiguousarray(target, self.dt)
        c = None if conf is None else np.ascontiguousarray(conf, self.dt)
        self.L.ora_hfbs_set_target_conf(self.h, _p(t), _p(c))

    def backward(self, grad_out):
        """dL/dtarget, dL/dconfidence of the last optimize for dL/doutput."""
        g = np.ascontiguousarray(grad_out, self.dt)
        gt = np.empty((self.hh, self.w), self.dt)
        gc = np.empty((self.hh, self.w), self.dt)
        if self.L.ora_hfbs_backward(self.h, _p(g), _p(gt), _p(gc)) != 0:
            raise ValueError("no completed optimize to differentiate")
        return gt, gc

    def download(self, image_type):
        out = np.empty((self.hh, self.w), self.dt)
        self.L.ora_hfbs_download(self.h, int(image_type), _p(out))
        return out

    def grid_dims(self):
        gx, gy, gl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.L.ora_hfbs_grid_dims(self.h, ctypes.byref(gx), ctypes.byref(gy),
                                  ctypes.byref(gl))
        return gx.value, gy.value, gl.value

    def grid(self, which):
        gx, gy, gl = self.grid_dims()
        out = np.zeros((gl, gy, gx), self.dt)
        self.L.ora_hfbs_grid(self.h, GRID_NAMES.index(which) if isinstance(which, str)
                             else which, _p(out))
        return out


# ---- soft-window DTS ---------------------------------------------------------
def soft_solve(eh, ev, t, c, opt, tau, real="f64"):
    """Soft-window Optimize from edge weights eh / ev (HxW), target t and
    confidence c (None: ones); opt as DomainOptimizeParams fields."""
    dt = _dtype(real)
    eh, ev, t = (np.ascontiguousarray(a, dt) for a in (eh, ev, t))
    c = None if c is None else np.ascontiguousarray(c, dt)
    h, w = t.shape
    out = np.empty((h, w), dt)
    lib(real).ora_soft_solve(w, h, _p(eh), _p(ev), _p(t), _p(c), opt["num_iterations"],
                             int(opt["loss"]), opt["lambda_"], opt["sigma_z"],
                             opt["step_size"], tau, _p(out))
    return out


def soft_backward(eh, ev, t, c, opt, tau, grad_out, real="f64"):
    """(dL/dt, dL/dc, dL/deh, dL/dev) of soft_solve for dL/dout."""
    dt = _dtype(real)
    eh, ev, t, g = (np.ascontiguousarray(a, dt) for a in (eh, ev, t, grad_out))
    c = None if c is None else np.ascontiguousarray(c, dt)
    h, w = t.shape
    outs = [np.empty((h, w), dt) for _ in range(4)]
    lib(real).ora_soft_backward(w, h, _p(eh), _p(ev), _p(t), _p(c), opt["num_iterations"],
                                int(opt["loss"]), opt["lambda_"], opt["sigma_z"],
                                opt["step_size"], tau, _p(g), *[_p(o) for o in outs])
    return tuple(outs)


def edge_weights(rgba, color_space, sigma_x, sigma_y, sigma_r, real="f64"):
    """dH, dV of the guide as ComputeColorSpaceDifferential computes them
    (through the DTS mirror's DIFFERENTIAL path)."""
    h, w = rgba.shape[:2]
    o = OracleDTS(w, h, real=real)
    o.init_frame(color_space, rgba)
    o.differential(sigma_x, sigma_y, sigma_r)
    dh = o.download(1)
    # dV: the same weights of the transposed guide along its rows
    ot = OracleDTS(h, w, real=real)
    ot.init_frame(color_space, np.ascontiguousarray(np.transpose(rgba, (1, 0, 2))))
    ot.differential(sigma_y, sigma_x, sigma_r)
    dv = np.ascontiguousarray(ot.download(1).T)
    return dh, dv


# ---- whole-solve conveniences ----------------------------------------------
def dts_solve(inst_rgba, target, conf, color_space, filt, opt, overwrite=-1.0,
              real="f64", ref_y_limit=True, overrides=None):
    """ClearAll -> InitFrame -> differential -> integrate -> Optimize.
    overrides: optional {(axis, sigma): (l, u)} windows to use instead of the
    oracle's own search."""
    h, w = target.shape
    o = OracleDTS(w, h, real=real, ref_y_limit=ref_y_limit)
    o.clear_all()
    o.init_frame(color_space, inst_rgba, target, conf)
    o.differential(filt["sigma_x"], filt["sigma_y"], filt["sigma_r"])
    o.integrate()
    for (axis, sigma), (l, u) in (overrides or {}).items():
        o.add_bounds_override(axis, sigma, l, u)
    o.optimize(opt["num_iterations"], opt["loss"], opt["lambda_"], opt["sigma_z"],
               opt["step_size"], overwrite)
    return o.download(5), o


def hfbs_solve(rgba, target, conf, color_space, params, max_grid=None, real="f64"):
    h, w = target.shape
    gx, gy, gl = max_grid or (w, h, 64)
    o = OracleHFBS(w, h, gx, gy, gl, real=real)
    o.clear_all()
    o.set_params(**params)
    o.init_frame(color_space, rgba, target, conf)
    status = o.optimize()
    return o.download(5), o, status
