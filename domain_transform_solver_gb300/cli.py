"""Benchmark drivers with the reference CLIs' flags and output lines, without
OpenCV or gflags:

    python -m domain_transform_solver_gb300.cli depth_super_res \\
        --path_to_data_top_dir DIR [--algorithm_name dts|hfbs] \\
        [--algorithm_input_name bicubic]
    python -m domain_transform_solver_gb300.cli stereo --path_to_data_top_dir DIR
    python -m domain_transform_solver_gb300.cli colorization \\
        --path_to_data_top_dir DIR [--algorithm_name dts|hfbs]

depth_super_res follows src/benchmark_depth_super_res_cli.cpp and
src/depth_super_res_dataset.h: the twelve images of the Barron/Poole depth
super-resolution layout (three scenes x four upsampling levels), DTS or HFBS
with that CLI's options, the result written back as an 8-bit PNG under
DIR/<algorithm_name>/.  stereo follows src/benchmark_stereo_cli.cpp: the
Middlebury "Art" layout (im0/im1 PNG, im0.png_disp.bin initialisation,
calib.txt doff, disp0GT.pfm ground truth), DomainTransformStereo with
ComputeConfidence, the result written as DIR/dts_<scene>.png.
colorization follows src/benchmark_colorization_cli.cpp: BMP grey image,
scribbles and ground truth per image, Cb and Cr solved separately (DTS with
the 0.85 confidence overwrite, or HFBS), SSIM and PSNR lines per image.  All
print
"Using ... algorithm." and "RMSE <geometric mean>, time <ms> ms, num_pixels
<n>" like the reference (src/benchmark_util.h: BenchmarkResult).  The time
is the host wall time of the solve and the blocking download of its result.
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

from . import imageio as IO
from . import solvers as S


def rms_error(gt: np.ndarray, res: np.ndarray) -> float:
    """RMSError (src/benchmark_util.h): sqrt(||gt - res||^2 / #values)."""
    d = gt.astype(np.float64) - res.astype(np.float64)
    return math.sqrt(float(np.sum(d * d)) / d.size)


class Result:
    """BenchmarkResult<N>: geometric-mean RMSE, mean time and pixels."""

    def __init__(self, n: int):
        self.n = n
        self.log_rmse = np.zeros(n)
        self.time = np.zeros(n)
        self.pixels = np.zeros(n)

    def add(self, i: int, rmse: float, ms: float, px: int) -> None:
        self.log_rmse[i] += math.log(rmse) if rmse > 0 else -math.inf
        self.time[i] += ms
        self.pixels[i] += px

    def line(self, trials: int = 1) -> str:
        k = self.n * trials
        return (f"RMSE {math.exp(self.log_rmse.sum() / k):g}, time {self.time.sum() / k:g} "
                f"ms, num_pixels {self.pixels.sum() / k:g}")


def _to_uint8(v: np.ndarray, scale: float) -> np.ndarray:
    """convertTo(CV_8UC1, scale): round to nearest (ties to even), saturate."""
    return np.clip(np.rint(v.astype(np.float64) * scale), 0, 255).astype(np.uint8)


def _timed(fn):
    """Wall time in ms of fn, which ends with a blocking download."""
    import time
    t0 = time.perf_counter()
    fn()
    return (time.perf_counter() - t0) * 1e3


# ---- depth super-resolution ------------------------------------------------------
FOLDERS = ["art_big", "books_big", "moebius_big"]
OUTPUTS = ["output_1_n", "output_2_n", "output_3_n", "output_4_n"]
WEIGHTS = ["weight_1_n", "weight_2_n", "weight_3_n", "weight_4_n"]
_SCALE16 = 1.0 / (256.0 * 256.0 - 1)


def depth_super_res(top: str, algorithm: str, init_name: str, out=None,
                    err=None) -> Result:
    out = out or sys.stdout
    err = err or sys.stderr
    if algorithm not in ("dts", "hfbs"):
        print("Unsupported algorithm.", file=err)
        raise SystemExit(-1)
    print(f"Using {algorithm} algorithm.", file=out)
    max_dim = S.ImageDim(1536, 1536)
    if algorithm == "dts":
        solver = S.DomainTransformSolver(max_dim)
    else:
        solver = S.HFBS(max_dim, max_dim.width, max_dim.height, 64)
    res = Result(len(FOLDERS) * len(OUTPUTS))
    k = 0
    for folder in FOLDERS:
        for level, (oname, wname) in enumerate(zip(OUTPUTS, WEIGHTS)):
            up = 2 ** (level + 1)
            rgba = IO.read_rgba(os.path.join(top, "_input", folder, folder + "_color.png"))
            target = IO.read_float_16bit(os.path.join(top, init_name, folder, oname + ".png"),
                                         _SCALE16)
            gt = IO.read_gray(os.path.join(top, "_gth", folder + ".png"))
            bump = IO.read_float_16bit(os.path.join(top, "weights", folder, wname + ".png"),
                                       _SCALE16)
            conf = (bump / bump.max()).astype(np.float32)
            h, w = target.shape
            dims = S.ImageDim(w, h)
            if algorithm == "dts":
                opt = S.DtsOptions(
                    filter_options=S.DomainFilterParams(8.0 * up, 8.0 * up, 0.1),
                    optim_options=S.DomainOptimizeParams(
                        num_iterations=10, loss=S.RobustLoss.L2, lambda_=0.99,
                        sigma_z=8.0 * up / (1 + 0.2 * 4), step_size=0.99,
                        photo_consis_lambda=0.02),
                    conf_params=S.DomainFilterParamsVec1(8.0, 8.0, 0.2, [16.0, 0.0]),
                    color_space=S.COLOR_SPACE.YCbCr, image_dims=dims)
                t_in = target
            else:
                opt = S.HfbsOptions(
                    grid_params=S.HFBSGridParams(sigma_x=8.0 * up, sigma_y=8.0 * up,
                                                 sigma_l=16.0),
                    color_space=S.COLOR_SPACE.YCbCr, image_dims=dims)
                t_in = ((target - 0.5) * 128).astype(np.float32)
            result = {}

            def run():
                result["v"], _ = S.EdgeAwareOptimize(rgba, t_in, conf, opt, solver)

            ms = _timed(run)
            v = result["v"]
            if algorithm == "hfbs":
                v = v / 128.0 + 0.5
            v8 = _to_uint8(v, 255.0)
            res.add(k, rms_error(gt, v8), ms, h * w)
            os.makedirs(os.path.join(top, algorithm, folder), exist_ok=True)
            IO.write_png(os.path.join(top, algorithm, folder, oname + ".png"), v8)
            k += 1
    print(res.line(), file=err)
    return res


# ---- stereo ------------------------------------------------------------------
def _read_doff(path: str) -> int:
    """ReadDoffFromFile: the first token of the third line, 'doff=<int>'."""
    try:
        with open(path) as f:
            lines = f.read().split("\n")
        tok = lines[2].split()[0].split("=")
        return int(tok[1]) if len(tok) == 2 else 0
    except (OSError, IndexError, ValueError):
        print(f"Could not open calibration file at {path}", file=sys.stderr)
        return 0


def stereo(top: str, out=None, err=None) -> Result:
    out = out or sys.stdout
    err = err or sys.stderr
    print("Using DTS algorithm.", file=out)
    scene = "Art"
    d = os.path.join(top, scene)
    left = IO.read_rgba(os.path.join(d, "im0.png"))
    right = IO.read_rgba(os.path.join(d, "im1.png"))
    h, w = left.shape[:2]
    target = IO.read_disparity_bin(os.path.join(d, "im0.png_disp.bin"), w, h)
    doff = _read_doff(os.path.join(d, "calib.txt"))
    gt = IO.read_pfm(os.path.join(d, "disp0GT.pfm"))[::-1].copy()  # stored bottom-up
    gt[np.isinf(gt)] = 0
    solver = S.DomainTransformStereo(S.ImageDim(768, 768))
    filt = S.DomainFilterParams(8.0, 8.0, 0.1)
    optp = S.DomainOptimizeParams(num_iterations=1, loss=S.RobustLoss.CHARBONNIER,
                                  lambda_=0.99, sigma_z=30.0, step_size=0.99,
                                  photo_consis_lambda=0.01, DT_lambda=0.0)
    conf = S.DomainFilterParamsVec1(8.0, 8.0, 0.2, [16.0, 0.0])
    solver.SetImageDim(S.ImageDim(w, h))
    solver.ClearAll()
    solver.InitFrame(S.COLOR_SPACE.RGB, left, target, None)
    solver.InitRightFrame(float(doff), S.COLOR_SPACE.RGB, right)

    def run():
        solver.ComputeConfidence(conf, 20)
        solver.ComputeColorSpaceDifferential(filt)
        solver.IntegrateColorDifferentials()
        solver.ProcessRightFrame()
        solver.Optimize(optp, -1.0)
        result["v"] = solver.Download(S.ImageType.OPTIMIZED_QUANTITY)

    result = {}
    ms = _timed(run)
    v = result["v"]
    res = Result(1)
    res.add(0, rms_error(gt, v), ms, h * w)
    IO.write_png(os.path.join(top, f"dts_{scene}.png"), _to_uint8(v, 1.0))
    print(res.line(), file=err)
    return res


# ---- colorization ---------------------------------------------------------------
COLOR_IMAGES = ["IMG_3743", "IMG_3748"]


def bgr_to_ycbcr_planes(bgr: np.ndarray):
    """BGR2YCbCr (float planes) of src/benchmark_colorization_cli.cpp."""
    b, g, r = (bgr[..., k].astype(np.float32) for k in range(3))
    f = np.float32
    y = f(0.299) * r + f(0.587) * g + f(0.114) * b
    cb = f(128) - f(0.168736) * r - f(0.331264) * g + f(0.5) * b
    cr = f(128) + f(0.5) * r - f(0.418688) * g - f(0.081312) * b
    return y, cb, cr


def bgr_to_ycbcr_u8(bgr: np.ndarray) -> np.ndarray:
    """BGR2YCbCr into an 8-bit image: each float converts by truncation."""
    return np.stack([p.astype(np.uint8) for p in bgr_to_ycbcr_planes(bgr)], axis=-1)


def ycbcr_to_bgr(y, cb, cr) -> np.ndarray:
    """YCbCrBGR: rounded and clamped to [0, 255]."""
    f = np.float32
    r = y + f(1.402) * (cr - 128)
    g = (y - f(0.344136) * (cb - 128)).astype(np.float64) - 0.714136 * (cr - 128)
    b = y + f(1.772) * (cb - 128)
    out = [np.clip(np.where(v > 255, 255, np.where(v < 0, 0, np.round(v))), 0, 255)
           for v in (b, g, r)]
    return np.stack(out, axis=-1).astype(np.uint8)


def _gaussian_blur(img: np.ndarray, ksize: int = 11, sigma: float = 1.5) -> np.ndarray:
    """cv::GaussianBlur on float planes: separable, BORDER_REFLECT_101."""
    r = ksize // 2
    k = np.exp(-((np.arange(ksize) - r) ** 2) / (2 * sigma * sigma))
    k = (k / k.sum()).astype(np.float32)
    pad = np.pad(img, [(r, r), (r, r)] + [(0, 0)] * (img.ndim - 2), mode="reflect")
    tmp = sum(k[i] * pad[:, i:i + img.shape[1]] for i in range(ksize))
    return sum(k[i] * tmp[i:i + img.shape[0]] for i in range(ksize)).astype(np.float32)


def ssim(a: np.ndarray, b: np.ndarray):
    """SSIM of the colorization driver: per-channel mean SSIM map."""
    c1, c2 = (0.01 * 255) ** 2, (0.03 * 255) ** 2
    a = a.astype(np.float32)
    b = b.astype(np.float32)
    mu1, mu2 = _gaussian_blur(a), _gaussian_blur(b)
    s11 = _gaussian_blur(a * a) - mu1 * mu1
    s22 = _gaussian_blur(b * b) - mu2 * mu2
    s12 = _gaussian_blur(a * b) - mu1 * mu2
    m = ((2 * mu1 * mu2 + c1) * (2 * s12 + c2)) / ((mu1 * mu1 + mu2 * mu2 + c1) * (s11 + s22 + c2))
    return [float(m[..., k].mean()) for k in range(m.shape[-1])]


def psnr(gt: np.ndarray, test: np.ndarray) -> float:
    """PSNR of the driver: 20 log10(255) - 10 log10(RMSE) (as written there)."""
    return 20 * math.log10(255) - 10 * math.log10(rms_error(gt, test))


def colorization(top: str, algorithm: str, out=None, err=None) -> Result:
    out = out or sys.stdout
    err = err or sys.stderr
    if algorithm not in ("dts", "hfbs"):
        print("Unsupported algorithm.", file=err)
        raise SystemExit(-1)
    print(f"Using {algorithm} algorithm.", file=out)
    max_dim = S.ImageDim(3280, 3280)
    if algorithm == "dts":
        solver = S.DomainTransformSolver(max_dim)
    else:
        g = math.ceil(3280.0 / 8)
        solver = S.HFBS(max_dim, g, g, 64)
    res = Result(len(COLOR_IMAGES))
    for k, name in enumerate(COLOR_IMAGES):
        gray = IO.read_bmp(os.path.join(top, name + ".bmp"))[..., 0]
        yyya = np.empty(gray.shape + (4,), np.uint8)
        yyya[..., :3] = gray[..., None]
        yyya[..., 3] = 0  # mixChannels from a one-channel source: -1 fills 0
        _, cb_t, cr_t = bgr_to_ycbcr_planes(IO.read_bmp(os.path.join(top, name + "_strokes.bmp")))
        cb8, cr8 = cb_t.astype(np.uint8), cr_t.astype(np.uint8)
        marked = (cb8 > 129) | (cb8 < 127) | (cr8 > 129) | (cr8 < 127)
        conf = marked.astype(np.float32)
        gt = bgr_to_ycbcr_u8(IO.read_bmp(os.path.join(top, name + "_gt.bmp")))
        h, w = gray.shape
        dims = S.ImageDim(w, h)
        if algorithm == "dts":
            opt = S.DtsOptions(
                filter_options=S.DomainFilterParams(64.0, 64.0, 0.25),
                optim_options=S.DomainOptimizeParams(
                    num_iterations=10, loss=S.RobustLoss.CHARBONNIER, lambda_=0.99,
                    sigma_z=30.0, step_size=0.99, photo_consis_lambda=0.0, DT_lambda=0.0),
                conf_params=S.DomainFilterParamsVec1(8.0, 8.0, 0.2, [16.0, 0.0]),
                color_space=S.COLOR_SPACE.RGB, image_dims=dims,
                overwrite_target_above_conf=0.85)
        else:
            opt = S.HfbsOptions(
                grid_params=S.HFBSGridParams(sigma_x=8.0, sigma_y=8.0, sigma_l=4.0,
                                             optim_iter_max=140, bistoch_iter_max=20,
                                             lambda_=8.0),
                color_space=S.COLOR_SPACE.RGB, image_dims=dims)
        est, ms = [], 0.0
        for t in (cb_t, cr_t):
            c = conf
            if algorithm == "hfbs":
                t = (t - 128).astype(np.float32)
                c = (conf * 110000000164).astype(np.float32)
            result = {}

            def run():
                result["v"], _ = S.EdgeAwareOptimize(yyya, t, c, opt, solver)

            ms += _timed(run)
            v = result["v"]
            est.append(v + 128 if algorithm == "hfbs" else v)
        res.add(k, 0.0, ms, h * w)  # the reference records no RMSE here
        bgr = ycbcr_to_bgr(gray.astype(np.float32), est[0], est[1])
        IO.write_bmp(os.path.join(top, f"{algorithm}_{name}.bmp"), bgr)
        test = bgr_to_ycbcr_u8(bgr)
        s3 = ssim(gt, test)
        p3 = [0.0, psnr(gt[..., 1], test[..., 1]), psnr(gt[..., 2], test[..., 2]), 0.0]
        print(f"{name}, SSIM: [{s3[0]:g}, {s3[1]:g}, {s3[2]:g}, 0], PSNR: "
              f"[{p3[0]:g}, {p3[1]:g}, {p3[2]:g}, {p3[3]:g}]", file=out)
    print(res.line(), file=err)
    return res


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m domain_transform_solver_gb300.cli")
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("depth_super_res")
    a.add_argument("--path_to_data_top_dir", default="")
    a.add_argument("--algorithm_name", default="dts")
    a.add_argument("--algorithm_input_name", default="bicubic")
    b = sub.add_parser("stereo")
    b.add_argument("--path_to_data_top_dir", default="")
    c = sub.add_parser("colorization")
    c.add_argument("--path_to_data_top_dir", default="")
    c.add_argument("--algorithm_name", default="dts")
    args = ap.parse_args(argv)
    if not args.path_to_data_top_dir:
        print("Invalid command line inputs.", file=sys.stderr)
        return -1
    if args.cmd == "depth_super_res":
        if not args.algorithm_name or not args.algorithm_input_name:
            print("Invalid command line inputs.", file=sys.stderr)
            return -1
        depth_super_res(args.path_to_data_top_dir, args.algorithm_name,
                        args.algorithm_input_name)
    elif args.cmd == "colorization":
        colorization(args.path_to_data_top_dir, args.algorithm_name)
    else:
        stereo(args.path_to_data_top_dir)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
