"""Benchmark of the DTS / HFBS hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload cfg3|cfg3dts|cfg0|cfg1|cfg2|cfg4|cfg1grad|cfg4soft]

One JSON line on stdout (rank 0).  A step is one pass of the workload's
solves with inputs already resident in HBM: for DTS the reference's timed
window (src/edge_aware_solver.h:72-84: differential, integration, all
iterations), for HFBS the whole HFBS::Optimize.  `e2e` times the same step
through the public C ABI with pinned host buffers, the upload and the
download included (configs 3 and 4: dtsgb_pipeline_run / _run_grad, which
overlap the copies of one chunk of instances with the solves of another;
--e2e-chunks).
Steps are timed with the library's per-kernel profiler off; a second pass of
the same steps with it on gives the kernel table and the roofline (its events
slow steps of small kernels).  Under torchrun the batched workloads (64
ragged instances, 16 differentiable instances) are split over the ranks by
pixel count (sharding.partition_lpt; independent instances, no collective):
strong scaling.  Single-image workloads run one replica per rank.

--impl reference times the reference algorithm's CPU restatement (the FP32
oracle port, all host threads, plus one single-thread sample) on the same
workload; the reference's own CUDA build cannot be built with this
toolchain.  That arm never loads the product library: the input generators
are loaded from their file, not through the package.
"""
from __future__ import annotations

import argparse
import ctypes
import importlib.util
import json
import math
import os
import platform
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

METRIC = "DTS/HFBS solve Mpix/s at fixed iters, fwd+bwd Mpix/s, %HBM peak; RMSE vs FP64"
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 256 << 20
KERNEL_NAMES = {0: "k_bounds", 1: "k_dts_iter", 2: "k_filter", 3: "k_splat",
                4: "k_bistoch", 5: "k_solve (HFBS heavy-ball)", 6: "hfbs setup kernels",
                7: "k_slice", 8: "k_to_float", 9: "k_dts_adjoint",
                10: "hfbs adjoint (whole backward)",
                11: "soft-window plans, line scans and other",
                12: "k_soft_half_plan X", 13: "k_soft_adjoint_fused X",
                14: "k_soft_adjoint_fused Y", 15: "k_soft_half_plan Y"}
HFBS_TB_STEPS = 4  # heavy-ball steps per launch of the temporally blocked kernel


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


_W = None


def workloads_module():
    """domain_transform_solver_gb300/workloads.py loaded from its file: the
    input generators without the package (whose import loads libdtsgb.so)."""
    global _W
    if _W is None:
        path = ROOT / "domain_transform_solver_gb300" / "workloads.py"
        spec = importlib.util.spec_from_file_location("dtsgb_bench_workloads", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        _W = mod
    return _W


def tuning_signature(tuning) -> str:
    """The knobs a traffic record was measured under, as one string."""
    if not tuning:
        return "default"
    keys = ("dts_tile", "bounds_segment", "hfbs_solve_steps", "hfbs_group_voxels")
    return ",".join(f"{k}={tuning[k]}" for k in keys if k in tuning)


def autotune_cache() -> str:
    """The autotune cache file: $DTSGB_AUTOTUNE_CACHE, else the package's
    autotune_cache.txt (choices timed on GB300 for the workloads here; a case
    not in it is timed and appended)."""
    return os.environ.get("DTSGB_AUTOTUNE_CACHE") or str(
        ROOT / "domain_transform_solver_gb300" / "autotune_cache.txt")


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---- clocks ------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_id: str):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50", "-i", device_id],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.12)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _pinned_copy(a: np.ndarray) -> np.ndarray:
    import torch
    t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
    out = t.numpy()
    out[...] = a  # the array's base is the pinned tensor, which it keeps alive
    return out


def _pinned_empty(shape, dtype=np.float32) -> np.ndarray:
    import torch
    t = torch.empty(shape, dtype=getattr(torch, np.dtype(dtype).name), pin_memory=True)
    return t.numpy()


def _ptrs(arrays):
    arr = (ctypes.c_void_p * len(arrays))()
    for i, a in enumerate(arrays):
        arr[i] = a.ctypes.data
    return arr


def _check(status):
    from domain_transform_solver_gb300._lib import check
    check(status)


def _stratified(sizes, k: int) -> list[int]:
    """Every k-th instance in order of pixel count (a sample with the
    batch's size distribution and about 1/k of its pixels)."""
    order = sorted(range(len(sizes)), key=lambda i: (sizes[i][0] * sizes[i][1], i))
    return sorted(order[k // 2::k]) if k > 1 else list(range(len(sizes)))


# ---- workloads ---------------------------------------------------------------
# Byte models per step, by kernel id (one step's launches together):
#   pass_model_bytes: the reference's pass model (each pass reads each input
#     once and writes each output once at the storage format used): DTS
#     setup 4 + 2*s_dH B/px, per iteration X (read v, t, c, dH; write v) and
#     Y (read v, dV; write v); HFBS splat (guide, t, c) + 12 B/vx, per
#     bistochastization step 12 B/vx, invA 16 + blur 48 + init 12 B/vx, per
#     heavy-ball step 28 B/vx, slice 8 B/px.  Kernels it does not describe
#     (the iterate initialisation, the adjoints) use the fused contract.
#   fused_bytes: what the fused kernels here must move at minimum (the DTS
#     iteration reads v, t, c and the packed bounds once and writes v; the
#     temporally blocked heavy-ball launch reads z, n, b, invA, h once and
#     writes h, z for four steps).
class Batched:
    """Shared parts of the many-instance workloads."""

    scaling = "strong"
    reuse_note = "off (every step recomputes all of it)"

    def config(self, world):
        c = {"workload": self.name, "pixels_per_step": self.total_pixels,
             "voxels_per_step": self.total_voxels, "iterations": self.iters,
             "instances": self.n_total,
             "l2": ("inputs larger than L2" if self.total_pixels * 16 > 2 * (129 << 20)
                    else "flushed between steps (256 MB write)"),
             "parallelism": (f"{world} GPUs, instances split by pixel count "
                             "(longest first to the least loaded)" if world > 1
                             else "1 GPU"),
             "guide_state_reuse": self.reuse_note}
        return c

    def reference_subset(self):
        return None  # the whole workload per step


class Cfg3(Batched):
    """64 ragged instances (W~U[256,1920], H~U[256,1080]), each solved by DTS
    (the depth super-resolution parameters: sigma 8/8/0.1, lambda 0.99,
    sigma_z 8, 10 iterations) and HFBS (the colorization parameters: 8x8
    spatial, sigma_l 16, 64 iterations; luma from YCbCr), BF16
    target/confidence storage, FP32 math, one launch per kernel across all
    instances, CUDA-graph replay."""

    name = "cfg3_batched_dts_hfbs_64_ragged_bf16"
    dtype = "bf16 storage, f32 math"
    solvers = ("dts", "hfbs")

    def __init__(self, rank: int = 0, world: int = 1, scale: float = 1.0,
                 e2e_chunks: int = 16):
        W = workloads_module()
        self.W = W
        self.e2e_chunks = e2e_chunks
        # scale < 1 shrinks every instance (profiling captures of a smaller
        # case); the reported workload is scale 1
        if scale != 1.0:
            self.name = f"{self.name}_scale{scale:g}"
        all_sizes = [W.scaled_size(w, h, scale) for w, h in W.batched_sizes()]
        self.n_total = len(all_sizes)
        if world > 1:
            from domain_transform_solver_gb300.sharding import partition_lpt
            share = partition_lpt(all_sizes, world)[rank]
        else:
            share = list(range(len(all_sizes)))
        self.share = share
        self.insts = W.batched_instances(scale=scale, indices=set(share))
        self.sizes = [(i.width, i.height) for i in self.insts]
        self.pixels = sum(w * h for w, h in self.sizes)
        self.total_pixels = sum(w * h for w, h in all_sizes)
        self.iters = W.CFG0_OPT["num_iterations"]
        self.hp = dict(W.CFG1_HFBS)

        def vox(sz):
            return sum(math.ceil(np.float32(w) / np.float32(8.0)) *
                       math.ceil(np.float32(h) / np.float32(8.0)) * 16 for w, h in sz)
        hf = "hfbs" in self.solvers
        self.voxels = vox(self.sizes) if hf else 0
        self.total_voxels = vox(all_sizes) if hf else 0

    def setup(self, stream_handle: int):
        import domain_transform_solver_gb300 as D
        W = self.W
        self.D = D
        self.b = D.Batch(self.sizes, flags=D.FLAG_BF16_STORAGE)
        # every step solves the same inputs: keeping the guide-derived windows
        # and HFBS normalisation across steps would skip work, so it is off
        self.b.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)
        self.b.set_stream(stream_handle)
        self.b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in self.insts],
                      [i.target for i in self.insts], [i.confidence for i in self.insts])
        self.fp = D.DomainFilterParams(**W.CFG0_FILTER)._c()
        self.op = D.DomainOptimizeParams(**W.CFG0_OPT)._c()
        self.hpc = D.HFBSGridParams(**self.hp)._c()
        self.lib = self.b._lib
        # pinned host buffers (kept alive by these lists)
        self._rgba = [_pinned_copy(i.rgba) for i in self.insts]
        self._t = [_pinned_copy(i.target) for i in self.insts]
        self._c = [_pinned_copy(i.confidence) for i in self.insts]
        self._o0 = [_pinned_empty((h, w)) for w, h in self.sizes]
        self._o1 = [_pinned_empty((h, w)) for w, h in self.sizes]
        self.h_rgba, self.h_t, self.h_c = _ptrs(self._rgba), _ptrs(self._t), _ptrs(self._c)
        self.h_o0, self.h_o1 = _ptrs(self._o0), _ptrs(self._o1)
        # the host-to-host path: chunks of instances on their own streams
        self.pipe = D.Pipeline(self.sizes, flags=D.FLAG_BF16_STORAGE,
                               n_chunks=self.e2e_chunks)
        self.pipe.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)
        self.e2e_api = f"dtsgb_pipeline_run, {self.pipe.n_chunks} chunks"

    def autotune(self):
        """The batch's tuning knobs chosen by timing (outside the timed
        region), or read from the autotune cache file; returns the chosen
        values and where they came from."""
        D = self.D
        hit = self.b.autotune(D.DomainFilterParams(**self.W.CFG0_FILTER),
                              D.DomainOptimizeParams(**self.W.CFG0_OPT),
                              D.HFBSGridParams(**self.hp) if "hfbs" in self.solvers else None,
                              reps=2, cache_path=autotune_cache())
        return {**self.b.tuning(), "source": "cache file" if hit else "timed"}

    def step(self):
        if "dts" in self.solvers:
            _check(self.lib.dtsgb_batch_solve_dts(self.b.handle, ctypes.byref(self.fp),
                                                  ctypes.byref(self.op), ctypes.c_float(-1.0)))
        if "hfbs" in self.solvers:
            _check(self.lib.dtsgb_batch_solve_hfbs(self.b.handle, ctypes.byref(self.hpc)))

    def step_e2e(self):
        dts, hfbs = "dts" in self.solvers, "hfbs" in self.solvers
        _check(self.lib.dtsgb_pipeline_run(
            self.pipe.handle, 1, self.h_rgba, self.h_t, self.h_c,
            ctypes.byref(self.fp) if dts else None, ctypes.byref(self.op) if dts else None,
            ctypes.c_float(-1.0), ctypes.byref(self.hpc) if hfbs else None,
            self.h_o0 if dts else None, self.h_o1 if hfbs else None))

    def e2e_bytes(self):
        return self.pixels * (4 + 4 + 4), self.pixels * 4 * len(self.solvers)

    def fused_bytes(self):
        px, vx, it = self.pixels, self.voxels, self.iters
        k = self.hp["optim_iter_max"]
        b = {}
        if "dts" in self.solvers:
            b.update({0: 8 * px,            # read guide, write packed bounds
                      1: 16 * px * it,      # read v f32, t bf16, c bf16, bounds; write v f32
                      8: 6 * px})           # read t bf16, write v f32
        if "hfbs" in self.solvers:
            b.update({3: 8 * px + 12 * vx,  # read guide, t, c; write b, sum c, count
                      4: 12 * vx * self.hp["bistoch_iter_max"],
                      5: 28 * vx * math.ceil(k / HFBS_TB_STEPS),
                      6: 76 * vx,
                      7: 8 * px})           # read guide, write result (grid reads cached)
        return b

    def pass_model_bytes(self):
        px, vx, it = self.pixels, self.voxels, self.iters
        b = {}
        if "dts" in self.solvers:
            b.update({0: (4 + 2 * 2) * px,            # guide in, dH and dV (bf16) out
                      1: (14 + 10) * px * it,         # X: v4 t2 c2 dH2 + v4; Y: v4 dV2 + v4
                      8: 6 * px})
        if "hfbs" in self.solvers:
            b.update({3: 8 * px + 12 * vx, 4: 12 * vx * self.hp["bistoch_iter_max"],
                      5: 28 * vx * self.hp["optim_iter_max"], 6: 76 * vx, 7: 8 * px})
        return b

    def cpu_sizes(self):
        return self.sizes

    def cpu_sample(self, real="f32", subset=None):
        """The FP32 oracle port over the instances of `subset` (default: all),
        DTS and/or HFBS each, as the batch solves them."""
        import oracle as O
        W = self.W
        idx = range(len(self.insts)) if subset is None else subset
        px = 0
        for i in idx:
            inst = self.insts[i]
            if "dts" in self.solvers:
                O.dts_solve(inst.rgba, inst.target, inst.confidence, 1, W.CFG0_FILTER,
                            W.CFG0_OPT, real=real)
            if "hfbs" in self.solvers:
                O.hfbs_solve(inst.rgba, inst.target, inst.confidence, 1, self.hp,
                             max_grid=(inst.width, inst.height, 64), real=real)
            px += inst.width * inst.height
        what = " + ".join(s.upper() for s in self.solvers)
        if subset is None or len(idx) == len(self.insts):
            return px, f"all {len(self.insts)} instances, {what} each"
        step = max(1, round(len(self.insts) / max(1, len(idx))))
        return px, (f"{len(idx)} of the {len(self.insts)} instances (one in "
                    f"{step} by pixel count), {what} each")


class Cfg3Dts(Cfg3):
    """The 64-instance batch's DTS solve alone (BF16 storage, 10
    iterations): the batched form of the 640x480 depth super-resolution, for
    the batched versus single-image comparison."""

    name = "cfg3dts_batched_dts_64_ragged_bf16"
    solvers = ("dts",)


class Single:
    """Shared parts of the single-image workloads (one replica per rank)."""

    scaling = "weak"
    n_total = 1

    def config(self, world):
        return {"workload": self.name, "pixels_per_step": self.pixels,
                "voxels_per_step": self.voxels, "iterations": self.iters,
                "l2": "flushed between steps (256 MB write)",
                "parallelism": (f"{world} independent replicas (a single image does not "
                                "shard)" if world > 1 else "1 GPU"),
                "guide_state_reuse": "off (every step recomputes all of it)"}

    @property
    def total_pixels(self):
        return self.pixels

    def reference_subset(self):
        return None

    def cpu_sizes(self):
        return [(self.inst.width, self.inst.height)]


class _DtsSingle(Single):
    """Single-image DTS through the class API."""

    voxels = 0
    color_space = 1
    bf16 = False

    def setup(self, stream_handle: int):
        import domain_transform_solver_gb300 as D
        w, h = self.inst.width, self.inst.height
        self.s = D.DomainTransformSolver(D.ImageDim(w, h),
                                         flags=D.FLAG_BF16_STORAGE if self.bf16 else 0)
        self.s.SetStream(stream_handle)
        self.s.ClearAll()
        self.s.InitFrame(D.COLOR_SPACE(self.color_space), self.inst.rgba, self.inst.target,
                         self.inst.confidence)
        self.fpar = D.DomainFilterParams(**self.filt)
        self.opar = D.DomainOptimizeParams(**self.opt)
        self.h_rgba = _pinned_copy(self.inst.rgba)
        self.h_t = _pinned_copy(self.inst.target)
        self.h_c = _pinned_copy(self.inst.confidence)
        self.h_out = _pinned_empty((h, w))

    def step(self):
        self.s.ComputeColorSpaceDifferential(self.fpar)
        self.s.IntegrateColorDifferentials()
        self.s.Optimize(self.opar)

    def step_e2e(self):
        lib, h = self.s._lib, self.s.handle
        _check(lib.dtsgb_dts_init_frame(h, self.color_space,
                                        ctypes.c_void_p(self.h_rgba.ctypes.data),
                                        ctypes.c_void_p(self.h_t.ctypes.data),
                                        ctypes.c_void_p(self.h_c.ctypes.data)))
        self.step()
        _check(lib.dtsgb_dts_download(h, 5, ctypes.c_void_p(self.h_out.ctypes.data)))

    def e2e_bytes(self):
        return self.pixels * 12, self.pixels * 4

    def fused_bytes(self):
        px, it, s = self.pixels, self.iters, 2 if self.bf16 else 4
        return {0: 8 * px, 1: (12 + 2 * s) * px * it, 8: (4 + s) * px}

    def pass_model_bytes(self):
        px, it, s = self.pixels, self.iters, 2 if self.bf16 else 4
        return {0: (4 + 2 * s) * px, 1: (16 + 4 * s) * px * it, 8: (4 + s) * px}

    def cpu_sample(self, real="f32", subset=None):
        import oracle as O
        O.dts_solve(self.inst.rgba, self.inst.target, self.inst.confidence,
                    self.color_space, self.filt, self.opt, real=real)
        return self.pixels, "one full solve"


class Cfg0(_DtsSingle):
    """DTS depth super-resolution 640x480, FP32, 10 iterations."""

    name = "cfg0_dts_depth_superres_640x480"
    dtype = "f32"

    def __init__(self, rank: int = 0, world: int = 1):
        W = workloads_module()
        self.inst = W.depth_sr_instance(W.SEED_BASE)
        self.pixels = self.inst.width * self.inst.height
        self.filt, self.opt = W.CFG0_FILTER, W.CFG0_OPT
        self.iters = self.opt["num_iterations"]


class Cfg2(_DtsSingle):
    """DTS with a given confidence, 1280x384 RGB, Charbonnier, sigma_z 30, 15
    iterations, BF16 storage of target and confidence."""

    name = "cfg2_dts_charbonnier_1280x384_bf16"
    dtype = "bf16 storage, f32 math"
    color_space = 0
    bf16 = True

    def __init__(self, rank: int = 0, world: int = 1):
        W = workloads_module()
        self.inst = W.stereo_instance()
        self.pixels = self.inst.width * self.inst.height
        self.filt, self.opt = W.CFG2_FILTER, W.CFG2_OPT
        self.iters = self.opt["num_iterations"]


class Cfg1(Single):
    """HFBS colorization 640x480, U and V channels, 64 iterations."""

    name = "cfg1_hfbs_colorization_640x480_uv"
    dtype = "f32"

    def __init__(self, rank: int = 0, world: int = 1):
        W = workloads_module()
        self.W = W
        self.u, self.v = W.colorization_instance()
        self.inst = self.u
        self.pixels = 2 * self.u.width * self.u.height
        self.iters = W.CFG1_HFBS["optim_iter_max"]
        self.voxels = 2 * 80 * 60 * 16

    def setup(self, stream_handle: int):
        import domain_transform_solver_gb300 as D
        W = self.W
        w, h = self.u.width, self.u.height
        self.b = D.Batch([(w, h), (w, h)])
        self.b.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)  # full work every step
        self.b.set_stream(stream_handle)
        self.b.upload(D.COLOR_SPACE.RGB, [self.u.rgba, self.u.rgba],
                      [self.u.target, self.v], [self.u.confidence, self.u.confidence])
        self.hpc = D.HFBSGridParams(**W.CFG1_HFBS)._c()
        self.lib = self.b._lib
        self._pin = [_pinned_copy(self.u.rgba), _pinned_copy(self.u.target),
                     _pinned_copy(self.v), _pinned_copy(self.u.confidence),
                     _pinned_empty((h, w)), _pinned_empty((h, w))]
        rg, tu, tv, cf, o0, o1 = self._pin
        self.h_rgba = _ptrs([rg, rg])
        self.h_t = _ptrs([tu, tv])
        self.h_c = _ptrs([cf, cf])
        self.h_o = _ptrs([o0, o1])

    def step(self):
        _check(self.lib.dtsgb_batch_solve_hfbs(self.b.handle, ctypes.byref(self.hpc)))

    def step_e2e(self):
        h = self.b.handle
        _check(self.lib.dtsgb_batch_upload(h, 0, self.h_rgba, self.h_t, self.h_c))
        self.step()
        _check(self.lib.dtsgb_batch_download(h, 1, self.h_o))

    def e2e_bytes(self):
        return self.pixels * 12, self.pixels * 4

    def fused_bytes(self):
        px, vx, hp = self.pixels, self.voxels, self.W.CFG1_HFBS
        return {3: 12 * px + 12 * vx, 4: 12 * vx * hp["bistoch_iter_max"],
                5: 28 * vx * math.ceil(hp["optim_iter_max"] / HFBS_TB_STEPS), 6: 76 * vx,
                7: 8 * px}

    def pass_model_bytes(self):
        px, vx, hp = self.pixels, self.voxels, self.W.CFG1_HFBS
        return {3: 12 * px + 12 * vx, 4: 12 * vx * hp["bistoch_iter_max"],
                5: 28 * vx * hp["optim_iter_max"], 6: 76 * vx, 7: 8 * px}

    def cpu_sample(self, real="f32", subset=None):
        import oracle as O
        W = self.W
        for t in (self.u.target, self.v):
            O.hfbs_solve(self.u.rgba, t, self.u.confidence, 0, W.CFG1_HFBS,
                         max_grid=(96, 96, 32), real=real)
        return self.pixels, "U and V solves"


class Cfg1Grad(Cfg1):
    """Differentiable HFBS: the 640x480 colorization (U and V, 64
    iterations), FP32, the batched forward keeping every heavy-ball iterate
    (the automatic checkpoint choice) plus the adjoint (dL/dtarget,
    dL/dconfidence) for an N(0,1) upstream gradient, both replayed from CUDA
    graphs.  One step = forward + backward of both channels; bins, counts
    and normalisation are held fixed (piecewise constant in the guide)."""

    name = "cfg1grad_hfbs_fwd_bwd_640x480_uv_f32"

    def setup(self, stream_handle: int):
        import torch
        import domain_transform_solver_gb300 as D
        super().setup(stream_handle)  # the plain batched forward, for the ratio
        w, h = self.u.width, self.u.height
        rng = np.random.default_rng(7)
        self.grads = [rng.standard_normal((h, w)).astype(np.float32) for _ in range(2)]
        self.gb = D.Batch([(w, h), (w, h)])
        self.gb.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)  # full work every step
        self.gb.set_stream(stream_handle)
        self.gb.enable_grad(True, 0)
        self.gb.upload(D.COLOR_SPACE.RGB, [self.u.rgba, self.u.rgba], [self.u.target, self.v],
                       [self.u.confidence, self.u.confidence])
        dev = torch.device("cuda")
        self.d_g = torch.from_numpy(np.stack(self.grads)).to(dev)
        self.d_gt = torch.empty_like(self.d_g)
        self.d_gc = torch.empty_like(self.d_g)
        self.p_g = (ctypes.c_void_p * 2)(*[self.d_g[i].data_ptr() for i in range(2)])
        self.p_gt = (ctypes.c_void_p * 2)(*[self.d_gt[i].data_ptr() for i in range(2)])
        self.p_gc = (ctypes.c_void_p * 2)(*[self.d_gc[i].data_ptr() for i in range(2)])
        self._g = [_pinned_copy(g) for g in self.grads]
        self._gt = [_pinned_empty((h, w)) for _ in range(2)]
        self._gc = [_pinned_empty((h, w)) for _ in range(2)]
        self.h_g, self.h_gt, self.h_gc = _ptrs(self._g), _ptrs(self._gt), _ptrs(self._gc)
        self.e2e_api = ("dtsgb_batch_upload, dtsgb_batch_solve_hfbs, dtsgb_batch_download, "
                        "dtsgb_batch_hfbs_backward")

    def step(self):
        h = self.gb.handle
        _check(self.lib.dtsgb_batch_solve_hfbs(h, ctypes.byref(self.hpc)))
        _check(self.lib.dtsgb_batch_hfbs_backward_device(h, self.p_g, self.p_gt, self.p_gc))

    def forward_only(self):
        Cfg1.step(self)

    def step_e2e(self):
        h = self.gb.handle
        _check(self.lib.dtsgb_batch_upload(h, 0, self.h_rgba, self.h_t, self.h_c))
        _check(self.lib.dtsgb_batch_solve_hfbs(h, ctypes.byref(self.hpc)))
        _check(self.lib.dtsgb_batch_download(h, 1, self.h_o))
        _check(self.lib.dtsgb_batch_hfbs_backward(h, self.h_g, self.h_gt, self.h_gc))

    def e2e_bytes(self):
        # rgba, target, confidence, upstream gradient in; result, dL/dt, dL/dc out
        return self.pixels * 16, self.pixels * 12

    def fused_bytes(self):
        px, vx, k = self.pixels, self.voxels, self.iters
        b = super().fused_bytes()
        # four heavy-ball steps per launch: read z, h, norm, b, invA; write z,
        # h and the three kept iterates
        b[5] = 40 * vx * math.ceil(k / HFBS_TB_STEPS)
        # the whole adjoint: read dL/dout, guide, target, confidence and
        # write dL/dt, dL/dc per pixel; per step 10 grid reads, 6 writes
        b[10] = 24 * px + 64 * vx * k
        return b

    def pass_model_bytes(self):
        b = super().pass_model_bytes()
        b[10] = self.fused_bytes()[10]  # the model has no adjoint: the fused contract
        return b

    def cpu_sample(self, real="f32", subset=None):
        import oracle as O
        W = self.W
        o = O.OracleHFBS(self.u.width, self.u.height, 96, 96, 32, real=real)
        o.clear_all()
        o.init_frame(0, self.u.rgba, self.u.target, self.u.confidence)
        o.set_params(**W.CFG1_HFBS)
        o.optimize()
        rng = np.random.default_rng(7)
        o.backward(rng.standard_normal((self.u.height, self.u.width)).astype(np.float32))
        return self.pixels // 2, "the U channel, forward + adjoint"


class Cfg4(Batched):
    """Differentiable DTS: 16 x 1024x768 depth super-resolution instances, FP32,
    L2, 10 iterations, the forward keeping its iterates (the automatic
    checkpoint choice: every iterate, as 14 planes fit in free memory) plus
    the adjoint (dL/dtarget, dL/dconfidence) for an N(0,1) upstream
    gradient.  One step = forward + backward; the guide's window bounds
    are held fixed (piecewise constant in the guide)."""

    name = "cfg4_dts_fwd_bwd_16x1024x768_f32"
    dtype = "f32"

    def __init__(self, rank: int = 0, world: int = 1, e2e_chunks: int = 4):
        W = workloads_module()
        self.W = W
        self.e2e_chunks = e2e_chunks
        n, w, h = 16, 1024, 768
        self.n_total = n
        if world > 1:
            from domain_transform_solver_gb300.sharding import partition_lpt
            share = partition_lpt([(w, h)] * n, world)[rank]
        else:
            share = list(range(n))
        self.insts, self.grads = W.grad_instances(indices=share)
        self.sizes = [(i.width, i.height) for i in self.insts]
        self.pixels = sum(w * h for w, h in self.sizes)
        self.total_pixels = n * w * h
        self.iters = W.CFG0_OPT["num_iterations"]
        self.voxels = self.total_voxels = 0

    def setup(self, stream_handle: int):
        import torch
        import domain_transform_solver_gb300 as D
        W = self.W
        self.D = D
        self.b = D.Batch(self.sizes)
        self.b.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)  # full work every step
        self.b.set_stream(stream_handle)
        self.b.enable_grad(True, 0)
        self.b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in self.insts],
                      [i.target for i in self.insts], [i.confidence for i in self.insts])
        self.fp = D.DomainFilterParams(**W.CFG0_FILTER)._c()
        self.op = D.DomainOptimizeParams(**W.CFG0_OPT)._c()
        self.lib = self.b._lib
        dev = torch.device("cuda")
        # upstream gradients resident in HBM; gradient outputs in HBM
        self.d_g = torch.from_numpy(np.stack(self.grads)).to(dev)
        self.d_gt = torch.empty_like(self.d_g)
        self.d_gc = torch.empty_like(self.d_g)
        n = len(self.sizes)
        self.p_g = (ctypes.c_void_p * n)(*[self.d_g[i].data_ptr() for i in range(n)])
        self.p_gt = (ctypes.c_void_p * n)(*[self.d_gt[i].data_ptr() for i in range(n)])
        self.p_gc = (ctypes.c_void_p * n)(*[self.d_gc[i].data_ptr() for i in range(n)])
        self._rgba = [_pinned_copy(i.rgba) for i in self.insts]
        self._t = [_pinned_copy(i.target) for i in self.insts]
        self._c = [_pinned_copy(i.confidence) for i in self.insts]
        self._g = [_pinned_copy(g) for g in self.grads]
        self._v = [_pinned_empty((h, w)) for w, h in self.sizes]
        self._ogt = [_pinned_empty((h, w)) for w, h in self.sizes]
        self._ogc = [_pinned_empty((h, w)) for w, h in self.sizes]
        self.h_rgba, self.h_t, self.h_c = _ptrs(self._rgba), _ptrs(self._t), _ptrs(self._c)
        self.h_g, self.h_v = _ptrs(self._g), _ptrs(self._v)
        self.h_gt, self.h_gc = _ptrs(self._ogt), _ptrs(self._ogc)
        # the host-to-host path: chunks of instances on their own streams
        self.pipe = D.Pipeline(self.sizes, n_chunks=self.e2e_chunks)
        self.pipe.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)
        self.e2e_api = f"dtsgb_pipeline_run_grad, {self.pipe.n_chunks} chunks"
        # the plain forward (no checkpoints) of the same batch, for the ratio
        self.fwd = D.Batch(self.sizes)
        self.fwd.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)
        self.fwd.set_stream(stream_handle)
        self.fwd.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in self.insts],
                        [i.target for i in self.insts], [i.confidence for i in self.insts])

    def autotune(self):
        D = self.D
        hit = self.b.autotune(D.DomainFilterParams(**self.W.CFG0_FILTER),
                              D.DomainOptimizeParams(**self.W.CFG0_OPT), None, reps=2,
                              cache_path=autotune_cache())
        for knob in (D.TUNE_DTS_TILE, D.TUNE_BOUNDS_SEGMENT):
            self.fwd.set_tuning(knob, self.b.get_tuning(knob))
        return {**self.b.tuning(), "source": "cache file" if hit else "timed"}

    def step(self):
        _check(self.lib.dtsgb_batch_solve_dts(self.b.handle, ctypes.byref(self.fp),
                                              ctypes.byref(self.op), ctypes.c_float(-1.0)))
        _check(self.lib.dtsgb_batch_dts_backward_device(self.b.handle, self.p_g, self.p_gt,
                                                        self.p_gc))

    def forward_only(self):
        _check(self.lib.dtsgb_batch_solve_dts(self.fwd.handle, ctypes.byref(self.fp),
                                              ctypes.byref(self.op), ctypes.c_float(-1.0)))

    def step_e2e(self):
        _check(self.lib.dtsgb_pipeline_run_grad(self.pipe.handle, 1, self.h_rgba, self.h_t,
                                                self.h_c, ctypes.byref(self.fp),
                                                ctypes.byref(self.op), self.h_g, self.h_v,
                                                self.h_gt, self.h_gc))

    def e2e_bytes(self):
        # rgba, target, confidence, upstream gradient in; v, dL/dt, dL/dc out
        return self.pixels * 16, self.pixels * 12

    def fused_bytes(self):
        px, it = self.pixels, self.iters
        return {
            0: 8 * px,        # read guide, write packed bounds
            1: 20 * px * it,  # read v, t, c, bounds; write v (f32)
            8: 8 * px,        # read t, write v
            9: 40 * px * it,  # read g, v_k, t, c, bounds; read+write dL/dt, dL/dc; write g
        }

    def pass_model_bytes(self):
        px, it = self.pixels, self.iters
        b = self.fused_bytes()  # the adjoint and the init: the fused contract
        b.update({0: 12 * px, 1: 32 * px * it})
        return b

    def reference_subset(self):
        return [0, 5, 10, 15]  # 4 of the 16 (identical sizes) keep a step near 3 s

    def cpu_sizes(self):
        return self.sizes

    def cpu_sample(self, real="f32", subset=None):
        """The FP32 port: forward + adjoint of the instances of `subset`."""
        import oracle as O
        W = self.W
        op = W.CFG0_OPT
        idx = range(len(self.insts)) if subset is None else subset
        px = 0
        for i in idx:
            inst, g = self.insts[i], self.grads[i]
            o = O.OracleDTS(inst.width, inst.height, real=real)
            o.init_frame(1, inst.rgba, inst.target, inst.confidence)
            o.differential(W.CFG0_FILTER["sigma_x"], W.CFG0_FILTER["sigma_y"],
                           W.CFG0_FILTER["sigma_r"])
            o.integrate()
            o.backward(op["num_iterations"], op["loss"], op["lambda_"], op["sigma_z"],
                       op["step_size"], g)
            px += inst.width * inst.height
        return px, f"{len(idx)} of the {len(self.insts)} instances, forward + adjoint"


class Cfg4Soft(Batched):
    """Config 4 with gradients with respect to the guide-derived edge
    weights: 16 x 1024x768, FP32, L2, 10 iterations of the soft-window solve
    (window ends ramped over tau = 1 transformed-domain unit around sigma_z)
    from the guides' edge weights dH, dV, plus its adjoint dL/dtarget,
    dL/dconfidence, dL/ddH, dL/ddV for an N(0,1) upstream gradient.  One
    step = forward + backward (every iterate kept)."""

    name = "cfg4soft_dts_soft_window_fwd_bwd_16x1024x768_f32"
    dtype = "f32"
    tau = 1.0

    def __init__(self, rank: int = 0, world: int = 1, instances: int = None):
        W = workloads_module()
        self.W = W
        n, w, h = 16, 1024, 768
        # instances < 16 keeps the first ones (profiling captures of a
        # smaller case); the reported workload is all 16
        if instances is not None and instances < n:
            n = max(1, instances)
            self.name = f"{self.name}_first{n}"
        self.n_total = n
        if world > 1:
            from domain_transform_solver_gb300.sharding import partition_lpt
            share = partition_lpt([(w, h)] * n, world)[rank]
        else:
            share = list(range(n))
        self.insts, self.grads = W.grad_instances(indices=share)
        self.sizes = [(i.width, i.height) for i in self.insts]
        self.pixels = sum(a * b for a, b in self.sizes)
        self.total_pixels = n * w * h
        self.iters = W.CFG0_OPT["num_iterations"]
        self.voxels = self.total_voxels = 0

    def setup(self, stream_handle: int):
        import torch
        import domain_transform_solver_gb300 as D
        W = self.W
        dev = torch.device("cuda")
        n = len(self.sizes)
        h, w = self.insts[0].target.shape
        self.s = D.SoftDTS(self.sizes)
        self.s.set_stream(stream_handle)
        self.op = D.DomainOptimizeParams(**W.CFG0_OPT)
        self.rgba = torch.from_numpy(np.stack([i.rgba for i in self.insts])).to(dev)
        self.t = torch.from_numpy(np.stack([i.target for i in self.insts])).to(dev)
        self.c = torch.from_numpy(np.stack([i.confidence for i in self.insts])).to(dev)
        self.g = torch.from_numpy(np.stack(self.grads)).to(dev)
        self.dh = torch.empty_like(self.t)
        self.dv = torch.empty_like(self.t)
        self.out = torch.empty_like(self.t)
        self.grad_planes = [torch.empty_like(self.t) for _ in range(4)]
        p = lambda x: [x[i].data_ptr() for i in range(n)]  # noqa: E731
        self.p = p
        self.s.edge_weights(D.COLOR_SPACE.YCbCr, p(self.rgba), D.DomainFilterParams(**W.CFG0_FILTER),
                            p(self.dh), p(self.dv))
        # pinned host copies for the end-to-end form
        self.h_in = [_pinned_copy(a.cpu().numpy()) for a in (self.dh, self.dv, self.t, self.c,
                                                             self.g)]
        self.h_out = [_pinned_empty((n, h, w)) for _ in range(5)]
        self.e2e_api = "dtsgb_soft_solve, dtsgb_soft_backward (device buffers filled from pinned host memory)"
        torch.cuda.synchronize()

    def _solve(self):
        p = self.p
        self.s.solve(p(self.dh), p(self.dv), p(self.t), p(self.c), self.op, self.tau, p(self.out))

    def step(self):
        p = self.p
        self._solve()
        self.s.backward(p(self.g), *[p(x) for x in self.grad_planes])

    def forward_only(self):
        self._solve()

    def step_e2e(self):
        import torch
        for dst, src in zip((self.dh, self.dv, self.t, self.c, self.g), self.h_in):
            dst.copy_(torch.from_numpy(src), non_blocking=True)
        self.step()
        for dst, src in zip(self.h_out, [self.out] + self.grad_planes):
            torch.from_numpy(dst).copy_(src, non_blocking=True)

    def e2e_bytes(self):
        return self.pixels * 20, self.pixels * 20

    def fused_bytes(self):
        """Per step: the planned half-steps (X reads v, the plan's counts and
        ramp weights, t, c and writes v, B: 32 B/px; Y 24 B/px) and adjoints
        (X reads a, n, B, x, t, c and the plan, reads and writes dL/dt, dL/dc
        and the band pair sums, writes a': 64 B/px; Y 40 B/px), once per
        iteration each."""
        px, it = self.pixels, self.iters
        return {12: px * 32 * it, 15: px * 24 * it, 13: px * 64 * it, 14: px * 40 * it}

    def pass_model_bytes(self):
        # the reference has no soft-window form: its pass model is the
        # fused contract
        return self.fused_bytes()

    def reference_subset(self):
        return [0]  # the oracle's soft adjoint is serial: one instance per step

    def cpu_sizes(self):
        return self.sizes

    def cpu_sample(self, real="f32", subset=None):
        """The soft-window forward + adjoint restated by the oracle (FP32
        build), from the oracle's own edge weights."""
        import oracle as O
        W = self.W
        idx = range(len(self.insts)) if subset is None else subset
        px = 0
        for i in idx:
            inst, g = self.insts[i], self.grads[i]
            eh, ev = O.edge_weights(inst.rgba, 1, real=real, **W.CFG0_FILTER)
            O.soft_backward(eh, ev, inst.target, inst.confidence, W.CFG0_OPT, self.tau, g,
                            real=real)
            px += inst.width * inst.height
        return px, f"{len(idx)} of the {len(self.insts)} instances, forward + adjoint"


WORKLOADS = {"cfg3": Cfg3, "cfg3dts": Cfg3Dts, "cfg0": Cfg0, "cfg1": Cfg1, "cfg2": Cfg2,
             "cfg4": Cfg4, "cfg1grad": Cfg1Grad, "cfg4soft": Cfg4Soft}


# ---- arms ----------------------------------------------------------------------
def make_workload(args, rank, world):
    if args.workload in ("cfg3", "cfg3dts"):
        return WORKLOADS[args.workload](rank, world, scale=args.scale,
                                        e2e_chunks=args.e2e_chunks or 16)
    if args.workload == "cfg4":
        return Cfg4(rank, world, e2e_chunks=args.e2e_chunks or 4)
    if args.workload == "cfg4soft":
        return Cfg4Soft(rank, world, instances=args.instances)
    return WORKLOADS[args.workload](rank, world)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_over_ranks(world, value, op="max"):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def _time_cpu(wl, subset, budget_s, min_runs=1):
    px, n, t0, desc = 0, 0, time.perf_counter(), ""
    while True:
        p, desc = wl.cpu_sample("f32", subset)
        px += p
        n += 1
        el = time.perf_counter() - t0
        if n >= min_runs and el >= budget_s:
            break
    return px / el / 1e6, n, el, desc


def single_thread_sample(wl, s_per_pass_all, threads, budget_s=15.0):
    """One thread over a sample with the workload's size distribution (every
    k-th instance by pixel count), k chosen so that the estimated time fits
    budget_s; s_per_pass_all: seconds of one all-thread pass."""
    import oracle as O
    subset = wl.reference_subset()
    base = list(range(len(wl.cpu_sizes()))) if subset is None else list(subset)
    est = s_per_pass_all * threads
    k = max(1, min(len(base), math.ceil(est / budget_s)))
    sizes = [wl.cpu_sizes()[i] for i in base]
    single = [base[j] for j in _stratified(sizes, k)]
    O.set_threads(1)
    try:
        v, n, el, desc = _time_cpu(wl, single, 0.0)
    finally:
        O.set_threads(0)
    return {"value": v, "unit": "Mpix/s", "cores": 1, "sample": f"{n} x ({desc}), {el:.1f} s"}


def cpu_baseline(wl, budget_s=10.0):
    """The FP32 oracle port on the host: all threads over the workload (its
    reference subset for cfg 4), then one thread over a sample."""
    import oracle as O
    O.build()
    threads = O.set_threads(0)
    subset = wl.reference_subset()
    wl.cpu_sample("f32", subset)  # warm-up (page-in, thread pool)
    v_all, n_all, el_all, desc = _time_cpu(wl, subset, budget_s)
    return {"value": v_all, "unit": "Mpix/s", "cores": threads, "kind": "port",
            "sample": f"{n_all} x ({desc}) of {wl.name} by the FP32 oracle port "
                      f"(OpenMP, {threads} threads), {el_all:.1f} s",
            "single_thread": single_thread_sample(wl, el_all / n_all, threads),
            "cpu_model": cpu_model(), "nproc": host_threads()}


def run_reference(args, world, rank):
    """The reference algorithm's CPU restatement (the FP32 oracle port) on
    this host's cores: every timed step solves the workload (cfg 3: all 64
    instances, DTS + HFBS each) with all threads.  Rank 0 only."""
    if rank != 0:
        return
    wl = make_workload(args, 0, 1)
    import oracle as O
    O.build()
    threads = O.set_threads(0)
    subset = wl.reference_subset()
    for _ in range(args.warmup):
        wl.cpu_sample("f32", subset)
    t0 = time.perf_counter()
    px, desc = 0, ""
    for _ in range(args.steps):
        p, desc = wl.cpu_sample("f32", subset)
        px += p
    el = time.perf_counter() - t0
    value = px / el / 1e6
    single = single_thread_sample(wl, el / args.steps, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpix/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
        "scaling": wl.scaling, "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, shapes of the reference's datasets)",
        "config": wl.config(world),
        "cpu_baseline": {"value": value, "unit": "Mpix/s", "cores": threads, "kind": "port",
                         "sample": f"every step: {desc}",
                         "single_thread": single, "cpu_model": cpu_model(),
                         "nproc": host_threads()},
        "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference's CUDA build cannot be built with this toolchain (empty "
                "libcua/CUB submodules, CUDA 8/9-era CUB API); its algorithm's CPU "
                "restatement (FP32) is timed on the host's threads",
    }
    print(json.dumps(line), flush=True)


def _timed_steps(fn, stream, steps, flush):
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for k in range(steps):
        if flush is not None:
            flush.zero_()  # L2 flush between steps, outside the step's events
        ev[k][0].record(stream)
        fn()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev)


def run_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    import domain_transform_solver_gb300 as D  # noqa: F401  (loads libdtsgb.so)
    from domain_transform_solver_gb300 import _lib
    lib = _lib.load()
    wl = make_workload(args, rank, world)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    wl.setup(stream.cuda_stream)
    tuning = wl.autotune() if hasattr(wl, "autotune") and not args.no_autotune else None
    big = wl.total_pixels * 16 > 2 * (129 << 20)
    flush = None if big else torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32,
                                         device="cuda")
    try:
        uid = str(torch.cuda.get_device_properties(local).uuid)
        dev_id = uid if uid.startswith("GPU-") else "GPU-" + uid
    except Exception:
        dev_id = str(local)
    for _ in range(max(args.warmup, 3)):
        wl.step()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev_id)
    barrier(world)
    torch.cuda.synchronize()
    step_total = _timed_steps(wl.step, stream, args.steps, flush)
    barrier(world)
    clocks = sampler.stop()
    total_ms = reduce_over_ranks(world, step_total, "max")
    ms_per_step = total_ms / args.steps
    all_pixels = reduce_over_ranks(world, wl.pixels, "sum")
    value = all_pixels / (ms_per_step * 1e-3) / 1e6

    # per-kernel launch durations: the same steps again with the library's
    # profiler on (CUDA events recorded on the launching stream around every
    # launch; graph replays keep the events of the latest replay, i.e. the
    # last step).  The events themselves slow a step of small kernels, so
    # the profiled pass is timed apart from the steps above and its shares
    # are of its own step time.
    lib.dtsgb_profile_enable(1)
    wl.step()  # captures the profiled graphs
    torch.cuda.synchronize()
    lib.dtsgb_profile_reset()
    prof_ms_per_step = _timed_steps(wl.step, stream, args.steps, flush) / args.steps
    per_kernel = {}
    for kid in range(len(KERNEL_NAMES)):
        n, t = ctypes.c_int(), ctypes.c_double()
        lib.dtsgb_profile_read(kid, ctypes.byref(n), ctypes.byref(t))
        if n.value:
            per_kernel[kid] = (n.value, t.value)
    lib.dtsgb_profile_enable(0)
    lib.dtsgb_profile_reset()
    graph_replayed = hasattr(wl, "b")
    steps_seen = 1 if graph_replayed else args.steps
    launches_per_step = sum(n for n, _ in per_kernel.values()) / steps_seen
    model, fused = wl.pass_model_bytes(), wl.fused_bytes()
    peak, peak_kind = peaks()
    traffic_rec = {}
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        traffic_rec = json.loads(tf.read_text()).get(wl.name, {})
    sig = tuning_signature(tuning)

    def traffic_of(kid, per_step):
        """DRAM bytes per launch of kernel kid from the ncu record: the entry
        measured under this run's tuning; else another tuning's bytes per
        step spread over this run's launches (an approximation, noted)."""
        entries = traffic_rec.get(KERNEL_NAMES[kid])
        if not entries:
            return None, None
        for e in entries:
            if e["tuning"] == sig:
                return e["bytes_per_launch"], f"measured under this tuning ({sig})"
        e = entries[0]
        return (e["bytes_per_launch"] * e["launches_per_step"] / per_step,
                f"approximate: the bytes per step measured under tuning {e['tuning']}")
    kernels = {}
    for kid, (n, t) in per_kernel.items():
        avg = t / n
        per_step = n / steps_seen
        rec = {"launches_per_step": per_step, "avg_launch_ms": avg,
               "share_of_step": (t / steps_seen) / prof_ms_per_step}
        for key, table in (("pass_model", model), ("fused_contract", fused)):
            if kid in table:
                gbs = table[kid] / per_step / (avg * 1e-3) / 1e9
                rec[f"{key}_gbs"] = gbs
                rec[f"{key}_frac"] = gbs / peak
        tr, _ = traffic_of(kid, per_step)
        if tr:
            rec["dram_bytes_per_launch"] = tr
            rec["dram_frac"] = tr / (avg * 1e-3) / 1e9 / peak
        kernels[KERNEL_NAMES[kid]] = rec
    dom = max(per_kernel, key=lambda k: per_kernel[k][1])
    n_dom, t_dom = per_kernel[dom]
    avg_dom = t_dom / n_dom
    per_step_dom = n_dom / steps_seen

    def form(table):
        if dom not in table:
            return None
        b = table[dom] / per_step_dom
        a = b / (avg_dom * 1e-3) / 1e9
        return {"bytes_per_launch": b, "achieved": a, "frac": a / peak}

    pm, fc = form(model), form(fused)
    traffic, traffic_note = traffic_of(dom, per_step_dom)
    roofline = {"bound": "hbm", "kernel": KERNEL_NAMES[dom],
                "achieved": pm["achieved"] if pm else None, "peak": peak, "unit": "GB/s",
                "frac": pm["frac"] if pm else None,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "traffic": traffic, "avg_launch_ms": avg_dom,
                "algorithmic_bytes_per_launch": pm["bytes_per_launch"] if pm else None,
                "byte_model": "pass model of the reference (each pass reads its inputs and "
                              "writes its outputs once, at the storage format used)",
                "fused_contract": fc,
                "dram_measured": ({"bytes_per_launch": traffic,
                                   "achieved": traffic / (avg_dom * 1e-3) / 1e9,
                                   "frac": traffic / (avg_dom * 1e-3) / 1e9 / peak,
                                   "source": "ncu dram__bytes_read.sum + "
                                             "dram__bytes_write.sum (profiles/traffic.json), "
                                             + traffic_note}
                                  if traffic else None)}

    # e2e through the C ABI with pinned host buffers
    for _ in range(2):
        wl.step_e2e()
    torch.cuda.synchronize()
    barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e_steps = max(1, min(args.steps, 10))
    e0.record(stream)
    for _ in range(e_steps):
        wl.step_e2e()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = reduce_over_ranks(world, e0.elapsed_time(e1), "max") / e_steps
    h2d, d2h = wl.e2e_bytes()
    e2e_value = all_pixels / (e2e_ms * 1e-3) / 1e6

    fwd_ratio = None
    if hasattr(wl, "forward_only"):
        for _ in range(3):
            wl.forward_only()
        torch.cuda.synchronize()
        fwd_ms = reduce_over_ranks(world, _timed_steps(wl.forward_only, stream, args.steps,
                                                       flush), "max") / args.steps
        fwd_ratio = {"forward_ms": fwd_ms, "fwd_bwd_ms": ms_per_step,
                     "fwd_bwd_over_forward": ms_per_step / fwd_ms}

    config = wl.config(world)
    if tuning:
        config["tuning"] = tuning
    line = {
        "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": wl.scaling, "vs_baseline": None,
        "dtype": wl.dtype, "data": "synthetic (seeded, shapes of the reference's datasets)",
        "config": config,
        "e2e": {"value": e2e_value, "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                **({"api": wl.e2e_api} if hasattr(wl, "e2e_api") else {})},
        "roofline": roofline,
        "kernels": kernels,
        "profiled_ms_per_step": prof_ms_per_step,
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "clocks": clocks,
    }
    if fwd_ratio:
        line["fwd_bwd"] = fwd_ratio
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="cfg3")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="cfg3 only: shrink every instance (smaller profiling case)")
    ap.add_argument("--instances", type=int, default=None,
                    help="cfg4soft only: the first N of the 16 instances (smaller profiling case)")
    ap.add_argument("--e2e-chunks", type=int, default=None,
                    help="chunks of the overlapped host-to-host e2e run (cfg3: 16, cfg4: 4)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default tuning instead of timing the knobs first")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU baseline leg (profiling runs)")
    args = ap.parse_args()
    if args.impl == "reference":
        # rank 0 alone times the host CPU; no process group is needed
        world = int(os.environ.get("WORLD_SIZE", "1"))
        run_reference(args, world, int(os.environ.get("RANK", "0")))
        return
    world, rank, local = dist_setup()
    run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
