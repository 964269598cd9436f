"""Benchmark of the DTS / HFBS hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload cfg3|cfg3dts|cfg0|cfg1|cfg2|cfg4|cfg1grad]

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
slow steps of small kernels).  Under torchrun every rank solves its own copy
of the workload (independent instances, no collective): weak scaling.

--impl reference times the reference algorithm's CPU restatement (the FP32
oracle port, all host threads) on a bounded sample of the same workload; the
reference's own CUDA build cannot be built with this toolchain.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
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
                10: "hfbs adjoint (whole backward)"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


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


# ---- workloads ---------------------------------------------------------------
class Cfg3:
    """64 ragged instances (W~U[256,1920], H~U[256,1080]), each solved by DTS
    (the depth super-resolution parameters: sigma 8/8/0.1, lambda 0.99,
    sigma_z 8, 10 iterations) and HFBS (the colorization parameters: 8x8
    spatial, sigma_l 16, 64 iterations; luma from YCbCr), BF16
    target/confidence storage, FP32 math, one launch per kernel across all
    instances, CUDA-graph replay."""

    name = "cfg3_batched_dts_hfbs_64_ragged_bf16"
    dtype = "bf16 storage, f32 math"

    def __init__(self, rank: int, scale: float = 1.0, e2e_chunks: int = 16):
        import domain_transform_solver_gb300 as D
        self.e2e_chunks = e2e_chunks
        from domain_transform_solver_gb300 import workloads as W
        self.D, self.W = D, W
        # scale < 1 shrinks every instance (profiling captures of a smaller
        # case); the reported workload is scale 1
        self.insts = W.batched_instances(scale=scale)
        if scale != 1.0:
            self.name = f"{self.name}_scale{scale:g}"
        self.sizes = [(i.width, i.height) for i in self.insts]
        self.pixels = sum(w * h for w, h in self.sizes)
        self.iters = W.CFG0_OPT["num_iterations"]
        self.hp = dict(W.CFG1_HFBS)
        self.voxels = sum(math.ceil(np.float32(w) / np.float32(8.0)) *
                          math.ceil(np.float32(h) / np.float32(8.0)) * 16
                          for w, h in self.sizes)

    def setup(self, stream_handle: int):
        D, W = self.D, self.W
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

    def step(self):
        from domain_transform_solver_gb300._lib import check
        check(self.lib.dtsgb_batch_solve_dts(self.b.handle, ctypes.byref(self.fp),
                                             ctypes.byref(self.op), ctypes.c_float(-1.0)))
        check(self.lib.dtsgb_batch_solve_hfbs(self.b.handle, ctypes.byref(self.hpc)))

    def step_e2e(self):
        from domain_transform_solver_gb300._lib import check
        check(self.lib.dtsgb_pipeline_run(self.pipe.handle, 1, self.h_rgba, self.h_t,
                                          self.h_c, ctypes.byref(self.fp),
                                          ctypes.byref(self.op), ctypes.c_float(-1.0),
                                          ctypes.byref(self.hpc), self.h_o0, self.h_o1))

    def e2e_bytes(self):
        return self.pixels * (4 + 4 + 4), self.pixels * 4 * 2

    def algorithmic_bytes(self):
        """Bytes each launch of a kernel must move at minimum, per kernel id."""
        px, vx = self.pixels, self.voxels
        return {
            0: 8 * px,            # read guide, write packed bounds
            1: 16 * px,           # read v f32, t bf16, c bf16, bounds; write v f32
            3: 8 * px + 12 * vx,  # read guide, t, c; write b, sum c, count
            4: 12 * vx,           # read n, count; write n
            5: 28 * vx,           # read z, n, b, invA, h; write h, z
            7: 8 * px,            # read guide, write result (grid reads cached)
            8: 6 * px,            # read t bf16, write v f32
        }

    def cpu_sample(self, real="f32"):
        """A bounded sample: the four smallest instances, DTS + HFBS each."""
        import oracle as O
        W = self.W
        order = sorted(range(len(self.insts)), key=lambda i: self.sizes[i][0] * self.sizes[i][1])
        px = 0
        for i in order[:4]:
            inst = self.insts[i]
            O.dts_solve(inst.rgba, inst.target, inst.confidence, 1, W.CFG0_FILTER,
                        W.CFG0_OPT, real=real)
            O.hfbs_solve(inst.rgba, inst.target, inst.confidence, 1, self.hp,
                         max_grid=(inst.width, inst.height, 64), real=real)
            px += inst.width * inst.height
        return px, "4 smallest of the 64 instances, DTS + HFBS each"


class Cfg3Dts(Cfg3):
    """The 64-instance batch's DTS solve alone (BF16 storage, 10
    iterations): the batched form of the 640x480 depth super-resolution, for
    the batched versus single-image comparison."""

    name = "cfg3dts_batched_dts_64_ragged_bf16"

    def __init__(self, rank: int, scale: float = 1.0, e2e_chunks: int = 16):
        super().__init__(rank, scale=scale, e2e_chunks=e2e_chunks)
        self.voxels = 0
        if scale != 1.0:
            self.name = f"{Cfg3Dts.name}_scale{scale:g}"

    def step(self):
        from domain_transform_solver_gb300._lib import check
        check(self.lib.dtsgb_batch_solve_dts(self.b.handle, ctypes.byref(self.fp),
                                             ctypes.byref(self.op), ctypes.c_float(-1.0)))

    def step_e2e(self):
        from domain_transform_solver_gb300._lib import check
        check(self.lib.dtsgb_pipeline_run(self.pipe.handle, 1, self.h_rgba, self.h_t,
                                          self.h_c, ctypes.byref(self.fp),
                                          ctypes.byref(self.op), ctypes.c_float(-1.0), None,
                                          self.h_o0, None))

    def e2e_bytes(self):
        return self.pixels * (4 + 4 + 4), self.pixels * 4

    def cpu_sample(self, real="f32"):
        import oracle as O
        W = self.W
        order = sorted(range(len(self.insts)), key=lambda i: self.sizes[i][0] * self.sizes[i][1])
        px = 0
        for i in order[:4]:
            inst = self.insts[i]
            O.dts_solve(inst.rgba, inst.target, inst.confidence, 1, W.CFG0_FILTER,
                        W.CFG0_OPT, real=real)
            px += inst.width * inst.height
        return px, "4 smallest of the 64 instances, DTS"


class Cfg0:
    """DTS depth super-resolution 640x480, FP32, 10 iterations."""

    name = "cfg0_dts_depth_superres_640x480"
    dtype = "f32"

    def __init__(self, rank: int):
        import domain_transform_solver_gb300 as D
        from domain_transform_solver_gb300 import workloads as W
        self.D, self.W = D, W
        self.inst = W.depth_sr_instance(W.SEED_BASE)
        self.pixels = self.inst.width * self.inst.height
        self.iters = W.CFG0_OPT["num_iterations"]
        self.voxels = 0

    def setup(self, stream_handle: int):
        D, W = self.D, self.W
        w, h = self.inst.width, self.inst.height
        self.s = D.DomainTransformSolver(D.ImageDim(w, h))
        self.s.SetStream(stream_handle)
        self.s.ClearAll()
        self.s.InitFrame(D.COLOR_SPACE.YCbCr, self.inst.rgba, self.inst.target,
                         self.inst.confidence)
        self.fp = D.DomainFilterParams(**W.CFG0_FILTER)
        self.op = D.DomainOptimizeParams(**W.CFG0_OPT)
        self.h_rgba = _pinned_copy(self.inst.rgba)
        self.h_t = _pinned_copy(self.inst.target)
        self.h_c = _pinned_copy(self.inst.confidence)
        self.h_out = _pinned_empty((h, w))

    def step(self):
        self.s.ComputeColorSpaceDifferential(self.fp)
        self.s.IntegrateColorDifferentials()
        self.s.Optimize(self.op)

    def step_e2e(self):
        from domain_transform_solver_gb300._lib import check
        lib, h = self.s._lib, self.s.handle
        check(lib.dtsgb_dts_init_frame(h, 1, ctypes.c_void_p(self.h_rgba.ctypes.data),
                                       ctypes.c_void_p(self.h_t.ctypes.data),
                                       ctypes.c_void_p(self.h_c.ctypes.data)))
        self.step()
        check(lib.dtsgb_dts_download(h, 5, ctypes.c_void_p(self.h_out.ctypes.data)))

    def e2e_bytes(self):
        return self.pixels * 12, self.pixels * 4

    def algorithmic_bytes(self):
        return {0: 8 * self.pixels, 1: 20 * self.pixels, 8: 8 * self.pixels}

    def cpu_sample(self, real="f32"):
        import oracle as O
        W = self.W
        O.dts_solve(self.inst.rgba, self.inst.target, self.inst.confidence, 1,
                    W.CFG0_FILTER, W.CFG0_OPT, real=real)
        return self.pixels, "one full solve"


class Cfg2:
    """DTS with a given confidence, 1280x384 RGB, Charbonnier, sigma_z 30, 15
    iterations, BF16 storage of target and confidence."""

    name = "cfg2_dts_charbonnier_1280x384_bf16"
    dtype = "bf16 storage, f32 math"

    def __init__(self, rank: int):
        import domain_transform_solver_gb300 as D
        from domain_transform_solver_gb300 import workloads as W
        self.D, self.W = D, W
        self.inst = W.stereo_instance()
        self.pixels = self.inst.width * self.inst.height
        self.iters = W.CFG2_OPT["num_iterations"]
        self.voxels = 0

    def setup(self, stream_handle: int):
        D, W = self.D, self.W
        w, h = self.inst.width, self.inst.height
        self.s = D.DomainTransformSolver(D.ImageDim(w, h), flags=D.FLAG_BF16_STORAGE)
        self.s.SetStream(stream_handle)
        self.s.ClearAll()
        self.s.InitFrame(D.COLOR_SPACE.RGB, self.inst.rgba, self.inst.target,
                         self.inst.confidence)
        self.fp = D.DomainFilterParams(**W.CFG2_FILTER)
        self.op = D.DomainOptimizeParams(**W.CFG2_OPT)
        self.h_rgba = _pinned_copy(self.inst.rgba)
        self.h_t = _pinned_copy(self.inst.target)
        self.h_c = _pinned_copy(self.inst.confidence)
        self.h_out = _pinned_empty((h, w))

    def step(self):
        self.s.ComputeColorSpaceDifferential(self.fp)
        self.s.IntegrateColorDifferentials()
        self.s.Optimize(self.op)

    def step_e2e(self):
        from domain_transform_solver_gb300._lib import check
        lib, h = self.s._lib, self.s.handle
        check(lib.dtsgb_dts_init_frame(h, 0, ctypes.c_void_p(self.h_rgba.ctypes.data),
                                       ctypes.c_void_p(self.h_t.ctypes.data),
                                       ctypes.c_void_p(self.h_c.ctypes.data)))
        self.step()
        check(lib.dtsgb_dts_download(h, 5, ctypes.c_void_p(self.h_out.ctypes.data)))

    def e2e_bytes(self):
        return self.pixels * 12, self.pixels * 4

    def algorithmic_bytes(self):
        return {0: 8 * self.pixels, 1: 16 * self.pixels, 8: 6 * self.pixels}

    def cpu_sample(self, real="f32"):
        import oracle as O
        W = self.W
        O.dts_solve(self.inst.rgba, self.inst.target, self.inst.confidence, 0,
                    W.CFG2_FILTER, W.CFG2_OPT, real=real)
        return self.pixels, "one full solve"


class Cfg1:
    """HFBS colorization 640x480, U and V channels, 64 iterations."""

    name = "cfg1_hfbs_colorization_640x480_uv"
    dtype = "f32"

    def __init__(self, rank: int):
        import domain_transform_solver_gb300 as D
        from domain_transform_solver_gb300 import workloads as W
        self.D, self.W = D, W
        self.u, self.v = W.colorization_instance()
        self.pixels = 2 * self.u.width * self.u.height
        self.iters = W.CFG1_HFBS["optim_iter_max"]
        self.voxels = 2 * 80 * 60 * 16

    def setup(self, stream_handle: int):
        D, W = self.D, self.W
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
        from domain_transform_solver_gb300._lib import check
        check(self.lib.dtsgb_batch_solve_hfbs(self.b.handle, ctypes.byref(self.hpc)))

    def step_e2e(self):
        from domain_transform_solver_gb300._lib import check
        h = self.b.handle
        check(self.lib.dtsgb_batch_upload(h, 0, self.h_rgba, self.h_t, self.h_c))
        self.step()
        check(self.lib.dtsgb_batch_download(h, 1, self.h_o))

    def e2e_bytes(self):
        return self.pixels * 12, self.pixels * 4

    def algorithmic_bytes(self):
        px, vx = self.pixels, self.voxels
        return {3: 12 * px + 12 * vx, 4: 12 * vx, 5: 28 * vx, 7: 8 * px}

    def cpu_sample(self, real="f32"):
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
        super().setup(stream_handle)  # the plain batched forward, for the ratio
        D, W = self.D, self.W
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
        from domain_transform_solver_gb300._lib import check
        h = self.gb.handle
        check(self.lib.dtsgb_batch_solve_hfbs(h, ctypes.byref(self.hpc)))
        check(self.lib.dtsgb_batch_hfbs_backward_device(h, self.p_g, self.p_gt, self.p_gc))

    def forward_only(self):
        Cfg1.step(self)

    def step_e2e(self):
        from domain_transform_solver_gb300._lib import check
        h = self.gb.handle
        check(self.lib.dtsgb_batch_upload(h, 0, self.h_rgba, self.h_t, self.h_c))
        check(self.lib.dtsgb_batch_solve_hfbs(h, ctypes.byref(self.hpc)))
        check(self.lib.dtsgb_batch_download(h, 1, self.h_o))
        check(self.lib.dtsgb_batch_hfbs_backward(h, self.h_g, self.h_gt, self.h_gc))

    def e2e_bytes(self):
        # rgba, target, confidence, upstream gradient in; result, dL/dt, dL/dc out
        return self.pixels * 16, self.pixels * 12

    def algorithmic_bytes(self):
        px, vx, k = self.pixels, self.voxels, self.iters
        return {
            3: 12 * px + 12 * vx,
            # four heavy-ball steps: read z, h, norm, b, invA; write z, h and
            # the three kept iterates
            5: 40 * vx,
            7: 8 * px,
            # the whole adjoint: read dL/dout, guide, target, confidence and
            # write dL/dt, dL/dc per pixel; per step 10 grid reads, 6 writes
            10: 24 * px + 64 * vx * k,
        }

    def cpu_sample(self, real="f32"):
        import oracle as O
        W = self.W
        o = O.OracleHFBS(self.u.width, self.u.height, 96, 96, 32, real=real)
        o.clear_all()
        o.init_frame(0, self.u.rgba, self.u.target, self.u.confidence)
        o.set_params(**W.CFG1_HFBS)
        o.optimize()
        o.backward(self.grads[0])
        return self.pixels // 2, "the U channel, forward + adjoint"


class Cfg4:
    """Differentiable DTS: 16 x 1024x768 depth super-resolution instances, FP32,
    L2, 10 iterations, the forward keeping its iterates (the automatic
    checkpoint choice: every iterate, as 14 planes fit in free memory) plus
    the adjoint (dL/dtarget, dL/dconfidence) for an N(0,1) upstream
    gradient.  One step = forward + backward; the guide's window bounds
    are held fixed (piecewise constant in the guide)."""

    name = "cfg4_dts_fwd_bwd_16x1024x768_f32"
    dtype = "f32"

    def __init__(self, rank: int, e2e_chunks: int = 4):
        self.e2e_chunks = e2e_chunks
        import domain_transform_solver_gb300 as D
        from domain_transform_solver_gb300 import workloads as W
        self.D, self.W = D, W
        self.insts, self.grads = W.grad_instances()
        self.sizes = [(i.width, i.height) for i in self.insts]
        self.pixels = sum(w * h for w, h in self.sizes)
        self.iters = W.CFG0_OPT["num_iterations"]
        self.voxels = 0

    def setup(self, stream_handle: int):
        import torch
        D, W = self.D, self.W
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
        # the plain forward (no checkpoints) of the same batch, for the ratio
        # the host-to-host path: chunks of instances on their own streams
        self.pipe = D.Pipeline(self.sizes, n_chunks=self.e2e_chunks)
        self.pipe.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)
        self.e2e_api = f"dtsgb_pipeline_run_grad, {self.pipe.n_chunks} chunks"
        self.fwd = D.Batch(self.sizes)
        self.fwd.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)
        self.fwd.set_stream(stream_handle)
        self.fwd.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in self.insts],
                        [i.target for i in self.insts], [i.confidence for i in self.insts])

    def step(self):
        from domain_transform_solver_gb300._lib import check
        check(self.lib.dtsgb_batch_solve_dts(self.b.handle, ctypes.byref(self.fp),
                                             ctypes.byref(self.op), ctypes.c_float(-1.0)))
        check(self.lib.dtsgb_batch_dts_backward_device(self.b.handle, self.p_g, self.p_gt,
                                                       self.p_gc))

    def forward_only(self):
        from domain_transform_solver_gb300._lib import check
        check(self.lib.dtsgb_batch_solve_dts(self.fwd.handle, ctypes.byref(self.fp),
                                             ctypes.byref(self.op), ctypes.c_float(-1.0)))

    def step_e2e(self):
        from domain_transform_solver_gb300._lib import check
        check(self.lib.dtsgb_pipeline_run_grad(self.pipe.handle, 1, self.h_rgba, self.h_t,
                                               self.h_c, ctypes.byref(self.fp),
                                               ctypes.byref(self.op), self.h_g, self.h_v,
                                               self.h_gt, self.h_gc))

    def e2e_bytes(self):
        # rgba, target, confidence, upstream gradient in; v, dL/dt, dL/dc out
        return self.pixels * 16, self.pixels * 12

    def algorithmic_bytes(self):
        px = self.pixels
        return {
            0: 8 * px,   # read guide, write packed bounds
            1: 20 * px,  # read v, t, c, bounds; write v (f32)
            8: 8 * px,   # read t, write v
            9: 40 * px,  # read g, v_k, t, c, bounds; read+write dL/dt, dL/dc; write g
        }

    def cpu_sample(self, real="f32"):
        """A bounded sample: one instance, forward + adjoint by the FP32 port."""
        import oracle as O
        W = self.W
        inst, g = self.insts[0], self.grads[0]
        o = O.OracleDTS(inst.width, inst.height, real=real)
        o.init_frame(1, inst.rgba, inst.target, inst.confidence)
        o.differential(W.CFG0_FILTER["sigma_x"], W.CFG0_FILTER["sigma_y"],
                       W.CFG0_FILTER["sigma_r"])
        o.integrate()
        op = W.CFG0_OPT
        o.backward(op["num_iterations"], op["loss"], op["lambda_"], op["sigma_z"],
                   op["step_size"], g)
        return inst.width * inst.height, "1 of the 16 instances, forward + adjoint"


WORKLOADS = {"cfg3": Cfg3, "cfg3dts": Cfg3Dts, "cfg0": Cfg0, "cfg1": Cfg1, "cfg2": Cfg2,
             "cfg4": Cfg4, "cfg1grad": Cfg1Grad}


# ---- arms ----------------------------------------------------------------------
def make_workload(args, rank):
    if args.workload == "cfg3":
        return Cfg3(rank, scale=args.scale, e2e_chunks=args.e2e_chunks)
    if args.workload == "cfg3dts":
        return Cfg3Dts(rank, scale=args.scale, e2e_chunks=args.e2e_chunks)
    if args.workload == "cfg4":
        return Cfg4(rank, e2e_chunks=args.e2e_chunks if args.e2e_chunks_set else 4)
    return WORKLOADS[args.workload](rank)


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


def max_over_ranks(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cores_used():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def cpu_baseline(wl, budget_s=12.0, real="f32"):
    import oracle as O
    O.build()
    wl.cpu_sample(real)  # warm-up (page-in, thread pool)
    px, t0, n = 0, time.perf_counter(), 0
    desc = ""
    while True:
        p, desc = wl.cpu_sample(real)
        px += p
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 500:
            break
    return {"value": px / el / 1e6, "unit": "Mpix/s", "cores": cores_used(), "kind": "port",
            "sample": f"{n} x ({desc}) of {wl.name} by the FP32 oracle port "
                      f"(OpenMP, {cores_used()} threads), {el:.1f} s"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    wl = make_workload(args, rank)
    import oracle as O
    O.build()
    desc = ""
    for _ in range(args.warmup):
        wl.cpu_sample()
    t0 = time.perf_counter()
    px = 0
    for _ in range(args.steps):
        p, desc = wl.cpu_sample()
        px += p
    el = time.perf_counter() - t0
    value = px / el / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpix/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.name, "pixels_per_step": wl.pixels,
                   "iterations": wl.iters, "sample_per_step": desc},
        "cpu_baseline": {"value": value, "unit": "Mpix/s", "cores": cores_used(),
                         "kind": "port", "sample": f"{args.steps} x ({desc})"},
        "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference's CUDA build cannot be built with this toolchain (empty "
                "libcua/CUB submodules, CUDA 8/9-era CUB API); its algorithm's CPU "
                "restatement is timed on all host threads",
    }
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    import domain_transform_solver_gb300 as D  # noqa: F401  (loads libdtsgb.so)
    from domain_transform_solver_gb300 import _lib
    lib = _lib.load()
    wl = make_workload(args, rank)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    wl.setup(stream.cuda_stream)
    big = wl.pixels * 16 > 2 * (129 << 20)
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
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    for k in range(args.steps):
        if flush is not None:
            flush.zero_()  # L2 flush between steps, outside the step's events
        ev[k][0].record(stream)
        wl.step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(world, sum(step_ms))
    ms_per_step = total_ms / args.steps
    value = world * wl.pixels / (ms_per_step * 1e-3) / 1e6

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
    pev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for k in range(args.steps):
        if flush is not None:
            flush.zero_()
        pev[k][0].record(stream)
        wl.step()
        pev[k][1].record(stream)
    torch.cuda.synchronize()
    prof_ms_per_step = sum(a.elapsed_time(b) for a, b in pev) / args.steps
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
    algo = wl.algorithmic_bytes()
    peak, peak_kind = peaks()
    kernels = {}
    for kid, (n, t) in per_kernel.items():
        avg = t / n
        rec = {"launches_per_step": n / steps_seen, "avg_launch_ms": avg,
               "share_of_step": (t / steps_seen) / prof_ms_per_step}
        if kid in algo:
            rec["achieved_gbs"] = algo[kid] / (avg * 1e-3) / 1e9
            rec["frac_of_measured_hbm"] = rec["achieved_gbs"] / peak
        kernels[KERNEL_NAMES[kid]] = rec
    dom = max(per_kernel, key=lambda k: per_kernel[k][1])
    n_dom, t_dom = per_kernel[dom]
    avg_dom = t_dom / n_dom
    achieved = algo[dom] / (avg_dom * 1e-3) / 1e9 if dom in algo else None
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get(wl.name, {}).get(KERNEL_NAMES[dom])

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
    e2e_ms = max_over_ranks(world, e0.elapsed_time(e1)) / e_steps
    h2d, d2h = wl.e2e_bytes()
    e2e_value = world * wl.pixels / (e2e_ms * 1e-3) / 1e6

    fwd_ratio = None
    if hasattr(wl, "forward_only"):
        for _ in range(3):
            wl.forward_only()
        torch.cuda.synchronize()
        f_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                for _ in range(args.steps)]
        for k in range(args.steps):
            if flush is not None:
                flush.zero_()
            f_ev[k][0].record(stream)
            wl.forward_only()
            f_ev[k][1].record(stream)
        torch.cuda.synchronize()
        fwd_ms = max_over_ranks(world, sum(a.elapsed_time(b) for a, b in f_ev)) / args.steps
        fwd_ratio = {"forward_ms": fwd_ms, "fwd_bwd_ms": ms_per_step,
                     "fwd_bwd_over_forward": ms_per_step / fwd_ms}

    line = {
        "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": wl.dtype, "data": "synthetic (seeded, shapes of the reference's datasets)",
        "config": {"workload": wl.name, "pixels_per_step": wl.pixels,
                   "voxels_per_step": wl.voxels, "iterations": wl.iters,
                   "l2": ("inputs larger than L2" if big
                          else "flushed between steps (256 MB write)"),
                   "parallelism": f"independent instances x{world} GPUs",
                   "guide_state_reuse": "off (every step recomputes all of it)"},
        "e2e": {"value": e2e_value, "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                **({"api": wl.e2e_api} if hasattr(wl, "e2e_api") else {})},
        "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES[dom], "achieved": achieved,
                     "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": traffic, "avg_launch_ms": avg_dom,
                     "algorithmic_bytes_per_launch": algo.get(dom)},
        "kernels": kernels,
        "profiled_ms_per_step": prof_ms_per_step,
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "clocks": clocks,
    }
    if fwd_ratio:
        line["fwd_bwd"] = fwd_ratio
    if rank == 0 and world == 1:
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
    ap.add_argument("--e2e-chunks", type=int, default=None,
                    help="chunks of the overlapped host-to-host e2e run (cfg3: 16, cfg4: 4)")
    args = ap.parse_args()
    args.e2e_chunks_set = args.e2e_chunks is not None
    if args.e2e_chunks is None:
        args.e2e_chunks = 16
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
