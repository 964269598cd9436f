"""The allocation-free DTS entry point, dtsgb_dts_solve_noalloc.

It serves callers that cannot call cudaMalloc (code inside another
framework's CUDA-graph capture, real-time pipelines that forbid allocation
after start-up, hosts whose own allocator must own all device memory): they
pass device inputs and the output, and the solve's scratch lives in a static
device array of the library.  This file sorts last so that a run stopping at
the first failure has run everything else first; it also passes alone.
"""
import ctypes

import numpy as np
import pytest

import parity as P

pytestmark = pytest.mark.gpu


def _class_api_solve(D, inst, cs, filt, opt):
    h, w = inst.target.shape
    s = D.DomainTransformSolver(D.ImageDim(w, h))
    s.ClearAll()
    s.InitFrame(D.COLOR_SPACE(cs), inst.rgba, inst.target, inst.confidence)
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(**filt))
    s.IntegrateColorDifferentials()
    s.Optimize(D.DomainOptimizeParams(**opt))
    return s.Download(D.ImageType.OPTIMIZED_QUANTITY)


def _noalloc_solve(D, lib, inst, cs, filt, opt, use_conf=True):
    import torch
    dev = torch.device("cuda", 0)
    h, w = inst.target.shape
    # the test owns the device buffers; the entry point allocates nothing
    rgba = torch.from_numpy(inst.rgba.copy()).to(dev)
    t = torch.from_numpy(inst.target.copy()).to(dev)
    c = torch.from_numpy(inst.confidence.copy()).to(dev) if use_conf else None
    out = torch.full((h, w), float("nan"), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = lib.dtsgb_dts_solve_noalloc(
        w, h, int(cs), ctypes.c_void_p(rgba.data_ptr()), ctypes.c_void_p(t.data_ptr()),
        ctypes.c_void_p(c.data_ptr()) if c is not None else None,
        ctypes.byref(D.DomainFilterParams(**filt)._c()),
        ctypes.byref(D.DomainOptimizeParams(**opt)._c()), ctypes.c_float(-1.0),
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert st == 0, lib.dtsgb_last_error()
    stream.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_the_allocating_entry_point_on_two_calls(gpu_ready):
    D = gpu_ready
    from domain_transform_solver_gb300 import _lib
    from domain_transform_solver_gb300 import workloads as W
    lib = _lib.load()
    # two calls in a row on different images: the second reuses the static
    # scratch the first left behind
    cases = [
        (W.depth_sr_instance(901, 320, 240, n_poly=12), 1, W.CFG0_FILTER, W.CFG0_OPT),
        (W.stereo_instance(902, 200, 150, n_poly=9), 0, W.CFG2_FILTER,
         dict(W.CFG2_OPT, num_iterations=5)),
    ]
    for inst, cs, filt, opt in cases:
        ref = _class_api_solve(D, inst, cs, filt, opt)
        out = _noalloc_solve(D, lib, inst, cs, filt, opt)
        assert np.isfinite(out).all()
        assert np.abs(out - ref).max() <= P.TOL_REL * P.target_range(inst.target)


def test_noalloc_rejects_images_beyond_its_scratch(gpu_ready):
    from domain_transform_solver_gb300 import _lib
    lib = _lib.load()
    D = gpu_ready
    st = lib.dtsgb_dts_solve_noalloc(
        2048, 1024, 1, ctypes.c_void_p(16), ctypes.c_void_p(16), None,
        ctypes.byref(D.DomainFilterParams(8, 8, 0.1)._c()),
        ctypes.byref(D.DomainOptimizeParams()._c()), ctypes.c_float(-1.0),
        ctypes.c_void_p(32), None)
    assert st == _lib.DTSGB_ERR_UNSUPPORTED
    assert b"exceeds its static scratch" in lib.dtsgb_last_error()
