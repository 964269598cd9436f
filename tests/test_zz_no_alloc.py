"""The allocation-free DTS entry point, dtsgb_dts_solve_noalloc.

It serves callers that cannot call cudaMalloc (code inside another
framework's CUDA-graph capture, real-time pipelines that forbid allocation
after start-up, hosts whose own allocator must own all device memory): they
pass device inputs and the output, and the solve's scratch lives in a static
device array of the library.  Its window bounds sum edge weights in float
where the allocating path takes fixed-point prefix differences, so the two
paths agree within the parity tolerance, not bit for bit; against the FP64
oracle it is held to the same bar as the allocating path.  This file sorts
last so that a run stopping at the first failure has run everything else
first; it also passes alone.
"""
import ctypes

import numpy as np
import pytest

import parity as P

pytestmark = pytest.mark.gpu


def _class_api_solve(D, inst, cs, filt, opt, conf=True, overwrite=-1.0):
    h, w = inst.target.shape
    s = D.DomainTransformSolver(D.ImageDim(w, h))
    s.ClearAll()
    s.InitFrame(D.COLOR_SPACE(cs), inst.rgba, inst.target, inst.confidence if conf else None)
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(**filt))
    s.IntegrateColorDifferentials()
    s.Optimize(D.DomainOptimizeParams(**opt), overwrite)
    return s.Download(D.ImageType.OPTIMIZED_QUANTITY)


def _noalloc_solve(D, lib, inst, cs, filt, opt, use_conf=True, overwrite=-1.0):
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
        ctypes.byref(D.DomainOptimizeParams(**opt)._c()), ctypes.c_float(overwrite),
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert st == 0, lib.dtsgb_last_error()
    stream.synchronize()
    return out.cpu().numpy()


def _lib(D):
    from domain_transform_solver_gb300 import _lib
    return _lib.load()


def test_noalloc_matches_the_allocating_entry_point_on_two_calls(gpu_ready):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    lib = _lib(D)
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


@pytest.mark.parametrize("loss,iters,use_conf,overwrite", [
    (1, 6, True, 0.5),    # overwrite in (0, 1): both halves of the X pass
    (1, 6, False, -1.0),  # no confidence: ones
    (2, 4, False, 0.5),   # Charbonnier, no confidence, overwrite everywhere
    (0, 5, True, -1.0),   # L1 runs no kernel: the target
    (1, 0, True, -1.0),   # zero iterations: the target
    (1, 1, True, 0.5),    # one iteration, odd ping-pong
])
def test_noalloc_variants_match_the_allocating_entry_point(gpu_ready, loss, iters, use_conf,
                                                          overwrite):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    lib = _lib(D)
    inst = W.depth_sr_instance(911 + iters, 173, 129, n_poly=10, sample_frac=0.3)
    rng = np.random.default_rng(iters)
    inst.confidence = rng.random(inst.target.shape).astype(np.float32)  # graded
    opt = dict(W.CFG0_OPT, loss=loss, num_iterations=iters)
    ref = _class_api_solve(D, inst, 1, W.CFG0_FILTER, opt, use_conf, overwrite)
    for _ in range(2):  # two calls in a row
        out = _noalloc_solve(D, lib, inst, 1, W.CFG0_FILTER, opt, use_conf, overwrite)
        if loss == 0 or iters == 0:
            assert np.array_equal(out, inst.target)
        assert np.abs(out - ref).max() <= P.TOL_REL * P.target_range(inst.target)


def test_noalloc_against_the_fp64_oracle(gpu_ready, oracle_mod):
    """An instance whose every window decision lies at least 2.7e-4 from its
    threshold (a margin some hundred times the FP32 rounding of a window
    sum), so each window the float sums choose must be the oracle's: the
    output is held to max-abs 1e-4 x range against the FP64 oracle on the
    oracle's own windows."""
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    lib = _lib(D)
    inst = W.depth_sr_instance(1048, 120, 90, n_poly=8, sample_frac=0.2)
    f, sz = W.CFG0_FILTER, W.CFG0_OPT["sigma_z"]
    o = oracle_mod.OracleDTS(120, 90)
    o.init_frame(1, inst.rgba, inst.target, inst.confidence)
    o.differential(f["sigma_x"], f["sigma_y"], f["sigma_r"])
    o.integrate()
    for axis in (0, 1):
        _, _, margin = o.bounds(axis, sz)
        assert np.abs(margin).min() > 3e-5 * (sz + 1.0)
    for loss, overwrite, use_conf in ((1, -1.0, True), (2, 0.5, True), (1, -1.0, False)):
        opt = dict(W.CFG0_OPT, loss=loss, num_iterations=8)
        o.init_frame(1, inst.rgba, inst.target, inst.confidence if use_conf else None)
        o.differential(f["sigma_x"], f["sigma_y"], f["sigma_r"])
        o.integrate()
        o.optimize(opt["num_iterations"], loss, opt["lambda_"], sz, opt["step_size"],
                   overwrite)
        ref = o.download(5)
        out = _noalloc_solve(D, lib, inst, 1, f, opt, use_conf, overwrite)
        err = float(np.abs(out - ref).max()) / P.target_range(inst.target)
        assert err <= P.TOL_REL, (loss, overwrite, use_conf, err)


def test_noalloc_rejects_what_it_cannot_run(gpu_ready):
    """Host-side checks, made before anything is enqueued (the pointers
    below are never dereferenced)."""
    D = gpu_ready
    from domain_transform_solver_gb300 import _lib as L
    lib = L.load()
    fp = ctypes.byref(D.DomainFilterParams(8, 8, 0.1)._c())

    def call(w, h, opt, ptrs=(16, 16, 32)):
        return lib.dtsgb_dts_solve_noalloc(
            w, h, 1, ctypes.c_void_p(ptrs[0]), ctypes.c_void_p(ptrs[1]), None, fp,
            ctypes.byref(opt._c()), ctypes.c_float(-1.0), ctypes.c_void_p(ptrs[2]), None)

    assert call(2048, 1024, D.DomainOptimizeParams()) == L.DTSGB_ERR_UNSUPPORTED
    assert b"exceeds its static scratch" in lib.dtsgb_last_error()
    big_sigma = D.DomainOptimizeParams(num_iterations=2, loss=1, sigma_z=97.0)
    assert call(64, 64, big_sigma) == L.DTSGB_ERR_UNSUPPORTED
    assert b"sigma_z must be in (0, 97)" in lib.dtsgb_last_error()
    ok_sigma = D.DomainOptimizeParams(num_iterations=2, loss=1, sigma_z=8.0)
    assert call(64, 64, ok_sigma, ptrs=(16, 18, 32)) == L.DTSGB_ERR_INVALID_ARGUMENT
    assert b"4-byte aligned" in lib.dtsgb_last_error()
