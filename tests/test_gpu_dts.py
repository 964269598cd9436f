"""GPU parity of the DTS path (DomainTransformFilter / DomainTransformSolver)
against the FP64 oracle, through the C ABI."""
import numpy as np
import pytest

import parity as P

pytestmark = pytest.mark.gpu


def _solver(D, w, h, flags=0, max_dims=None):
    mw, mh = max_dims or (w, h)
    s = D.DomainTransformSolver(D.ImageDim(mw, mh), flags=flags)
    s.SetImageDim(D.ImageDim(w, h))
    s.ClearAll()
    return s


def _run_dts(D, inst, cs, filt, opt, overwrite=-1.0, flags=0, conf=True):
    h, w = inst.target.shape
    s = _solver(D, w, h, flags)
    s.InitFrame(D.COLOR_SPACE(cs), inst.rgba, inst.target,
                inst.confidence if conf else None)
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(**filt))
    s.IntegrateColorDifferentials()
    s.Optimize(D.DomainOptimizeParams(**opt), overwrite)
    return s.Download(D.ImageType.OPTIMIZED_QUANTITY), s


def _parity_dts(D, O, inst, cs, filt, opt, overwrite=-1.0, flags=0, bf16=False,
                ref_y=True):
    v_gpu, s = _run_dts(D, inst, cs, filt, opt, overwrite, flags)
    t, c = inst.target, inst.confidence
    if bf16:
        t, c = P.bf16_round(t), P.bf16_round(c)
    sz = float(np.float32(opt["sigma_z"]))
    # windows: GPU vs FP64 search on the FP64 domain transform
    o = O.OracleDTS(t.shape[1], t.shape[0], ref_y_limit=ref_y)
    o.init_frame(cs, inst.rgba, t, c)
    o.differential(filt["sigma_x"], filt["sigma_y"], filt["sigma_r"])
    o.integrate()
    stats = {}
    overrides = {}
    for axis in (0, 1):
        g = s.DebugBounds(axis, sz)
        ob = o.bounds(axis, sz)
        stats[axis] = P.check_bounds(g, ob, sz)
        assert stats[axis][1] == 0, f"axis {axis}: non-tie bound mismatches {stats[axis]}"
        overrides[(axis, sz)] = g
    # value path on the GPU's windows
    v_ora, _ = O.dts_solve(inst.rgba, t, c, cs, filt, opt, overwrite,
                           ref_y_limit=ref_y, overrides=overrides)
    rng_t = P.target_range(t)
    err = np.abs(v_gpu.astype(np.float64) - v_ora)
    assert np.isfinite(v_gpu).all()
    assert err.max() <= P.TOL_REL * rng_t, (err.max(), rng_t)
    # end to end against the oracle's own windows: RMSE bar
    v_own, _ = O.dts_solve(inst.rgba, t, c, cs, filt, opt, overwrite, ref_y_limit=ref_y)
    rmse = float(np.sqrt(np.mean((v_gpu - v_own) ** 2)))
    assert rmse <= P.TOL_REL * rng_t, (rmse, rng_t, stats)
    return v_gpu, stats


def test_cfg0_depth_superres_full_size(gpu_ready, oracle_mod):
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(W.SEED_BASE)
    _parity_dts(gpu_ready, oracle_mod, inst, 1, W.CFG0_FILTER, W.CFG0_OPT)


def test_cfg2_stereo_charbonnier_bf16_storage(gpu_ready, oracle_mod):
    from domain_transform_solver_gb300 import workloads as W
    inst = W.stereo_instance()
    _parity_dts(gpu_ready, oracle_mod, inst, 0, W.CFG2_FILTER, W.CFG2_OPT,
                flags=gpu_ready.FLAG_BF16_STORAGE, bf16=True)


@pytest.mark.parametrize("w,h", [(1, 1), (1, 9), (9, 1), (3, 200), (200, 3),
                                 (65, 65), (129, 77), (40, 300), (333, 250)])
@pytest.mark.parametrize("ref_y", [True, False])
def test_ragged_and_tiny_sizes(gpu_ready, oracle_mod, w, h, ref_y):
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(w * 7 + h, w, h, n_poly=6, stride=3)
    flags = 0 if ref_y else gpu_ready.FLAG_FIX_Y_LIMIT
    _parity_dts(gpu_ready, oracle_mod, inst, 1, W.CFG0_FILTER,
                dict(W.CFG0_OPT, num_iterations=4), flags=flags, ref_y=ref_y)


@pytest.mark.parametrize("sigma_z", [0.5, 3.0, 8.0, 12.7, 30.0, 61.0])
def test_sigma_sweep_charbonnier(gpu_ready, oracle_mod, sigma_z):
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(99, 180, 130, n_poly=12, sample_frac=0.2)
    opt = dict(num_iterations=3, loss=2, lambda_=0.7, sigma_z=sigma_z, step_size=0.9)
    _parity_dts(gpu_ready, oracle_mod, inst, 2, dict(sigma_x=6.0, sigma_y=9.0,
                                                     sigma_r=0.2), opt)


def test_overwrite_target_above_conf(gpu_ready, oracle_mod):
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(5, 160, 120, n_poly=10, sample_frac=0.1)
    rng = np.random.default_rng(1)
    inst.confidence[:] = rng.random(inst.confidence.shape).astype(np.float32)
    _parity_dts(gpu_ready, oracle_mod, inst, 1, W.CFG0_FILTER,
                dict(W.CFG0_OPT, num_iterations=5), overwrite=0.6)


def test_l1_loss_and_zero_iterations_return_target(gpu_ready):
    from domain_transform_solver_gb300 import workloads as W
    D = gpu_ready
    inst = W.depth_sr_instance(8, 70, 50, n_poly=5)
    for opt in (dict(W.CFG0_OPT, loss=0), dict(W.CFG0_OPT, num_iterations=0)):
        v, _ = _run_dts(D, inst, 1, W.CFG0_FILTER, opt)
        assert np.array_equal(v, inst.target)


def test_optimize_without_differential_uses_zero_transform(gpu_ready, oracle_mod):
    """After ClearAll the reference's dH/ct buffers are zero: every window is
    the pixel itself, so the X step sees B = v."""
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(9, 64, 48, n_poly=5, sample_frac=0.3)
    s = _solver(D, 64, 48)
    s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, inst.confidence)
    s.Optimize(D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=3)))
    v = s.Download(D.ImageType.OPTIMIZED_QUANTITY)
    o = oracle_mod.OracleDTS(64, 48)
    o.clear_all()
    o.init_frame(1, inst.rgba, inst.target, inst.confidence)
    o.optimize(3, 1, 0.99, 8.0, 0.99)
    assert np.abs(v - o.download(5)).max() <= 1e-5 * P.target_range(inst.target)


def test_downloads_color_differential_integral(gpu_ready, oracle_mod):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(10, 300, 200, n_poly=10)
    s = _solver(D, 300, 200, max_dims=(320, 240))
    s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, None)
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(8.0, 8.0, 0.2))
    s.IntegrateColorDifferentials()
    o = oracle_mod.OracleDTS(300, 200)
    o.init_frame(1, inst.rgba, inst.target, None)
    o.differential(8.0, 8.0, 0.2)
    o.integrate()
    assert np.array_equal(s.Download(D.ImageType.COLOR_IMAGE), o.download(0))
    dh = s.Download(D.ImageType.DIFFERENTIAL)
    assert np.allclose(dh, o.download(1), rtol=1e-6, atol=0)
    ct = s.Download(D.ImageType.INTEGRAL)
    assert np.allclose(ct, o.download(2), rtol=1e-5, atol=1e-4)
    assert np.array_equal(s.Download(D.ImageType.TARGET), inst.target)
    assert np.array_equal(s.Download(D.ImageType.CONFIDENCE), np.ones_like(inst.target))


@pytest.mark.parametrize("num_iter", [1, 3, 7])
def test_filter_parity(gpu_ready, oracle_mod, num_iter):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(12, 256, 192, n_poly=15)
    rng = np.random.default_rng(3)
    inp = rng.normal(0, 2, (192, 256)).astype(np.float32)
    f = D.DomainTransformFilter(D.ImageDim(256, 192))
    f.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba)
    out = f.Filter(D.DomainFilterParams(8.0, 8.0, 0.2), inp, num_iter)
    o = oracle_mod.OracleDTS(256, 192)
    o.init_frame(1, inst.rgba)
    o.differential(8.0, 8.0, 0.2)
    o.integrate()
    for sx, sy in P.filter_sigmas(8.0, 8.0, num_iter):
        for axis, sg in ((0, sx), (1, sy)):
            g = f.DebugBounds(axis, sg)
            assert P.check_bounds(g, o.bounds(axis, sg), sg)[1] == 0
            o.add_bounds_override(axis, sg, *g)
    ref = o.filter(8.0, 8.0, 0.2, inp, num_iter)
    assert np.abs(out - ref).max() <= P.TOL_REL * P.target_range(inp)
    # the filter-only class does not expose solver images
    assert np.array_equal(f.Download(D.ImageType.OPTIMIZED_QUANTITY),
                          np.zeros_like(inp))


def test_compute_confidence_and_auto_confidence_solve(gpu_ready, oracle_mod):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(13, 200, 150, n_poly=12, sample_frac=0.5)
    inst.target[:] = np.where(inst.confidence > 0, inst.target, 3.0)
    cp = D.DomainFilterParamsVec1(8.0, 8.0, 0.2, [16.0, 0.0])
    s = _solver(D, 200, 150)
    s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, None)
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(8.0, 8.0, 0.1))
    s.IntegrateColorDifferentials()
    s.ComputeConfidence(cp, 7)
    conf = s.Download(D.ImageType.CONFIDENCE)
    o = oracle_mod.OracleDTS(200, 150)
    o.init_frame(1, inst.rgba, inst.target, None)
    o.differential(8.0, 8.0, 0.2)
    o.integrate()
    for sx, sy in P.filter_sigmas(8.0, 8.0, 3):
        for axis, sg in ((0, sx), (1, sy)):
            g = s.DebugBounds(axis, sg)
            assert P.check_bounds(g, o.bounds(axis, sg), sg)[1] == 0
            o.add_bounds_override(axis, sg, *g)
    o.compute_confidence(8.0, 8.0, 0.2, 16.0, 7)
    ref = o.download(4)
    assert (conf[:, :8] == 0).all()
    # DT(t^2) - DT(t)^2 within rounding of 0 may change sign between FP32 and
    # FP64 (conf 0 vs ~1): such pixels are counted, not compared
    dtz2 = o.download(5)
    dtz = o.filter(8.0, 8.0, 0.2, inst.target, 3)
    var64 = dtz2 - dtz ** 2
    near0 = np.abs(var64) <= 1e-5 * np.abs(dtz2).max()
    err = np.abs(conf - ref)
    bad = (err > 1e-4) & ~near0
    assert bad.sum() == 0, (int(bad.sum()), float(err[~near0].max()))
    # the DT of the confidence sigmas stays in place for Optimize (reference
    # ordering of Solve<DtsOptions>)
    opt = dict(W.CFG0_OPT, num_iterations=3)
    s.Optimize(D.DomainOptimizeParams(**opt))
    v = s.Download(D.ImageType.OPTIMIZED_QUANTITY)
    o.clear_bounds_override()
    o2 = oracle_mod.OracleDTS(200, 150)
    o2.init_frame(1, inst.rgba, inst.target, conf)
    o2.differential(8.0, 8.0, 0.2)
    o2.integrate()
    for axis in (0, 1):
        o2.add_bounds_override(axis, 8.0, *s.DebugBounds(axis, 8.0))
    o2.optimize(3, 1, 0.99, 8.0, 0.99)
    assert np.abs(v - o2.download(5)).max() <= P.TOL_REL * P.target_range(inst.target)


def test_deterministic_and_error_paths(gpu_ready):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(14, 128, 96, n_poly=8)
    a, _ = _run_dts(D, inst, 1, W.CFG0_FILTER, W.CFG0_OPT)
    b, s = _run_dts(D, inst, 1, W.CFG0_FILTER, W.CFG0_OPT)
    assert np.array_equal(a, b)
    with pytest.raises(D.DtsgbError) as e:
        s.SetImageDim(D.ImageDim(129, 96))
    assert e.value.status == 2
    with pytest.raises(D.DtsgbError):
        s.Optimize(D.DomainOptimizeParams(num_iterations=2, sigma_z=float("nan")))
    with pytest.raises(D.DtsgbError):
        s.Optimize(D.DomainOptimizeParams(num_iterations=2, sigma_z=300.0))
    with pytest.raises(D.DtsgbError):
        s.ComputeColorSpaceDifferential(D.DomainFilterParams(8.0, 8.0, 0.0))
    # the handle stays usable after rejected calls
    c, _ = _run_dts(D, inst, 1, W.CFG0_FILTER, W.CFG0_OPT)
    assert np.array_equal(a, c)
