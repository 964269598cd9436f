"""Guide-state reuse in the class API (dtsgb_dts_upload_targets,
dtsgb_hfbs_upload_targets): video frames whose target changes while the
guide stays.  Each frame's result equals a fresh handle's InitFrame + solve
bitwise, the window-bound search (DTS) and the bistochastization (HFBS)
run only for the first frame, and a changed sigma_z, grid or guide makes
them run again."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K_BOUNDS, K_BISTOCH = 0, 4


def _launches(L, kind):
    n, ms = ctypes.c_int(), ctypes.c_double()
    assert L.dtsgb_profile_read(kind, ctypes.byref(n), ctypes.byref(ms)) == 0
    return n.value


@pytest.fixture
def profiled(gpu_ready):
    from domain_transform_solver_gb300 import _lib
    L = _lib.load()
    L.dtsgb_profile_enable(1)
    L.dtsgb_profile_reset()
    yield L
    L.dtsgb_profile_enable(0)


def _frames(inst, n=3):
    rng = np.random.default_rng(7)
    return [(inst.target * (1.0 + 0.1 * k) + rng.normal(0, 0.01, inst.target.shape))
            .astype(np.float32) for k in range(n)]


def test_dts_class_api_keeps_the_windows(gpu_ready, profiled):
    D, L = gpu_ready, profiled
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(41, 300, 200, n_poly=10, sample_frac=0.2)
    h, w = inst.target.shape
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    s = D.DomainTransformSolver(D.ImageDim(w, h))
    s.ClearAll()
    for k, frame in enumerate(_frames(inst) + [inst.target]):
        sz = 8.0 if k < 3 else 6.0  # the last frame changes sigma_z
        op = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=4, sigma_z=sz))
        before = _launches(L, K_BOUNDS)
        if k == 0:
            s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, frame, inst.confidence)
            s.ComputeColorSpaceDifferential(fp)
            s.IntegrateColorDifferentials()
        else:
            s.UploadTargets(frame, inst.confidence)
        s.Optimize(op)
        out = s.Download(D.ImageType.OPTIMIZED_QUANTITY)
        searched = _launches(L, K_BOUNDS) - before
        assert searched == (1 if k in (0, 3) else 0), (k, searched)
        fresh = D.DomainTransformSolver(D.ImageDim(w, h))
        fresh.ClearAll()
        fresh.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, frame, inst.confidence)
        fresh.ComputeColorSpaceDifferential(fp)
        fresh.IntegrateColorDifferentials()
        fresh.Optimize(op)
        assert np.array_equal(out, fresh.Download(D.ImageType.OPTIMIZED_QUANTITY))
    # a new guide through InitFrame searches again
    before = _launches(L, K_BOUNDS)
    s.InitFrame(D.COLOR_SPACE.YCbCr, np.ascontiguousarray(inst.rgba[::-1]), inst.target,
                inst.confidence)
    s.ComputeColorSpaceDifferential(fp)
    s.IntegrateColorDifferentials()
    s.Optimize(D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=2)))
    assert _launches(L, K_BOUNDS) - before == 1


def test_dts_upload_targets_without_confidence_means_ones(gpu_ready):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(42, 160, 120, n_poly=6)
    s = D.DomainTransformSolver(D.ImageDim(160, 120))
    s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, inst.confidence)
    s.UploadTargets(inst.target)
    assert (s.Download(D.ImageType.CONFIDENCE) == 1.0).all()
    assert np.array_equal(s.Download(D.ImageType.TARGET), inst.target)


def test_hfbs_class_api_keeps_the_normalisation(gpu_ready, profiled):
    D, L = gpu_ready, profiled
    from domain_transform_solver_gb300 import workloads as W
    u, _ = W.colorization_instance(43, 240, 160, n_poly=6, frac=0.05)
    h, w = u.target.shape
    base = dict(W.CFG1_HFBS, optim_iter_max=12)
    s = D.HFBS(D.ImageDim(w, h), 64, 64, 32)
    s.SetImageDim(D.ImageDim(w, h))
    s.ClearAll()
    for k, frame in enumerate(_frames(u, 3) + [u.target]):
        params = base if k < 3 else dict(base, sigma_l=20.0)  # the last frame: other grid
        s.SetFilterParams(D.HFBSGridParams(**params))
        before = _launches(L, K_BISTOCH)
        if k == 0:
            s.InitFrame(D.COLOR_SPACE.YYY, u.rgba, frame, u.confidence)
        else:
            s.UploadTargets(frame, u.confidence)
        s.Optimize()
        out = s.Download(D.ImageType.OPTIMIZED_QUANTITY)
        ran = _launches(L, K_BISTOCH) - before
        assert (ran > 0) == (k in (0, 3)), (k, ran)
        fresh = D.HFBS(D.ImageDim(w, h), 64, 64, 32)
        fresh.SetImageDim(D.ImageDim(w, h))
        fresh.SetFilterParams(D.HFBSGridParams(**params))
        fresh.ClearAll()
        fresh.InitFrame(D.COLOR_SPACE.YYY, u.rgba, frame, u.confidence)
        fresh.Optimize()
        assert np.array_equal(out, fresh.Download(D.ImageType.OPTIMIZED_QUANTITY))
    # ClearAll clears the grids: the next solve bistochastizes again
    s.ClearAll()
    s.InitFrame(D.COLOR_SPACE.YYY, u.rgba, u.target, u.confidence)
    before = _launches(L, K_BISTOCH)
    s.Optimize()
    assert _launches(L, K_BISTOCH) - before > 0
