"""The committed golden fixtures (tests/golden/, written by
tests/golden/make_golden.py from the FP64 oracle): the oracle must still
reproduce them (CPU), and the CUDA path must match them through the C ABI
(GPU) -- windows and counts exactly, float outputs within 1e-4 of the target
range, gradients within 1e-4 of their largest magnitude."""
from pathlib import Path

import numpy as np
import pytest

import parity as P

GOLDEN = Path(__file__).resolve().parent / "golden"
DTS_FILTER = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.1)
DTS_OPT = dict(num_iterations=5, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
HFBS = dict(sigma_x=8.0, sigma_y=8.0, sigma_l=16.0, lambda_=8.0, alpha=1.0, beta=0.9,
            bistoch_iter_max=20, optim_iter_max=24, neg_exp_beta=0.9)
HFBS_GRID = (12, 8, 32)


def _load(name):
    return np.load(GOLDEN / name)


def test_fixture_parameters_are_the_generators():
    import sys
    sys.path.insert(0, str(GOLDEN))
    import make_golden as M
    from domain_transform_solver_gb300 import workloads as W
    assert M.DTS_FILTER == dict(W.CFG0_FILTER) == DTS_FILTER
    assert M.DTS_OPT == DTS_OPT
    assert M.HFBS == HFBS and M.HFBS_GRID == HFBS_GRID


# ---- the oracle still reproduces its fixtures (CPU) --------------------------
def test_oracle_reproduces_golden_dts(oracle_mod):
    d = _load("dts_depth_sr_96x64.npz")
    o = oracle_mod.OracleDTS(96, 64)
    o.init_frame(1, d["rgba"], d["target"], d["confidence"])
    o.differential(DTS_FILTER["sigma_x"], DTS_FILTER["sigma_y"], DTS_FILTER["sigma_r"])
    o.integrate()
    for a, (lk, uk) in enumerate((("lx", "ux"), ("ly", "uy"))):
        l, u, _ = o.bounds(a, DTS_OPT["sigma_z"])
        assert np.array_equal(l, d[lk]) and np.array_equal(u, d[uk])
    o.optimize(DTS_OPT["num_iterations"], DTS_OPT["loss"], DTS_OPT["lambda_"],
               DTS_OPT["sigma_z"], DTS_OPT["step_size"])
    assert np.allclose(o.download(5), d["v"], rtol=0, atol=1e-12)


def test_oracle_reproduces_golden_hfbs(oracle_mod):
    d = _load("hfbs_colorization_96x64.npz")
    o = oracle_mod.OracleHFBS(96, 64, *HFBS_GRID)
    o.clear_all()
    o.init_frame(0, d["rgba"], d["target"], d["confidence"])
    o.set_params(**HFBS)
    assert o.optimize() == 0
    assert np.array_equal(o.grid("splat_sum"), d["count"])
    assert np.allclose(o.download(5), d["out"], rtol=0, atol=1e-12, equal_nan=True)
    gt, gc = o.backward(d["grad_out"].astype(np.float64))
    assert np.allclose(gt, d["grad_target"], rtol=0, atol=1e-12)
    assert np.allclose(gc, d["grad_confidence"], rtol=0, atol=1e-12)


def test_oracle_reproduces_golden_color(oracle_mod):
    d = _load("color_64x64.npz")
    assert np.array_equal(oracle_mod.color_convert(1, d["rgba"]), d["ycbcr"])
    assert np.array_equal(oracle_mod.color_convert(2, d["rgba"]), d["yyy"])


# ---- the CUDA path against the fixtures (GPU) --------------------------------
@pytest.mark.gpu
def test_gpu_matches_golden_dts(gpu_ready):
    D = gpu_ready
    d = _load("dts_depth_sr_96x64.npz")
    s = D.DomainTransformSolver(D.ImageDim(96, 64))
    s.ClearAll()
    s.InitFrame(D.COLOR_SPACE.YCbCr, d["rgba"], d["target"], d["confidence"])
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(**DTS_FILTER))
    s.IntegrateColorDifferentials()
    for a, (lk, uk) in enumerate((("lx", "ux"), ("ly", "uy"))):
        l, u = s.DebugBounds(a, DTS_OPT["sigma_z"])
        assert np.array_equal(l, d[lk]) and np.array_equal(u, d[uk])
    s.Optimize(D.DomainOptimizeParams(**DTS_OPT))
    v = s.Download(D.ImageType.OPTIMIZED_QUANTITY)
    assert np.abs(v - d["v"]).max() <= P.TOL_REL * P.target_range(d["target"])


@pytest.mark.gpu
def test_gpu_matches_golden_hfbs_and_its_adjoint(gpu_ready):
    D = gpu_ready
    d = _load("hfbs_colorization_96x64.npz")
    h = D.HFBS(D.ImageDim(96, 64), *HFBS_GRID)
    h.SetFilterParams(D.HFBSGridParams(**HFBS))
    h.ClearAll()
    h.EnableGrad(True, 0)
    h.InitFrame(D.COLOR_SPACE.RGB, d["rgba"], d["target"], d["confidence"])
    h.Optimize()
    assert np.array_equal(h.DebugGrid(0), d["count"].astype(np.float32))
    out = h.Download(D.ImageType.OPTIMIZED_QUANTITY)
    fin = np.isfinite(d["out"])
    assert np.array_equal(np.isfinite(out), fin)
    assert np.abs(out[fin] - d["out"][fin]).max() <= P.TOL_REL * P.target_range(d["target"])
    gt, gc = h.Backward(d["grad_out"])
    for a, r in ((gt, d["grad_target"]), (gc, d["grad_confidence"])):
        assert np.abs(a - r).max() <= 1e-4 * np.abs(r).max()


@pytest.mark.gpu
@pytest.mark.parametrize("cs,key", [(1, "ycbcr"), (2, "yyy")])
def test_gpu_matches_golden_color(gpu_ready, cs, key):
    from domain_transform_solver_gb300 import _lib
    d = _load("color_64x64.npz")
    px = np.ascontiguousarray(d["rgba"].reshape(-1, 4))
    out = np.empty_like(px)
    _lib.check(_lib.load().dtsgb_debug_color_convert(cs, px.ctypes.data, out.ctypes.data,
                                                     px.shape[0]))
    assert np.array_equal(out.reshape(d[key].shape), d[key])
