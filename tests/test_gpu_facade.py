"""The C++ facade (include/domain_transform_gb300.hpp) drives the library
exactly like the Python mirror: a C++ program written like the reference's
own tests is compiled against it and must reproduce the Python path bit for
bit."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def test_cpp_facade_matches_python(gpu_ready, oracle_mod, tmp_path):
    D = gpu_ready
    import parity as P
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(77, 200, 120, n_poly=10, stride=4)
    h, w = inst.target.shape
    # the calls through the Python mirror, checked against the FP64 oracle
    s = D.DomainTransformSolver(D.ImageDim(w, h))
    s.SetImageDim(D.ImageDim(w, h))
    s.ClearAll()
    s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, inst.confidence)
    fp = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.1)
    op = dict(num_iterations=10, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(**fp))
    s.IntegrateColorDifferentials()
    s.Optimize(D.DomainOptimizeParams(**op))
    py_dts = s.Download(D.ImageType.OPTIMIZED_QUANTITY)
    ov = {(a, 8.0): s.DebugBounds(a, 8.0) for a in (0, 1)}
    ref, _ = oracle_mod.dts_solve(inst.rgba, inst.target, inst.confidence, 1, fp, op,
                                  overrides=ov)
    assert np.abs(py_dts - ref).max() <= P.TOL_REL * P.target_range(inst.target)
    # the same calls from C++ through the facade header
    inst.rgba.tofile(tmp_path / "rgba.bin")
    inst.target.tofile(tmp_path / "target.bin")
    inst.confidence.tofile(tmp_path / "conf.bin")
    (tmp_path / "dims.txt").write_text(f"{w} {h}\n")
    exe = tmp_path / "facade_test"
    pkg = ROOT / "domain_transform_solver_gb300"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "facade_solver_test.cpp"), "-o", str(exe),
                    f"-L{pkg}", "-ldtsgb", f"-Wl,-rpath,{pkg}"], check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "facade ok" in r.stdout
    dts = np.fromfile(tmp_path / "dts.bin", np.float32).reshape(h, w)
    assert np.array_equal(dts, py_dts)
    color = np.fromfile(tmp_path / "color.bin", np.uint8).reshape(h, w, 4)
    assert np.array_equal(color, s.Download(D.ImageType.COLOR_IMAGE))
    f = D.DomainTransformFilter(D.ImageDim(w, h))
    f.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba)
    filt = f.Filter(D.DomainFilterParams(8, 8, 0.2), inst.target, 5)
    assert np.array_equal(np.fromfile(tmp_path / "filter.bin", np.float32).reshape(h, w),
                          filt)
    hb = D.HFBS(D.ImageDim(w, h), (w + 7) // 8 + 1, (h + 7) // 8 + 1, 17)
    hb.SetImageDim(D.ImageDim(w, h))
    hb.SetFilterParams(D.HFBSGridParams(sigma_l=16, optim_iter_max=20))
    hb.ClearAll()
    hb.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, inst.confidence)
    hb.Optimize()
    hf = np.fromfile(tmp_path / "hfbs.bin", np.float32).reshape(h, w)
    ref = hb.Download(D.ImageType.OPTIMIZED_QUANTITY)
    assert np.array_equal(np.isnan(hf), np.isnan(ref))
    assert np.array_equal(hf[~np.isnan(hf)], ref[~np.isnan(ref)])
    hb.EnableGrad(True, 0)
    hb.Optimize()
    gt, gc = hb.Backward(inst.target)
    assert np.array_equal(np.fromfile(tmp_path / "hfbs_gt.bin", np.float32).reshape(h, w), gt)
    assert np.array_equal(np.fromfile(tmp_path / "hfbs_gc.bin", np.float32).reshape(h, w), gc)
