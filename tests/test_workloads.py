import numpy as np

from domain_transform_solver_gb300 import workloads as W


def test_cfg0_shapes_and_ranges():
    a = W.depth_sr_instance(W.SEED_BASE)
    b = W.depth_sr_instance(W.SEED_BASE)
    assert a.rgba.shape == (480, 640, 4) and a.rgba.dtype == np.uint8
    assert np.array_equal(a.rgba, b.rgba) and np.array_equal(a.target, b.target)
    assert (a.rgba[..., 3] == 255).all()
    s = a.confidence > 0
    assert s.sum() == 80 * 60
    assert a.target[s].min() > 0.4 and a.target[s].max() < 10.1
    assert (a.target[~s] == 0).all()


def test_cfg1_and_cfg2():
    u, v = W.colorization_instance()
    assert u.rgba.shape == (480, 640, 4)
    assert (u.rgba[..., 0] == u.rgba[..., 1]).all()
    frac = (u.confidence > 0).mean()
    assert 0.015 < frac < 0.025
    assert np.abs(u.target).max() <= 0.5 and np.abs(v).max() <= 0.5
    s = W.stereo_instance()
    assert s.target.shape == (384, 1280)
    assert 0 <= s.confidence.min() and s.confidence.max() <= 1


def test_cfg3_sizes():
    sizes = W.batched_sizes()
    assert len(sizes) == 64
    assert all(256 <= w <= 1920 and 256 <= h <= 1080 for w, h in sizes)
    assert any(w < h for w, h in sizes)
