"""CPU tests of the oracle: known-answer cases derived by hand from the
reference's algorithm, and agreement with an independent numpy restatement
(tests/refnumpy.py).  The reference ships no golden vectors for this path,
so these are what the oracle is checked against."""
import numpy as np
import pytest

import refnumpy as R


# ---- a1 colour conversion ---------------------------------------------------
def _all_triples(start, stop):
    idx = np.arange(start, stop, dtype=np.int64)
    r, g, b = idx >> 16, (idx >> 8) & 255, idx & 255
    return r, g, b


@pytest.mark.parametrize("cs", [1, 2])
def test_color_equals_exact_floor_off_integer_points(oracle_mod, cs):
    """Wherever the exact colour value is not an integer, any faithful double
    evaluation truncates to floor(N/den): checked for all 2^24 triples."""
    for start in range(0, 1 << 24, 1 << 22):
        r, g, b = _all_triples(start, start + (1 << 22))
        px = np.stack([r, g, b, np.full_like(r, 255)], 1).astype(np.uint8)
        out = oracle_mod.color_convert(cs, px).astype(np.int64)
        ny = 299 * r + 587 * g + 114 * b
        m = ny % 1000 != 0
        assert np.array_equal(out[m, 0], ny[m] // 1000)
        if cs == 1:
            ncb = 128_000_000 - 168736 * r - 331264 * g + 500000 * b
            ncr = 128_000_000 + 500000 * r - 418688 * g - 81312 * b
            m1 = ncb % 1_000_000 != 0
            m2 = ncr % 1_000_000 != 0
            assert np.array_equal(out[m1, 1], ncb[m1] // 1_000_000)
            assert np.array_equal(out[m2, 2], ncr[m2] // 1_000_000)
        else:
            assert np.array_equal(out[:, 1], out[:, 0])
            assert np.array_equal(out[:, 2], out[:, 0])
        assert np.array_equal(out[:, 3], np.full(len(r), 255))


@pytest.mark.parametrize("order", [1, 2])
def test_color_integer_points_match_exact_fma_evaluation(oracle_mod, order):
    rng = np.random.default_rng(7)
    grey = [(k, k, k) for k in range(256)]
    r, g, b = _all_triples(0, 1 << 24)
    ny = 299 * r + 587 * g + 114 * b
    ints = np.nonzero(ny % 1000 == 0)[0]
    pick = rng.choice(ints, 300, replace=False)
    trip = grey + [(int(r[i]), int(g[i]), int(b[i])) for i in pick]
    px = np.array([t + (9,) for t in trip], np.uint8)
    out = oracle_mod.color_convert(1, px, contract=order)
    for (rr, gg, bb), o in zip(trip, out):
        assert tuple(int(v) for v in o[:3]) == R.convert_pixel(rr, gg, bb, 1, order)
        assert o[3] == 9


def test_color_rgb_is_identity(oracle_mod):
    px = np.random.default_rng(1).integers(0, 256, (1000, 4)).astype(np.uint8)
    assert np.array_equal(oracle_mod.color_convert(0, px), px)


# ---- a4 window bounds: hand-derived known answers ---------------------------
def _const_guide(w, h, value=(0, 0, 0, 0)):
    return np.broadcast_to(np.array(value, np.uint8), (h, w, 4)).copy()


def test_bounds_constant_guide_known_answer(oracle_mod):
    """Constant all-zero guide: dH = 1 everywhere (the zero-boundary
    neighbour of x = 0 equals the pixel), ct(x) = x + 1 exactly, and the
    reference search gives, for sigma = 3 on a 20-wide row:
      lower = x-4 when x >= 4, else x-1 (nothing below ct(x)-3: border
      collapse); upper = x+3 when x+4 <= 19 (the first index beyond the
      window must exist inside the row), else x."""
    W, H, sigma = 20, 3, 3.0
    o = oracle_mod.OracleDTS(W, H)
    o.init_frame(0, _const_guide(W, H), np.zeros((H, W), np.float32))
    o.differential(8.0, 8.0, 0.2)
    o.integrate()
    l, u, m = o.bounds(0, sigma)
    exp_l = np.array([x - 4 if x >= 4 else x - 1 for x in range(W)])
    exp_u = np.array([x + 3 if x + 4 <= W - 1 else x for x in range(W)])
    assert np.array_equal(l[1], exp_l)
    assert np.array_equal(u[1], exp_u)
    # exact ties (D == sigma) are resolved as "not beyond" and have margin 0
    assert m.min() == 0.0


def test_bounds_y_limit_quirk(oracle_mod):
    """The Y search loop runs to the image width (filter.cuh:22): with W < H
    the upper bound of rows y >= W - 4 collapses to y."""
    W, H, sigma = 6, 12, 3.0
    o = oracle_mod.OracleDTS(W, H, ref_y_limit=True)
    o.init_frame(0, _const_guide(W, H), np.zeros((H, W), np.float32))
    o.differential(8.0, 8.0, 0.2)
    o.integrate()
    l, u, _ = o.bounds(1, sigma)
    exp_u = np.array([y + 3 if y + 4 <= W - 1 else y for y in range(H)])
    assert np.array_equal(u[:, 2], exp_u)
    o2 = oracle_mod.OracleDTS(W, H, ref_y_limit=False)
    o2.init_frame(0, _const_guide(W, H), np.zeros((H, W), np.float32))
    o2.differential(8.0, 8.0, 0.2)
    o2.integrate()
    _, u2, _ = o2.bounds(1, sigma)
    exp_u2 = np.array([y + 3 if y + 4 <= H - 1 else y for y in range(H)])
    assert np.array_equal(u2[:, 2], exp_u2)


def test_filter_does_not_leak_across_a_step_edge(oracle_mod):
    W, H = 64, 16
    g = _const_guide(W, H, (10, 10, 10, 255))
    g[:, W // 2:, :3] = 240
    t = np.zeros((H, W), np.float32)
    t[:, W // 2:] = 1.0
    o = oracle_mod.OracleDTS(W, H)
    o.init_frame(0, g)
    out = o.filter(8.0, 8.0, 0.2, t, 3)
    assert np.array_equal(out, t.astype(np.float64))


def test_filter_linear_ramp_constant_guide(oracle_mod):
    """Box mean of a linear ramp over (l, u] is the window midpoint."""
    W, H = 30, 2
    o = oracle_mod.OracleDTS(W, H)
    o.init_frame(0, _const_guide(W, H))
    ramp = np.tile(np.arange(W, dtype=np.float32), (H, 1))
    o.differential(1.0, 1.0, 0.2)
    o.integrate()
    l, u, _ = o.bounds(0, 2.0)
    out = o.filter(2.0, 1e-3, 0.2, ramp, 1)  # Y window of one pixel
    mid = (l + 1 + u) / 2.0
    assert np.allclose(out, mid, atol=1e-12)


def test_dts_constant_target_is_a_fixed_point(oracle_mod, tmp_path):
    W, H = 40, 30
    rng = np.random.default_rng(3)
    g = rng.integers(0, 256, (H, W, 4)).astype(np.uint8)
    t = np.full((H, W), 5.0, np.float32)
    c = rng.random((H, W)).astype(np.float32)
    v, _ = oracle_mod.dts_solve(g, t, c, 1, dict(sigma_x=8, sigma_y=8, sigma_r=0.1),
                                dict(num_iterations=5, loss=1, lambda_=0.99,
                                     sigma_z=8.0, step_size=0.99))
    assert np.array_equal(v, np.full((H, W), 5.0))


def test_dts_l1_loss_returns_target(oracle_mod):
    W, H = 20, 10
    rng = np.random.default_rng(4)
    g = rng.integers(0, 256, (H, W, 4)).astype(np.uint8)
    t = rng.random((H, W)).astype(np.float32)
    v, _ = oracle_mod.dts_solve(g, t, None, 1, dict(sigma_x=8, sigma_y=8, sigma_r=0.1),
                                dict(num_iterations=5, loss=0, lambda_=0.99,
                                     sigma_z=8.0, step_size=0.99))
    assert np.array_equal(v, t.astype(np.float64))


def test_confidence_of_constant_target(oracle_mod):
    """DT(t^2) - DT(t)^2 = 0 -> conf = exp(0) = 1, except x <= left_clear."""
    W, H = 32, 12
    rng = np.random.default_rng(5)
    g = rng.integers(0, 256, (H, W, 4)).astype(np.uint8)
    o = oracle_mod.OracleDTS(W, H)
    o.init_frame(1, g, np.full((H, W), 3.0, np.float32))
    o.compute_confidence(8.0, 8.0, 0.2, 16.0, 4)
    conf = o.download(4)
    assert np.array_equal(conf[:, :5], np.zeros((H, 5)))
    assert np.array_equal(conf[:, 5:], np.ones((H, W - 5)))


# ---- agreement with the independent numpy restatement -----------------------
CASES = [(37, 23, 3.5, 1), (23, 41, 8.0, 1), (64, 20, 8.0, 2), (9, 30, 30.0, 1)]


@pytest.mark.parametrize("W,H,sz,loss", CASES)
@pytest.mark.parametrize("ref_y", [True, False])
def test_oracle_matches_numpy_dts(oracle_mod, W, H, sz, loss, ref_y):
    rng = np.random.default_rng(W * 100 + H)
    g = rng.integers(0, 256, (H, W, 4)).astype(np.uint8)
    g[..., 3] = 255
    t = rng.uniform(0, 10, (H, W)).astype(np.float32)
    c = (rng.random((H, W)) < 0.3).astype(np.float32)
    filt = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.1)
    opt = dict(num_iterations=4, loss=loss, lambda_=0.99, sigma_z=sz, step_size=0.99)
    v, o = oracle_mod.dts_solve(g, t, c, 1, filt, opt, ref_y_limit=ref_y)
    conv = o.download(0)
    v2 = R.dts_solve(conv, t, c, filt, opt, ref_y_limit=ref_y)
    assert np.allclose(v, v2, rtol=0, atol=1e-9)


@pytest.mark.parametrize("W,H", [(33, 17), (12, 40)])
def test_oracle_matches_numpy_filter(oracle_mod, W, H):
    rng = np.random.default_rng(W + H)
    g = rng.integers(0, 256, (H, W, 4)).astype(np.uint8)
    inp = rng.normal(0, 1, (H, W)).astype(np.float32)
    o = oracle_mod.OracleDTS(W, H)
    o.init_frame(2, g)
    out = o.filter(6.0, 5.0, 0.3, inp, 3)
    out2 = R.dt_filter(o.download(0), inp, 6.0, 5.0, 0.3, 3)
    assert np.allclose(out, out2, rtol=0, atol=1e-9)


HFBS_CASES = [
    # (W, H, sigma_l, max_grid) -- covered / uncovered pads, luma overflow
    (40, 24, 32.0, (64, 64, 64)),
    (70, 30, 40.0, (64, 64, 64)),
    (64, 64, 16.0, (8, 8, 16)),
    (50, 20, 15.0, (64, 64, 64)),
    (50, 20, 15.0, (64, 64, 17)),
]


@pytest.mark.parametrize("W,H,sl,mg", HFBS_CASES)
def test_oracle_matches_numpy_hfbs(oracle_mod, W, H, sl, mg):
    rng = np.random.default_rng(W * H)
    g = rng.integers(0, 256, (H, W, 4)).astype(np.uint8)
    g[..., 3] = 255
    g[0, 0, 0] = 255  # exercise the luma-overflow bin when sigma_l divides 255
    t = rng.uniform(-0.5, 0.5, (H, W)).astype(np.float32)
    c = (rng.random((H, W)) < 0.4).astype(np.float32)
    p = dict(sigma_x=8.0, sigma_y=8.0, sigma_l=sl, lambda_=8.0, alpha=1.0, beta=0.9,
             bistoch_iter_max=7, optim_iter_max=9, neg_exp_beta=0.9)
    out, o, st = oracle_mod.hfbs_solve(g, t, c, 0, p, max_grid=mg)
    assert st == 0
    out2, info = R.hfbs_solve(g, t, c, p, mg)
    assert info is not None
    assert np.array_equal(o.grid("splat_sum"), info["count"])
    assert np.allclose(o.grid("splat_norm"), info["norm"], atol=1e-12)
    assert np.allclose(o.grid("z_final"), info["z"], atol=1e-9)
    assert np.allclose(out, out2, atol=1e-9, equal_nan=True)


def test_hfbs_grid_too_large_copies_target(oracle_mod):
    W, H = 64, 32
    rng = np.random.default_rng(2)
    g = rng.integers(0, 256, (H, W, 4)).astype(np.uint8)
    t = rng.random((H, W)).astype(np.float32)
    out, o, st = oracle_mod.hfbs_solve(g, t, None, 0, dict(sigma_x=8.0, sigma_y=8.0,
                                                           sigma_l=16.0),
                                       max_grid=(4, 4, 16))
    assert st == 1
    assert np.array_equal(out, t.astype(np.float64))


def test_f32_baseline_close_to_f64(oracle_mod):
    from domain_transform_solver_gb300 import workloads as WL
    inst = WL.depth_sr_instance(11, 96, 64)
    kw = dict(num_iterations=5, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    filt = WL.CFG0_FILTER
    v64, _ = oracle_mod.dts_solve(inst.rgba, inst.target, inst.confidence, 1, filt, kw)
    v32, _ = oracle_mod.dts_solve(inst.rgba, inst.target, inst.confidence, 1, filt, kw,
                                  real="f32")
    assert np.sqrt(np.mean((v64 - v32) ** 2)) < 1e-3 * np.ptp(inst.target)


# ---- DomainTransformStereo: photometric term --------------------------------
@pytest.mark.parametrize("loss", [1, 2])
def test_oracle_stereo_matches_numpy(oracle_mod, loss):
    W_, H_ = 40, 18
    rng = np.random.default_rng(31 + loss)
    left = rng.integers(0, 256, (H_, W_, 4)).astype(np.uint8)
    right = np.roll(left, -3, axis=1)
    right[..., :3] = np.clip(right[..., :3].astype(int) + rng.integers(-4, 5, right[..., :3].shape),
                             0, 255).astype(np.uint8)
    # disparities near half-integers so (int)(offset + x - d) is far from a tie
    t = (rng.integers(1, 8, (H_, W_)) + 0.5 + rng.uniform(-0.1, 0.1, (H_, W_))).astype(np.float32)
    c = (rng.random((H_, W_)) < 0.5).astype(np.float32)
    filt = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.2)
    opt = dict(num_iterations=3, loss=loss, lambda_=0.99, sigma_z=6.0, step_size=0.9)
    o = oracle_mod.OracleDTS(W_, H_)
    o.init_frame(1, left, t, c)
    o.init_right_frame(2.0, 1, right)
    o.differential(8.0, 8.0, 0.2)
    o.integrate()
    o.process_right_frame()
    o.optimize_stereo(3, loss, 0.99, 6.0, 0.9, 0.01)
    v = o.download(5)
    ref = R.dts_solve(o.download(0), t, c, filt, opt,
                      stereo=(oracle_mod.color_convert(1, right), 2.0, 0.01))
    assert np.allclose(v, ref, rtol=0, atol=1e-9)
    # the term is active: without it the result differs
    o2 = oracle_mod.OracleDTS(W_, H_)
    o2.init_frame(1, left, t, c)
    o2.differential(8.0, 8.0, 0.2)
    o2.integrate()
    o2.optimize(3, loss, 0.99, 6.0, 0.9)
    assert np.abs(o2.download(5) - v).max() > 1e-3


# ---- adjoint of the fixed-iteration solve ------------------------------------
@pytest.mark.parametrize("loss", [1, 2])
def test_oracle_adjoint_matches_central_differences(oracle_mod, loss):
    """dL/dt and dL/dc of L = <gout, v_N> against FP64 central differences of
    the forward solve with the same (fixed) windows."""
    W_, H_ = 24, 16
    rng = np.random.default_rng(5 + loss)
    g = rng.integers(0, 256, (H_, W_, 4)).astype(np.uint8)
    t = rng.uniform(0, 5, (H_, W_)).astype(np.float32)
    c = rng.uniform(0.1, 1.0, (H_, W_)).astype(np.float32)
    gout = rng.normal(0, 1, (H_, W_))
    filt = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.2)
    iters, lam, sz, step = 4, 0.9, 5.0, 0.8
    o = oracle_mod.OracleDTS(W_, H_)
    o.init_frame(1, g, t, c)
    o.differential(8.0, 8.0, 0.2)
    o.integrate()
    gt, gc = o.backward(iters, loss, lam, sz, step, gout)

    def L(tt, cc):
        o2 = oracle_mod.OracleDTS(W_, H_)
        o2.init_frame(1, g, tt, cc)
        o2.differential(8.0, 8.0, 0.2)
        o2.integrate()
        o2.optimize(iters, loss, lam, sz, step)
        return float((o2.download(5) * gout).sum())

    # the forward takes float32 inputs: perturb by exactly representable steps
    picks = rng.choice(W_ * H_, 12, replace=False)
    for k in picks:
        y, x = divmod(int(k), W_)
        for arr, grad in ((t, gt), (c, gc)):
            h = np.float32(2.0 ** -8)
            a = arr.copy(); a[y, x] += h
            b = arr.copy(); b[y, x] -= h
            args_p = (a, c) if arr is t else (t, a)
            args_m = (b, c) if arr is t else (t, b)
            fd = (L(*args_p) - L(*args_m)) / (2 * float(h))
            assert abs(fd - grad[y, x]) <= 2e-3 * max(1.0, abs(fd)), (k, fd, grad[y, x])


# ---- HFBS adjoint --------------------------------------------------------------
def _hfbs_fd_case(oracle_mod, seed, scale, K, sl=32.0, mg=(16, 16, 16), W_=48, H_=40):
    rng = np.random.default_rng(seed)
    g = rng.integers(0, 256, (H_, W_, 4)).astype(np.uint8)
    g[..., 3] = 255
    g[0, :8, 0] = 255  # luma-overflow bin when sigma_l divides 255
    t = rng.uniform(-0.5, 0.5, (H_, W_)) * scale
    c = rng.uniform(0.1, 1.0, (H_, W_)) * (rng.random((H_, W_)) < 0.5)
    gout = rng.standard_normal((H_, W_))
    o = oracle_mod.OracleHFBS(W_, H_, *mg)
    o.clear_all()
    o.init_frame(0, g, t.astype(np.float32), c.astype(np.float32))
    o.set_params(sigma_x=8.0, sigma_y=8.0, sigma_l=sl, lambda_=8.0, alpha=1.0, beta=0.9,
                 bistoch_iter_max=5, optim_iter_max=K, neg_exp_beta=0.9)

    def loss(tt, cc):
        o.set_target_conf(tt, cc)
        assert o.optimize() == 0
        return float(np.sum(gout * o.download(5)))

    loss(t, c)
    gt, gc = o.backward(gout)
    return rng, t, c, loss, gt, gc, o, gout


@pytest.mark.parametrize("scale,K,sl,mg", [(1.0, 12, 32.0, (16, 16, 16)),
                                          (20.0, 20, 32.0, (16, 16, 16)),  # Huber clamp active
                                          (1.0, 9, 17.0, (8, 8, 32))])    # overflow bin stored
def test_oracle_hfbs_adjoint_matches_central_differences(oracle_mod, scale, K, sl, mg):
    """ora_hfbs_backward against FP64 central differences of ora_hfbs_optimize
    (bins, counts and normalisation do not move under these perturbations)."""
    rng, t, c, loss, gt, gc, _, _ = _hfbs_fd_case(oracle_mod, 5, scale, K, sl, mg)
    H_, W_ = t.shape
    h = 1e-6
    for _ in range(20):
        y, x = int(rng.integers(0, H_)), int(rng.integers(0, W_))
        for which, an in ((0, gt[y, x]), (1, gc[y, x])):
            a = (t if which == 0 else c).copy()
            a[y, x] += h
            lp = loss(a, c) if which == 0 else loss(t, a)
            a[y, x] -= 2 * h
            lm = loss(a, c) if which == 0 else loss(t, a)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - an) <= 1e-5 * max(1e-2, abs(fd)), (which, y, x, fd, an)


def test_oracle_hfbs_adjoint_is_linear_in_the_upstream_gradient(oracle_mod):
    """The adjoint is linear in dL/doutput: backward(2*g1 - g2) equals
    2*backward(g1) - backward(g2), and a zero upstream gradient gives zero."""
    rng, t, c, loss, gt1, gc1, o, g1 = _hfbs_fd_case(oracle_mod, 7, 1.0, 10)
    g2 = rng.standard_normal(g1.shape)
    gt2, gc2 = o.backward(g2)
    gt3, gc3 = o.backward(2 * g1 - g2)
    assert np.allclose(gt3, 2 * gt1 - gt2, rtol=0, atol=1e-12)
    assert np.allclose(gc3, 2 * gc1 - gc2, rtol=0, atol=1e-12)
    gt0, gc0 = o.backward(np.zeros_like(g1))
    assert not gt0.any() and not gc0.any()
    assert np.abs(gt1).max() > 0 and np.abs(gc1).max() > 0
