"""Adjoint of the fixed-window DTS solve on the GPU (dtsgb_batch_dts_backward)
against the FP64 oracle: its adjoint (oracle.c ora_dts_backward) and central
finite differences of its forward, both evaluated on the windows the GPU
chose.  Checkpoint segment lengths give bitwise-identical gradients, and the
torch.autograd binding returns what the C ABI returns."""
import numpy as np
import pytest

import parity as P

pytestmark = pytest.mark.gpu

SIZES = [(96, 64), (71, 83)]
FILT = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.1)
# relative to max |gradient| of the FP64 oracle
TOL_GRAD = 1e-4


# Charbonnier's data-term slope is 0.5*(c/n)/sqrt(1e-6) = 500 c/n at the
# target: with c ~ 1 a step of 0.99 overshoots there and the iteration is not
# contractive, so FP32 and FP64 trajectories part ways and neither the adjoint
# comparison nor finite differences mean anything at such pixels.  Charbonnier
# cases therefore use confidences below 0.001 (0.99 * 500 * 0.001 / n < 1
# for every window size n >= 1).
CMAX = {1: 1.0, 2: 0.001}


def _inputs(seed, sizes=SIZES, cmax=1.0):
    from domain_transform_solver_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    out = []
    for i, (w, h) in enumerate(sizes):
        inst = W.depth_sr_instance(seed + i, w, h, n_poly=6, sample_frac=0.2)
        c = (cmax * rng.random((h, w))).astype(np.float32)  # graded confidence
        g = rng.standard_normal((h, w)).astype(np.float32)  # upstream dL/dv
        out.append((inst.rgba, inst.target, c, g))
    return out


def _batch(D, data, opt, segment=0, flags=0, graphs=True):
    b = D.Batch([(t.shape[1], t.shape[0]) for _, t, _, _ in data], flags=flags,
                use_graphs=graphs)
    b.enable_grad(True, segment)
    b.upload(D.COLOR_SPACE.YCbCr, [r for r, _, _, _ in data], [t for _, t, _, _ in data],
             [c for _, _, c, _ in data])
    b.solve_dts(D.DomainFilterParams(**FILT), D.DomainOptimizeParams(**opt))
    return b


def _gpu_windows(D, rgba, t, c, sigma_z, flags=0):
    h, w = t.shape
    s = D.DomainTransformSolver(D.ImageDim(w, h), flags=flags)
    s.InitFrame(D.COLOR_SPACE.YCbCr, rgba, t, c)
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(**FILT))
    s.IntegrateColorDifferentials()
    return {(a, sigma_z): s.DebugBounds(a, sigma_z) for a in (0, 1)}


def _oracle(O, rgba, t, c, windows):
    h, w = t.shape
    o = O.OracleDTS(w, h)
    o.init_frame(1, rgba)
    o.set_target_conf(t, c)  # FP64, so that FD perturbations survive
    o.differential(FILT["sigma_x"], FILT["sigma_y"], FILT["sigma_r"])
    o.integrate()
    for (axis, sg), (l, u) in windows.items():
        o.add_bounds_override(axis, sg, l, u)
    return o


def _oracle_loss(O, rgba, t, c, g, windows, opt):
    o = _oracle(O, rgba, t, c, windows)
    o.optimize(opt["num_iterations"], opt["loss"], opt["lambda_"], opt["sigma_z"],
               opt["step_size"])
    return float(np.sum(g.astype(np.float64) * o.download(5)))


@pytest.mark.parametrize("loss", [1, 2])
def test_adjoint_matches_oracle_adjoint(gpu_ready, oracle_mod, loss):
    D = gpu_ready
    data = _inputs(900 + loss, cmax=CMAX[loss])
    opt = dict(num_iterations=5, loss=loss, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    b = _batch(D, data, opt)
    gts, gcs = b.backward([g for _, _, _, g in data])
    for (rgba, t, c, g), gt, gc in zip(data, gts, gcs):
        win = _gpu_windows(D, rgba, t, c, opt["sigma_z"])
        o = _oracle(oracle_mod, rgba, t, c, win)
        rt, rc = o.backward(opt["num_iterations"], loss, opt["lambda_"], opt["sigma_z"],
                            opt["step_size"], g)
        _check_grad(gt, rt, loss)
        _check_grad(gc, rc, loss)


def _check_grad(got, ref, loss):
    """L2 is linear in the iterate: max-abs bar.  Charbonnier's h' and dh/dc
    change ~1000-fold faster than the residual v - t near v = t, so a pixel
    whose FP32 iterate sits within ~1e-3 of its target can move by more than
    the bar: RMSE bar plus 99.5% of pixels under the max-abs bar."""
    err = np.abs(got - ref)
    bar = TOL_GRAD * np.abs(ref).max()
    if loss == 1:
        assert err.max() <= bar
    else:
        assert float(np.sqrt(np.mean(err ** 2))) <= bar
        assert float(np.mean(err <= bar)) >= 0.995


@pytest.mark.parametrize("loss", [1, 2])
def test_adjoint_matches_fp64_central_differences(gpu_ready, oracle_mod, loss):
    """256 random entries (128 of the target, 128 of the confidence) of one
    instance: d/de sum(g * v) by central differences of the FP64 oracle."""
    D = gpu_ready
    data = _inputs(950 + loss, sizes=[(64, 48)], cmax=CMAX[loss])
    rgba, t, c, g = data[0]
    opt = dict(num_iterations=10, loss=loss, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    b = _batch(D, data, opt, segment=4)
    (gt,), (gc,) = b.backward([g])
    win = _gpu_windows(D, rgba, t, c, opt["sigma_z"])
    rng = np.random.default_rng(7)
    idx = rng.choice(t.size, 256, replace=False)
    scale_t = max(float(np.abs(t).max()), 1.0)
    bars = {"t": 2e-4 * max(np.abs(gt).max(), 1e-3), "c": 2e-4 * max(np.abs(gc).max(), 1e-3)}
    bad = []
    for k, flat in enumerate(idx):
        which = "t" if k < 128 else "c"
        base = t if which == "t" else c
        h = 1e-6 * (scale_t if which == "t" else 1.0)
        plus = base.astype(np.float64).copy()
        minus = plus.copy()
        plus.flat[flat] += h
        minus.flat[flat] -= h
        if which == "t":
            lp = _oracle_loss(oracle_mod, rgba, plus, c, g, win, opt)
            lm = _oracle_loss(oracle_mod, rgba, minus, c, g, win, opt)
            got = gt.flat[flat]
        else:
            lp = _oracle_loss(oracle_mod, rgba, t, plus, g, win, opt)
            lm = _oracle_loss(oracle_mod, rgba, t, minus, g, win, opt)
            got = gc.flat[flat]
        fd = (lp - lm) / (2 * h)
        if abs(got - fd) > bars[which]:
            bad.append((which, int(flat), float(got), fd))
    # Charbonnier: see _check_grad; at most 1% of the entries may sit at a
    # near-zero residual
    assert len(bad) <= (0 if loss == 1 else 2), bad


def test_checkpoint_segments_agree_bitwise(gpu_ready):
    D = gpu_ready
    data = _inputs(980)
    opt = dict(num_iterations=7, loss=2, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    go = [g for _, _, _, g in data]
    results = []
    for seg, graphs in ((1, True), (2, True), (3, False), (0, True), (7, True)):
        b = _batch(D, data, opt, segment=seg, graphs=graphs)
        results.append(b.backward(go))
        seg_used, planes = b.grad_info()
        # automatic: every iterate kept (these few planes fit any free memory)
        want = seg if seg else 1
        assert seg_used == want
        assert planes == -(-7 // want) - 1 + want + 4
        # the forward result is the plain solve's
        plain = D.Batch([(t.shape[1], t.shape[0]) for _, t, _, _ in data])
        plain.upload(D.COLOR_SPACE.YCbCr, [r for r, _, _, _ in data],
                     [t for _, t, _, _ in data], [c for _, _, c, _ in data])
        plain.solve_dts(D.DomainFilterParams(**FILT), D.DomainOptimizeParams(**opt))
        for v, w in zip(b.download(0), plain.download(0)):
            assert np.array_equal(v, w)
    for gts, gcs in results[1:]:
        for a, r in zip(gts + gcs, results[0][0] + results[0][1]):
            assert np.array_equal(a, r)


def test_memory_does_not_grow_with_iterations(gpu_ready):
    """Checkpoint segments of about sqrt(N) hold ceil(N/K) - 1 + K + 4 planes;
    the automatic choice keeps every iterate when that fits in free memory."""
    D = gpu_ready
    data = _inputs(990, sizes=[(40, 30)])
    for n, seg in ((16, 4), (100, 10)):
        opt = dict(num_iterations=n, loss=1, lambda_=0.99, sigma_z=4.0, step_size=0.99)
        b = _batch(D, data, opt, segment=seg)
        assert b.grad_info() == (seg, -(-n // seg) - 1 + seg + 4)
        b = _batch(D, data, opt)
        assert b.grad_info() == (1, n + 4)


def test_l1_and_zero_iterations_pass_the_gradient_to_the_target(gpu_ready):
    D = gpu_ready
    data = _inputs(995)
    go = [g for _, _, _, g in data]
    for opt in (dict(num_iterations=5, loss=0), dict(num_iterations=0, loss=1)):
        b = _batch(D, data, dict(opt, lambda_=0.99, sigma_z=8.0, step_size=0.99))
        gts, gcs = b.backward(go)
        for g, gt, gc in zip(go, gts, gcs):
            assert np.array_equal(gt, g)
            assert not gc.any()


def test_backward_needs_a_gradient_solve(gpu_ready):
    D = gpu_ready
    data = _inputs(996)
    b = D.Batch([(t.shape[1], t.shape[0]) for _, t, _, _ in data])
    b.upload(D.COLOR_SPACE.YCbCr, [r for r, _, _, _ in data], [t for _, t, _, _ in data])
    opt = D.DomainOptimizeParams(num_iterations=3, loss=1, lambda_=0.99, sigma_z=8.0,
                                 step_size=0.99)
    b.solve_dts(D.DomainFilterParams(**FILT), opt)
    with pytest.raises(D.DtsgbError):
        b.backward([g for _, _, _, g in data])
    b.enable_grad(True, 0)
    with pytest.raises(D.DtsgbError):  # the confidence overwrite has no adjoint
        b.solve_dts(D.DomainFilterParams(**FILT), opt, 0.5)
    b.solve_dts(D.DomainFilterParams(**FILT), opt)
    b.backward([g for _, _, _, g in data])
    b.upload(D.COLOR_SPACE.YCbCr, [r for r, _, _, _ in data], [t for _, t, _, _ in data])
    with pytest.raises(D.DtsgbError):  # new inputs invalidate the checkpoints
        b.backward([g for _, _, _, g in data])


def test_bf16_storage_adjoint_on_rounded_inputs(gpu_ready, oracle_mod):
    D = gpu_ready
    data = _inputs(997, sizes=[(96, 64)], cmax=CMAX[2])
    opt = dict(num_iterations=4, loss=2, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    b = _batch(D, data, opt, flags=D.FLAG_BF16_STORAGE)
    (gt,), (gc,) = b.backward([data[0][3]])
    rgba, t, c, g = data[0]
    tb, cb = P.bf16_round(t), P.bf16_round(c)
    win = _gpu_windows(D, rgba, tb, cb, opt["sigma_z"])
    rt, rc = _oracle(oracle_mod, rgba, tb, cb, win).backward(
        opt["num_iterations"], 2, opt["lambda_"], opt["sigma_z"], opt["step_size"], g)
    _check_grad(gt, rt, 2)
    _check_grad(gc, rc, 2)


def test_torch_autograd_binding(gpu_ready):
    D = gpu_ready
    torch = pytest.importorskip("torch")
    from domain_transform_solver_gb300.autograd import dts_solve
    data = _inputs(998, sizes=[(80, 60)] * 3)
    opt = dict(num_iterations=6, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    dev = torch.device("cuda:0")
    rgba = torch.from_numpy(np.stack([r for r, _, _, _ in data])).to(dev)
    t = torch.from_numpy(np.stack([t for _, t, _, _ in data])).to(dev).requires_grad_()
    c = torch.from_numpy(np.stack([c for _, _, c, _ in data])).to(dev).requires_grad_()
    g = torch.from_numpy(np.stack([g for _, _, _, g in data])).to(dev)
    v = dts_solve(rgba, t, c, D.DomainFilterParams(**FILT), D.DomainOptimizeParams(**opt),
                  segment=2)
    (v * g).sum().backward()
    b = _batch(D, data, opt, segment=2)
    gts, gcs = b.backward([x for _, _, _, x in data])
    for i in range(3):
        assert np.array_equal(v[i].detach().cpu().numpy(), b.download(0)[i])
        assert np.array_equal(t.grad[i].cpu().numpy(), gts[i])
        assert np.array_equal(c.grad[i].cpu().numpy(), gcs[i])


def test_pipeline_run_grad_matches_batch(gpu_ready):
    """dtsgb_pipeline_run_grad (chunks on their own streams) gives the batch's
    results and gradients bitwise."""
    D = gpu_ready
    data = _inputs(1010)
    opt = dict(num_iterations=6, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    go = [g for _, _, _, g in data]
    b = _batch(D, data, opt)
    ref_v = b.download(0)
    ref_gt, ref_gc = b.backward(go)
    sizes = [(t.shape[1], t.shape[0]) for _, t, _, _ in data]
    p = D.Pipeline(sizes, n_chunks=2)
    for _ in range(2):
        v, gt, gc = p.run_grad(D.COLOR_SPACE.YCbCr, [r for r, _, _, _ in data],
                               [t for _, t, _, _ in data], [c for _, _, c, _ in data],
                               D.DomainFilterParams(**FILT), D.DomainOptimizeParams(**opt), go)
        for a, r in zip(v + gt + gc, ref_v + ref_gt + ref_gc):
            assert np.array_equal(a, r)
    p.close()
