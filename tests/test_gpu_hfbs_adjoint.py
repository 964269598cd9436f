"""Adjoint of the HFBS solve on the GPU (dtsgb_hfbs_backward) against the
FP64 oracle: its adjoint (oracle.c ora_hfbs_backward) and central finite
differences of its forward.  Checkpoint segment lengths give
bitwise-identical gradients, and the torch.autograd binding returns what the
C ABI returns."""
import numpy as np
import pytest

import parity as P

pytestmark = pytest.mark.gpu

BASE = dict(sigma_x=8.0, sigma_y=8.0, sigma_l=16.0, lambda_=8.0, alpha=1.0, beta=0.9,
            bistoch_iter_max=20, optim_iter_max=64, neg_exp_beta=0.9)
# relative to max |gradient| of the FP64 oracle
TOL_GRAD = 1e-4


def _inputs(seed, w, h, conf="sparse", scale=1.0):
    rng = np.random.default_rng(seed)
    g = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    g[..., 3] = 255
    g[0, : min(8, w), 0] = 255  # the top luma value: the overflow bin when sigma_l divides 255
    t = (rng.uniform(-0.5, 0.5, (h, w)) * scale).astype(np.float32)
    if conf == "sparse":  # colorization-style: confidence 1 at 5% of pixels
        c = (rng.random((h, w)) < 0.05).astype(np.float32)
    elif conf == "graded":
        c = rng.uniform(0.0, 1.0, (h, w)).astype(np.float32)
    else:
        c = None
    gout = rng.standard_normal((h, w)).astype(np.float32)
    return g, t, c, gout


def _gpu(D, g, t, c, params, mg, gout, segment=0):
    h, w = t.shape
    s = D.HFBS(D.ImageDim(w, h), *mg)
    s.SetFilterParams(D.HFBSGridParams(**params))
    s.ClearAll()
    s.EnableGrad(True, segment)
    s.InitFrame(D.COLOR_SPACE.RGB, g, t, c)
    s.Optimize()
    out = s.Download(D.ImageType.OPTIMIZED_QUANTITY)
    gt, gc = s.Backward(gout)
    return out, gt, gc, s


def _oracle(O, g, t, c, params, mg, gout):
    h, w = t.shape
    o = O.OracleHFBS(w, h, *mg)
    o.clear_all()
    o.init_frame(0, g, t, c)
    o.set_params(**params)
    assert o.optimize() == 0
    out = o.download(5)
    gt, gc = o.backward(gout.astype(np.float64))
    return out, gt, gc, o


def _close(a, r, tol=TOL_GRAD):
    scale = max(1e-12, float(np.abs(r).max()))
    err = float(np.abs(a - r).max())
    assert err <= tol * scale, (err, scale)


CASES = [
    # (w, h, params, max grid, confidence)
    (96, 80, dict(BASE), (12, 10, 16), "sparse"),             # colorization-style, 64 steps
    (71, 53, dict(BASE, sigma_l=17.0, optim_iter_max=20), (9, 7, 32), "graded"),  # overflow bin stored
    (64, 48, dict(BASE, sigma_l=32.0, optim_iter_max=12), (8, 6, 8), None),  # default confidence
    (40, 24, dict(BASE, optim_iter_max=0), (5, 3, 16), "graded"),  # no heavy-ball step
    # 32 luma levels: the one-step heavy-ball kernel (FMA neighbour sums)
    (64, 40, dict(BASE, sigma_l=8.0, optim_iter_max=16), (8, 5, 40), "graded"),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_hfbs_adjoint_matches_oracle_adjoint(gpu_ready, oracle_mod, case):
    w, h, params, mg, conf = CASES[case]
    g, t, c, gout = _inputs(10 + case, w, h, conf)
    out, gt, gc, _ = _gpu(gpu_ready, g, t, c, params, mg, gout)
    ref, rt, rc, _ = _oracle(oracle_mod, g, t, c, params, mg, gout)
    fin = np.isfinite(ref)
    assert np.abs(out[fin] - ref[fin]).max() <= P.TOL_REL * P.target_range(t)
    _close(gt, rt)
    _close(gc, rc)


def test_hfbs_adjoint_with_the_huber_clamp_active(gpu_ready, oracle_mod):
    """Targets of +-10 put |grad| above 1.345 in the first steps.  Where a
    gradient passes within rounding of the threshold FP32 and FP64 take
    different branches; the comparison is held to RMSE <= 1e-4 x max|grad|
    and 99% of pixels within 1e-4 x max|grad|."""
    params = dict(BASE, optim_iter_max=20)
    g, t, c, gout = _inputs(21, 80, 64, "graded", scale=20.0)
    _, gt, gc, _ = _gpu(gpu_ready, g, t, c, params, (10, 8, 16), gout)
    _, rt, rc, o = _oracle(oracle_mod, g, t, c, params, (10, 8, 16), gout)
    for a, r in ((gt, rt), (gc, rc)):
        scale = float(np.abs(r).max())
        err = np.abs(a - r)
        assert float(np.sqrt(np.mean(err ** 2))) <= TOL_GRAD * scale
        assert float(np.mean(err <= TOL_GRAD * scale)) >= 0.99


def test_hfbs_adjoint_matches_fp64_central_differences(gpu_ready, oracle_mod):
    """dL/dtarget and dL/dconfidence of L = sum(gout * out) from the GPU
    against FP64 central differences of the oracle's forward on 64 random
    entries (h = 1e-6)."""
    w, h, params, mg = 64, 48, dict(BASE, optim_iter_max=24), (8, 6, 16)
    g, t, c, gout = _inputs(31, w, h, "graded")
    _, gt, gc, _ = _gpu(gpu_ready, g, t, c, params, mg, gout)
    o = oracle_mod.OracleHFBS(w, h, *mg)
    o.clear_all()
    o.init_frame(0, g, t, c)
    o.set_params(**params)
    t64, c64, go = t.astype(np.float64), c.astype(np.float64), gout.astype(np.float64)

    def loss(tt, cc):
        o.set_target_conf(tt, cc)
        assert o.optimize() == 0
        return float(np.sum(go * o.download(5)))

    rng = np.random.default_rng(3)
    fd_t, fd_c, an_t, an_c = [], [], [], []
    for _ in range(32):
        y, x = int(rng.integers(0, h)), int(rng.integers(0, w))
        for which in (0, 1):
            a = (t64 if which == 0 else c64).copy()
            a[y, x] += 1e-6
            lp = loss(a, c64) if which == 0 else loss(t64, a)
            a[y, x] -= 2e-6
            lm = loss(a, c64) if which == 0 else loss(t64, a)
            (fd_t if which == 0 else fd_c).append((lp - lm) / 2e-6)
            (an_t if which == 0 else an_c).append((gt if which == 0 else gc)[y, x])
    for fd, an, full in ((fd_t, an_t, gt), (fd_c, an_c, gc)):
        fd, an = np.array(fd), np.array(an)
        assert np.abs(fd - an).max() <= 1e-3 * float(np.abs(full).max()), (fd, an)


def test_hfbs_checkpoint_segments_agree_bitwise(gpu_ready):
    """Every iterate kept (segment 1) and segments recomputed from (z, h)
    checkpoints give the same gradients bit for bit, and the forward result
    of a differentiable solve is the plain solve's."""
    D = gpu_ready
    params = dict(BASE, optim_iter_max=30)
    g, t, c, gout = _inputs(41, 96, 64, "graded")
    res = [_gpu(D, g, t, c, params, (12, 8, 16), gout, segment=s) for s in (1, 4, 7, 30, 64)]
    for out, gt, gc, s in res[1:]:
        assert np.array_equal(out, res[0][0])
        assert np.array_equal(gt, res[0][1])
        assert np.array_equal(gc, res[0][2])
    # 8 adjoint grids, (z, h) at 8 checkpoints, 3 segment planes, 2 for h
    assert res[1][3].GradInfo() == (4, 8 + 2 * 8 + 3 + 2)
    plain = D.HFBS(D.ImageDim(96, 64), 12, 8, 16)
    plain.SetFilterParams(D.HFBSGridParams(**params))
    plain.ClearAll()
    plain.InitFrame(D.COLOR_SPACE.RGB, g, t, c)
    plain.Optimize()
    ref = plain.Download(D.ImageType.OPTIMIZED_QUANTITY)
    assert np.array_equal(res[0][0], ref)  # the same heavy-ball kernel


def test_hfbs_one_step_path_segments_agree_bitwise(gpu_ready):
    """Grids of more than 16 levels run one heavy-ball step per launch (h in
    place); checkpointed segments recompute with the same kernel."""
    D = gpu_ready
    params = dict(BASE, sigma_l=8.0, optim_iter_max=13)
    g, t, c, gout = _inputs(45, 64, 40, "graded")
    res = [_gpu(D, g, t, c, params, (8, 5, 40), gout, segment=s) for s in (1, 3, 5)]
    for out, gt, gc, _ in res[1:]:
        assert np.array_equal(out, res[0][0])
        assert np.array_equal(gt, res[0][1])
        assert np.array_equal(gc, res[0][2])
    plain = D.HFBS(D.ImageDim(64, 40), 8, 5, 40)
    plain.SetFilterParams(D.HFBSGridParams(**params))
    plain.ClearAll()
    plain.InitFrame(D.COLOR_SPACE.RGB, g, t, c)
    plain.Optimize()
    assert np.array_equal(res[0][0], plain.Download(D.ImageType.OPTIMIZED_QUANTITY))


def test_hfbs_automatic_segment_keeps_every_iterate(gpu_ready):
    D = gpu_ready
    g, t, c, gout = _inputs(51, 64, 48, "sparse")
    _, _, _, s = _gpu(D, g, t, c, dict(BASE, optim_iter_max=40), (8, 6, 16), gout)
    assert s.GradInfo() == (1, 8 + 40)  # 8 adjoint grids, every iterate


def test_hfbs_backward_needs_a_gradient_solve(gpu_ready):
    D = gpu_ready
    g, t, c, gout = _inputs(61, 48, 32, "graded")
    s = D.HFBS(D.ImageDim(48, 32), 6, 4, 16)
    s.SetFilterParams(D.HFBSGridParams(**dict(BASE, optim_iter_max=8)))
    s.InitFrame(D.COLOR_SPACE.RGB, g, t, c)
    s.Optimize()
    with pytest.raises(D.DtsgbError):
        s.Backward(gout)
    s.EnableGrad(True)
    s.Optimize()
    s.Backward(gout)  # fine now
    s.InitFrame(D.COLOR_SPACE.RGB, g, t, c)  # a new frame invalidates the solve
    with pytest.raises(D.DtsgbError):
        s.Backward(gout)


def test_hfbs_torch_autograd_binding(gpu_ready):
    torch = pytest.importorskip("torch")
    D = gpu_ready
    from domain_transform_solver_gb300 import autograd as A
    params = dict(BASE, optim_iter_max=16)
    data = [_inputs(71 + i, 64, 40, "graded") for i in range(2)]
    dev = torch.device("cuda:0")
    rgba = torch.tensor(np.stack([d[0] for d in data]), device=dev)
    t = torch.tensor(np.stack([d[1] for d in data]), device=dev, requires_grad=True)
    c = torch.tensor(np.stack([d[2] for d in data]), device=dev, requires_grad=True)
    go = torch.tensor(np.stack([d[3] for d in data]), device=dev)
    out = A.hfbs_solve(rgba, t, c, D.HFBSGridParams(**params), D.COLOR_SPACE.RGB)
    (out * go).sum().backward()
    for i, (g, tt, cc, gout) in enumerate(data):
        ref_out, rt, rc, _ = _gpu(D, g, tt, cc, params, (8, 5, 16), gout)
        assert np.array_equal(out[i].detach().cpu().numpy(), ref_out)
        assert np.array_equal(t.grad[i].cpu().numpy(), rt)
        assert np.array_equal(c.grad[i].cpu().numpy(), rc)


@pytest.mark.parametrize("bf16", [0, 1])
def test_batch_hfbs_backward_matches_single_handles(gpu_ready, bf16):
    """dtsgb_batch_hfbs_backward over ragged instances (one graph-replayed
    launch sequence) against one HFBS handle per instance.  The batch stores
    the overflow bin and pads like a handle whose max grid exceeds the grid;
    BF16 storage is compared on BF16-rounded inputs."""
    D = gpu_ready
    sizes = [(96, 64), (71, 53), (40, 24)]
    params = dict(BASE, optim_iter_max=24)
    data = [_inputs(81 + i, w, h, "graded") for i, (w, h) in enumerate(sizes)]
    b = D.Batch(sizes, flags=D.FLAG_BF16_STORAGE if bf16 else 0)
    b.enable_grad(True, 0)
    b.upload(D.COLOR_SPACE.RGB, [d[0] for d in data], [d[1] for d in data],
             [d[2] for d in data])
    b.solve_hfbs(D.HFBSGridParams(**params))
    outs = b.download(1)
    for rep in range(2):  # the second backward replays the captured graph
        gts, gcs = b.hfbs_backward([d[3] for d in data])
    assert b.hfbs_grad_info() == (1, 8 + 24)
    for i, ((w, h), (g, t, c, gout)) in enumerate(zip(sizes, data)):
        if bf16:
            t, c = P.bf16_round(t), P.bf16_round(c)
        gx, gy = -(-w // 8), -(-h // 8)
        out, gt, gc, _ = _gpu(D, g, t, c, params, (gx + 8, gy + 8, 24), gout)
        assert np.abs(outs[i] - out).max() <= 1e-6 * P.target_range(t)
        _close(gts[i], gt, 1e-5)
        _close(gcs[i], gc, 1e-5)
    b.upload(D.COLOR_SPACE.RGB, [d[0] for d in data], [d[1] for d in data],
             [d[2] for d in data])
    with pytest.raises(D.DtsgbError):  # new inputs: no differentiable solve
        b.hfbs_backward([d[3] for d in data])


def test_batch_hfbs_backward_device_matches_host(gpu_ready):
    """dtsgb_batch_hfbs_backward_device (caller device buffers, here torch
    tensors) returns what the host-pointer call returns, bit for bit, and a
    null confidence-gradient pointer array is skipped."""
    torch = pytest.importorskip("torch")
    D = gpu_ready
    sizes = [(96, 64), (71, 53)]
    params = dict(BASE, optim_iter_max=12)
    data = [_inputs(91 + i, w, h, "graded") for i, (w, h) in enumerate(sizes)]
    b = D.Batch(sizes)
    b.enable_grad(True, 0)
    b.upload(D.COLOR_SPACE.RGB, [d[0] for d in data], [d[1] for d in data],
             [d[2] for d in data])
    b.solve_hfbs(D.HFBSGridParams(**params))
    gts, gcs = b.hfbs_backward([d[3] for d in data])
    dev = torch.device("cuda:0")
    go = [torch.tensor(d[3], device=dev) for d in data]
    gt = [torch.empty_like(g) for g in go]
    gc = [torch.empty_like(g) for g in go]
    b.hfbs_backward_device([g.data_ptr() for g in go], [g.data_ptr() for g in gt],
                           [g.data_ptr() for g in gc])
    torch.cuda.synchronize()
    for i in range(2):
        assert np.array_equal(gt[i].cpu().numpy(), gts[i])
        assert np.array_equal(gc[i].cpu().numpy(), gcs[i])
    gt2 = [torch.zeros_like(g) for g in go]
    b.hfbs_backward_device([g.data_ptr() for g in go], [g.data_ptr() for g in gt2], None)
    torch.cuda.synchronize()
    for i in range(2):
        assert np.array_equal(gt2[i].cpu().numpy(), gts[i])


@pytest.mark.parametrize("w,h,conf,K,segment", [
    (40, 24, "zero", 12, 0),  # no data term: dL/dtarget = 0, dL/dconfidence is not
    (1, 1, "graded", 6, 0),   # a one-pixel image, a 1 x 1 x 16 grid
    (5, 3, "graded", 9, 4),   # a partial cell, segments of 4 steps
    (17, 9, "graded", 1, 3),  # a single step: the segment request is clamped
])
def test_hfbs_adjoint_edge_cases(gpu_ready, oracle_mod, w, h, conf, K, segment):
    params = dict(BASE, optim_iter_max=K, bistoch_iter_max=7)
    g, t, c, gout = _inputs(101 + w, w, h, "graded")
    if conf == "zero":
        c = np.zeros_like(t)
    mg = (-(-w // 8) + 1, -(-h // 8) + 1, 17)
    _, gt, gc, s = _gpu(gpu_ready, g, t, c, params, mg, gout, segment=segment)
    _, rt, rc, _ = _oracle(oracle_mod, g, t, c, params, mg, gout)
    if conf == "zero":
        assert not gt.any() and not rt.any()
    else:
        _close(gt, rt)
    _close(gc, rc)
    assert s.GradInfo()[0] == (1 if K <= 1 else (segment or 1))


def test_persistent_heavy_ball_matches_the_per_block_kernel(gpu_ready):
    """A plain HFBS solve runs the persistent heavy-ball kernel (one CTA per
    SM walking the blocks, the next block staged while one is solved); a
    differentiable solve runs the kernel with one CTA per block that keeps
    the iterates.  Their results agree bit for bit over ragged instances of
    many blocks, also when the instances are solved in groups."""
    D = gpu_ready
    sizes = [(400, 300), (333, 129), (180, 450), (64, 40)]
    params = dict(BASE, optim_iter_max=24)
    data = [_inputs(91 + i, w, h, "graded") for i, (w, h) in enumerate(sizes)]

    def run(grad, group):
        b = D.Batch(sizes)
        b.set_tuning(D.TUNE_HFBS_GROUP_VOXELS, group)
        if grad:
            b.enable_grad(True, 0)
        b.upload(D.COLOR_SPACE.RGB, [d[0] for d in data], [d[1] for d in data],
                 [d[2] for d in data])
        b.solve_hfbs(D.HFBSGridParams(**params))
        return b.download(1)

    ref = run(True, 0)
    for group in (0, 30000):
        for a, r in zip(run(False, group), ref):
            assert np.array_equal(a, r, equal_nan=True)
