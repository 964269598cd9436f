"""Soft-window DTS on the GPU (dtsgb_soft_*): the relaxation of the integer
windows that gives gradients with respect to the guide-derived edge weights
dH, dV.  Checked against the FP64 oracle's restatement of the same
relaxation (forward and adjoint) and against FP64 central differences of
the oracle's forward on 256 edge-weight entries."""
import numpy as np
import pytest

import parity as P

pytestmark = pytest.mark.gpu

FILT = dict(sigma_x=8.0, sigma_y=8.0, sigma_r=0.1)
TAU = 1.0
TOL_GRAD = 1e-4  # relative to max |oracle gradient|


def _inputs(seed, w, h, cmax=1.0):
    from domain_transform_solver_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    inst = W.depth_sr_instance(seed, w, h, n_poly=6, sample_frac=0.2)
    c = (cmax * rng.random((h, w))).astype(np.float32)
    g = rng.standard_normal((h, w)).astype(np.float32)
    return inst.rgba, inst.target, c, g


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def _gpu_edges(D, rgbas):
    import torch
    from domain_transform_solver_gb300.autograd import edge_weights
    dh, dv = edge_weights(_dev(np.stack(rgbas)), D.DomainFilterParams(**FILT))
    torch.cuda.synchronize()
    return dh, dv


def _gpu_soft(D, dh, dv, ts, cs, opt, gs=None):
    """forward (and backward for upstream gradients gs) through SoftDTS."""
    import torch
    n = dh.shape[0]
    h, w = dh.shape[1:]
    s = D.SoftDTS([(w, h)] * n)
    t, c = _dev(np.stack(ts)), _dev(np.stack(cs))
    out = torch.empty_like(t)
    p = lambda x: [x[i].data_ptr() for i in range(n)]  # noqa: E731
    s.solve(p(dh), p(dv), p(t), p(c), D.DomainOptimizeParams(**opt), TAU, p(out))
    torch.cuda.synchronize()
    res = [out.cpu().numpy()]
    if gs is not None:
        g = _dev(np.stack(gs))
        grads = [torch.empty_like(t) for _ in range(4)]
        s.backward(p(g), *[p(x) for x in grads])
        torch.cuda.synchronize()
        res += [x.cpu().numpy() for x in grads]
    s.close()
    return res


def test_edge_weights_match_the_oracle(gpu_ready, oracle_mod):
    D = gpu_ready
    data = [_inputs(700 + i, 70, 45) for i in range(2)]
    dh, dv = _gpu_edges(D, [r for r, _, _, _ in data])
    for i, (rgba, _, _, _) in enumerate(data):
        rh, rv = oracle_mod.edge_weights(rgba, 1, **FILT)
        assert np.abs(dh[i].cpu().numpy() - rh).max() <= 2e-6 * np.abs(rh).max()
        assert np.abs(dv[i].cpu().numpy() - rv).max() <= 2e-6 * np.abs(rv).max()


@pytest.mark.parametrize("loss,cmax", [(1, 1.0), (2, 0.001)])
def test_soft_forward_and_adjoint_match_the_oracle(gpu_ready, oracle_mod, loss, cmax):
    """Forward: max-abs 1e-4 x range.  Adjoint: a ramp end (|D - sigma| =
    tau/2) is a kink of the weights, and a pair whose FP32 distance falls on
    the other side of it than the FP64 one moves that edge weight's gradient
    by its pair term; such entries are counted (at most 0.1%) and the rest
    held to max-abs 1e-4 x max |gradient|."""
    D = gpu_ready
    data = [_inputs(720 + i + 10 * loss, w, h, cmax) for i, (w, h) in
            enumerate([(96, 64), (96, 64)])]
    opt = dict(num_iterations=6, loss=loss, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    dh, dv = _gpu_edges(D, [r for r, _, _, _ in data])
    out, gt, gc, geh, gev = _gpu_soft(D, dh, dv, [t for _, t, _, _ in data],
                                      [c for _, _, c, _ in data], opt,
                                      [g for _, _, _, g in data])
    for i, (rgba, t, c, g) in enumerate(data):
        eh, ev = dh[i].cpu().numpy(), dv[i].cpu().numpy()
        ref = oracle_mod.soft_solve(eh, ev, t, c, opt, TAU)
        assert np.abs(out[i] - ref).max() <= P.TOL_REL * P.target_range(t)
        rgrads = oracle_mod.soft_backward(eh, ev, t, c, opt, TAU, g)
        for got, r in zip((gt[i], gc[i], geh[i], gev[i]), rgrads):
            err = np.abs(got - r)
            bar = TOL_GRAD * max(float(np.abs(r).max()), 1e-12)
            assert float(np.mean(err > bar)) <= 1e-3, (float(err.max()), bar)


def _check_against_oracle(O, data, eh_all, ev_all, opt, res):
    out, gt, gc, geh, gev = res
    for i, (_, t, c, g) in enumerate(data):
        eh, ev = eh_all[i], ev_all[i]
        ref = O.soft_solve(eh, ev, t, c, opt, TAU)
        assert np.abs(out[i] - ref).max() <= P.TOL_REL * P.target_range(t)
        rgrads = O.soft_backward(eh, ev, t, c, opt, TAU, g)
        for got, r in zip((gt[i], gc[i], geh[i], gev[i]), rgrads):
            err = np.abs(got - r)
            bar = TOL_GRAD * max(float(np.abs(r).max()), 1e-12)
            assert float(np.mean(err > bar)) <= 1e-3, (float(err.max()), bar)


@pytest.mark.parametrize("sizes", [[(1100, 40), (45, 130)], [(1024, 30), (300, 70)]])
@pytest.mark.parametrize("scale", [1.0, 0.1])
def test_soft_ragged_tiles_and_small_weights(gpu_ready, oracle_mod, scale, sizes):
    """Instances that span several shared-memory tiles, with partial ones
    (1100 x 40: rows wider than 1024 pixels, whose X kernels take four pixels
    a thread; 45 x 130), rows of exactly 1024 pixels, and the same with
    edge weights scaled by 0.1, whose windows reach past the tiles' largest
    halo: those solves run the global-memory kernels.  All are held to the
    oracle's bars."""
    D = gpu_ready
    import torch
    data = [_inputs(800 + i, w, h) for i, (w, h) in enumerate(sizes)]
    opt = dict(num_iterations=4, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    s = D.SoftDTS(sizes)
    ehs, evs, ptrs = [], [], {}
    for i, (rgba, t, c, g) in enumerate(data):
        dh, dv = _gpu_edges(D, [rgba])
        ehs.append(dh[0].cpu().numpy() * np.float32(scale))
        evs.append(dv[0].cpu().numpy() * np.float32(scale))
    dev = {k: [_dev(x) for x in v] for k, v in
           (("eh", ehs), ("ev", evs), ("t", [d[1] for d in data]), ("c", [d[2] for d in data]),
            ("g", [d[3] for d in data]))}
    p = lambda xs: [x.data_ptr() for x in xs]  # noqa: E731
    out = [torch.empty_like(x) for x in dev["t"]]
    s.solve(p(dev["eh"]), p(dev["ev"]), p(dev["t"]), p(dev["c"]),
            D.DomainOptimizeParams(**opt), TAU, p(out))
    grads = [[torch.empty_like(x) for x in dev["t"]] for _ in range(4)]
    s.backward(p(dev["g"]), *[p(gr) for gr in grads])
    torch.cuda.synchronize()
    s.close()
    res = [[x.cpu().numpy() for x in out]] + [[x.cpu().numpy() for x in gr] for gr in grads]
    _check_against_oracle(oracle_mod, data, ehs, evs, opt, res)


def test_soft_edge_gradients_match_fp64_central_differences(gpu_ready, oracle_mod):
    """256 entries (128 of dH, 128 of dV) of one 64x48 instance: d/de sum(g*v)
    by central differences of the FP64 oracle's soft forward."""
    D = gpu_ready
    rgba, t, c, g = _inputs(760, 64, 48)
    opt = dict(num_iterations=10, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    dh, dv = _gpu_edges(D, [rgba])
    _, _, _, geh, gev = _gpu_soft(D, dh, dv, [t], [c], opt, [g])
    eh = dh[0].cpu().numpy().astype(np.float64)
    ev = dv[0].cpu().numpy().astype(np.float64)
    t64, c64, g64 = (a.astype(np.float64) for a in (t, c, g))
    rng = np.random.default_rng(13)
    idx = rng.choice(t.size, 256, replace=False)
    bars = {"h": 2e-4 * float(np.abs(geh[0]).max()), "v": 2e-4 * float(np.abs(gev[0]).max())}
    bad = []
    for k, flat in enumerate(idx):
        which = "h" if k < 128 else "v"
        base = eh if which == "h" else ev
        hstep = 1e-6
        plus, minus = base.copy(), base.copy()
        plus.flat[flat] += hstep
        minus.flat[flat] -= hstep
        args_p = (plus, ev) if which == "h" else (eh, plus)
        args_m = (minus, ev) if which == "h" else (eh, minus)
        lp = float(np.sum(g64 * oracle_mod.soft_solve(*args_p, t64, c64, opt, TAU)))
        lm = float(np.sum(g64 * oracle_mod.soft_solve(*args_m, t64, c64, opt, TAU)))
        fd = (lp - lm) / (2 * hstep)
        got = float((geh if which == "h" else gev)[0].flat[flat])
        if abs(got - fd) > bars[which]:
            bad.append((which, int(flat), got, fd))
    # a perturbation that crosses a ramp end (a kink) has no derivative
    assert len(bad) <= 2, bad


def test_soft_autograd_binding(gpu_ready):
    """soft_dts_solve returns what SoftDTS returns, and its gradients are
    the adjoint's."""
    torch = pytest.importorskip("torch")
    D = gpu_ready
    from domain_transform_solver_gb300.autograd import soft_dts_solve
    data = [_inputs(780 + i, 80, 60) for i in range(3)]
    opt = dict(num_iterations=5, loss=1, lambda_=0.99, sigma_z=8.0, step_size=0.99)
    dh, dv = _gpu_edges(D, [r for r, _, _, _ in data])
    ts, cs, gs = ([x[k] for x in data] for k in (1, 2, 3))
    ref = _gpu_soft(D, dh, dv, ts, cs, opt, gs)
    dh_ = dh.clone().requires_grad_()
    dv_ = dv.clone().requires_grad_()
    t_ = _dev(np.stack(ts)).requires_grad_()
    c_ = _dev(np.stack(cs)).requires_grad_()
    v = soft_dts_solve(dh_, dv_, t_, c_, D.DomainOptimizeParams(**opt), TAU)
    (v * _dev(np.stack(gs))).sum().backward()
    assert np.array_equal(v.detach().cpu().numpy(), ref[0])
    for got, r in zip((t_.grad, c_.grad, dh_.grad, dv_.grad), ref[1:]):
        assert np.array_equal(got.cpu().numpy(), r)


def test_soft_rejects_bad_arguments(gpu_ready):
    import torch
    D = gpu_ready
    s = D.SoftDTS([(16, 16)])
    x = torch.zeros((16, 16), device="cuda")
    p = [x.data_ptr()]
    with pytest.raises(D.DtsgbError):
        s.solve(p, p, p, None, D.DomainOptimizeParams(num_iterations=2, loss=1, sigma_z=4.0),
                9.0, p)  # tau above 2 sigma_z
    with pytest.raises(D.DtsgbError):
        s.backward(p)  # nothing solved
    s.close()
