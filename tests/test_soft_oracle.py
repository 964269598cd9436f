"""The oracle's soft-window DTS (the relaxation of the integer windows that
makes the solve differentiable in the edge weights) on the CPU: its adjoint
against FP64 central differences of its forward, and the relaxation's limit
as the ramp width goes to zero."""
import numpy as np
import pytest

OPT = dict(num_iterations=4, loss=1, lambda_=0.99, sigma_z=4.0, step_size=0.99)


def _inputs(seed, w=23, h=17):
    rng = np.random.default_rng(seed)
    eh = 1.0 + 2.0 * rng.random((h, w))
    ev = 1.0 + 2.0 * rng.random((h, w))
    t = rng.uniform(0.5, 10.0, (h, w))
    c = rng.random((h, w)) * (rng.random((h, w)) < 0.4)
    g = rng.standard_normal((h, w))
    return eh, ev, t, c, g


@pytest.mark.parametrize("loss,cmax", [(1, 1.0), (2, 0.001)])
def test_soft_adjoint_matches_central_differences(oracle_mod, loss, cmax):
    O = oracle_mod
    eh, ev, t, c, g = _inputs(3 + loss)
    c = c * cmax
    opt = dict(OPT, loss=loss)
    tau = 1.0
    gt, gc, geh, gev = O.soft_backward(eh, ev, t, c, opt, tau, g)
    rng = np.random.default_rng(9)
    bad = 0
    for name, arr, grad in (("eh", eh, geh), ("ev", ev, gev), ("t", t, gt), ("c", c, gc)):
        for flat in rng.choice(arr.size, 24, replace=False):
            h = 1e-6
            p, m = arr.copy(), arr.copy()
            p.flat[flat] += h
            m.flat[flat] -= h
            args = {"eh": eh, "ev": ev, "t": t, "c": c}
            lp = float(np.sum(g * O.soft_solve(**{**args, name: p}, opt=opt, tau=tau)))
            lm = float(np.sum(g * O.soft_solve(**{**args, name: m}, opt=opt, tau=tau)))
            fd = (lp - lm) / (2 * h)
            if abs(fd - grad.flat[flat]) > 1e-6 * max(1.0, np.abs(grad).max()):
                bad += 1
    # an entry whose perturbation crosses a ramp end (a kink) may differ
    assert bad <= 1


def test_soft_windows_tend_to_the_clipped_integer_windows(oracle_mod):
    """With a narrow ramp the soft solve equals the integer-window solve on
    windows clipped at the borders (computed here by brute force)."""
    O = oracle_mod
    eh, ev, t, c, _ = _inputs(11, w=15, h=12)
    opt = dict(OPT, num_iterations=3)
    soft = O.soft_solve(eh, ev, t, c, opt, tau=1e-7)
    # the oracle takes the parameters as float, like the C ABI
    sig, lam, st = (float(np.float32(opt[k])) for k in ("sigma_z", "lambda_", "step_size"))

    def half(v, e, axis, data):
        out = np.empty_like(v)
        H, W = v.shape
        for y in range(H):
            for x in range(W):
                i, L = (x, W) if axis == 0 else (y, H)
                line_e = e[y, :] if axis == 0 else e[:, x]
                line_v = v[y, :] if axis == 0 else v[:, x]
                cs = np.concatenate([[0.0], np.cumsum(line_e[1:])])  # ct relative to 0
                mem = [q for q in range(L) if abs(cs[q] - cs[i]) <= sig]
                n = len(mem)
                B = line_v[mem].mean()
                h = c[y, x] / n * (v[y, x] - t[y, x]) if data else 0.0
                out[y, x] = v[y, x] - st * (lam * (v[y, x] - B) + h)
        return out

    v = t.copy()
    for _ in range(opt["num_iterations"]):
        v = half(half(v, eh, 0, True), ev, 1, False)
    assert np.abs(soft - v).max() < 1e-9 * np.abs(v).max()
