"""Non-finite targets and confidences.

The DTS iteration sums its windows in fixed point, which has no form for an
infinity or a NaN.  A tile whose staged values (or X results) hold one
writes NaN instead (every pixel of the tile can reach that value within the
iteration), so a non-finite input spreads as NaN -- as the reference's float
prefix sums carry it along rows and columns -- and never becomes finite
garbage.  Checked here: every output pixel that depends on the bad input is
NaN, and every finite output pixel equals the solve with a finite value
there.  HFBS computes in float throughout: the Laplace blur carries a NaN
across the grid, so the whole result is NaN."""
import numpy as np
import pytest

import parity as P

pytestmark = pytest.mark.gpu


def _solve(D, insts, targets, confs, flags, opt):
    from domain_transform_solver_gb300 import workloads as W
    b = D.Batch([(i.width, i.height) for i in insts], flags=flags)
    b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], targets, confs)
    b.solve_dts(D.DomainFilterParams(**W.CFG0_FILTER), D.DomainOptimizeParams(**opt))
    out = b.download(0)
    b.close()
    return out


@pytest.mark.parametrize("flags", [0, 1])
@pytest.mark.parametrize("where,bad", [("target", np.nan), ("target", np.inf),
                                       ("confidence", np.nan), ("confidence", -np.inf)])
def test_dts_non_finite_input_spreads_as_nan(gpu_ready, flags, where, bad):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = [W.depth_sr_instance(60 + k, w, h, n_poly=10, sample_frac=0.2)
             for k, (w, h) in enumerate([(900, 700), (300, 200)])]
    opt = dict(W.CFG0_OPT, num_iterations=3)
    p = (350, 411)  # (y, x) in instance 0
    outs = {}
    for key, val in (("bad", bad), ("a", 0.0), ("b", 0.75)):
        ts = [i.target.copy() for i in insts]
        cs = [i.confidence.copy() for i in insts]
        arr = ts[0] if where == "target" else cs[0]
        arr[p] = val
        if where == "confidence":
            ts[0][p] = 4.0  # the confidence matters only where the target differs from v
        outs[key] = _solve(D, insts, ts, cs, flags, opt)
    rng_t = P.target_range(insts[0].target)
    bad0, a0, b0 = outs["bad"][0], outs["a"][0], outs["b"][0]
    depends = np.abs(a0 - b0) > 1e-4 * rng_t
    assert depends[p] and depends.sum() > 10
    assert np.isnan(bad0[depends]).all(), "a pixel that depends on the bad value is finite"
    fin = np.isfinite(bad0)
    assert fin.mean() > 0.3, "NaN spread beyond what three iterations can reach"
    assert np.abs(bad0[fin] - a0[fin]).max() <= 1e-5 * rng_t
    # the other instance of the batch is untouched
    assert np.array_equal(outs["bad"][1], outs["a"][1])


def test_hfbs_non_finite_target_gives_nan(gpu_ready):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(70, 200, 150, n_poly=6, sample_frac=0.2)
    t = inst.target.copy()
    c = inst.confidence.copy()
    t[40, 50], c[40, 50] = np.nan, 1.0
    b = D.Batch([(200, 150)])
    b.upload(D.COLOR_SPACE.YCbCr, [inst.rgba], [t], [c])
    b.solve_hfbs(D.HFBSGridParams(**dict(W.CFG1_HFBS, optim_iter_max=8)))
    out = b.download(1)[0]
    assert np.isnan(out).all()
