"""Batched solves of ragged instances: identical (bitwise) to solving each
image through the class API, with and without CUDA-graph replay, and the
BF16 storage form checked against the FP64 oracle."""
import numpy as np
import pytest

import parity as P

pytestmark = pytest.mark.gpu

SIZES = [(97, 61), (256, 300), (33, 190), (411, 129), (64, 64), (1, 17)]


def _instances(scale_sizes=SIZES):
    from domain_transform_solver_gb300 import workloads as W
    return [W.depth_sr_instance(400 + i, w, h, n_poly=8, sample_frac=0.05)
            for i, (w, h) in enumerate(scale_sizes)]


def _single_dts(D, inst, flags, filt, opt):
    h, w = inst.target.shape
    s = D.DomainTransformSolver(D.ImageDim(w, h), flags=flags)
    s.ClearAll()
    s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, inst.confidence)
    s.ComputeColorSpaceDifferential(D.DomainFilterParams(**filt))
    s.IntegrateColorDifferentials()
    s.Optimize(D.DomainOptimizeParams(**opt))
    return s.Download(D.ImageType.OPTIMIZED_QUANTITY)


def _single_hfbs(D, inst, params):
    h, w = inst.target.shape
    # max grid one larger than the grid on every axis, like a batch instance
    s = D.HFBS(D.ImageDim(w, h), -(-w // 8) + 1, -(-h // 8) + 1, 17)
    s.SetFilterParams(D.HFBSGridParams(**params))
    s.ClearAll()
    s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, inst.confidence)
    s.Optimize()
    return s.Download(D.ImageType.OPTIMIZED_QUANTITY)


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_matches_single_image_solves(gpu_ready, graphs):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances()
    b = D.Batch([(i.width, i.height) for i in insts], use_graphs=graphs)
    b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], [i.target for i in insts],
             [i.confidence for i in insts])
    opt = dict(W.CFG0_OPT, num_iterations=5)
    hp = dict(W.CFG1_HFBS, optim_iter_max=12)
    for rep in range(2):  # second pass replays the captured graphs
        b.solve_dts(D.DomainFilterParams(**W.CFG0_FILTER), D.DomainOptimizeParams(**opt))
        b.solve_hfbs(D.HFBSGridParams(**hp))
        dts_out = b.download(0)
        hfbs_out = b.download(1)
        for inst, v, hv in zip(insts, dts_out, hfbs_out):
            assert np.array_equal(v, _single_dts(D, inst, 0, W.CFG0_FILTER, opt))
            ref = _single_hfbs(D, inst, hp)
            assert np.array_equal(np.isnan(hv), np.isnan(ref))
            assert np.array_equal(hv[~np.isnan(hv)], ref[~np.isnan(ref)])


def test_batch_bf16_storage_against_oracle(gpu_ready, oracle_mod):
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances([(150, 90), (70, 201)])
    b = D.Batch([(i.width, i.height) for i in insts], flags=D.FLAG_BF16_STORAGE)
    b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], [i.target for i in insts],
             [i.confidence for i in insts])
    opt = dict(W.CFG0_OPT, num_iterations=6)
    b.solve_dts(D.DomainFilterParams(**W.CFG0_FILTER), D.DomainOptimizeParams(**opt))
    outs = b.download(0)
    for inst, v in zip(insts, outs):
        ref = _single_dts(D, inst, D.FLAG_BF16_STORAGE, W.CFG0_FILTER, opt)
        assert np.array_equal(v, ref)
        t, c = P.bf16_round(inst.target), P.bf16_round(inst.confidence)
        h, w = t.shape
        s = D.DomainTransformSolver(D.ImageDim(w, h), flags=D.FLAG_BF16_STORAGE)
        s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, inst.confidence)
        s.ComputeColorSpaceDifferential(D.DomainFilterParams(**W.CFG0_FILTER))
        ov = {(a, 8.0): s.DebugBounds(a, 8.0) for a in (0, 1)}
        v64, _ = oracle_mod.dts_solve(inst.rgba, t, c, 1, W.CFG0_FILTER, opt, overrides=ov)
        assert np.abs(v - v64).max() <= P.TOL_REL * P.target_range(t)


def test_batch_rejects_bad_arguments(gpu_ready):
    D = gpu_ready
    with pytest.raises(D.DtsgbError):
        D.Batch([(0, 10)])
    b = D.Batch([(16, 16)])
    with pytest.raises(D.DtsgbError):
        b.download(0)  # nothing solved yet


def test_tuning_knobs_and_autotune(gpu_ready):
    """HFBS grouping changes only the launch order: bitwise-identical grids.
    The DTS tile shape changes the fixed-point scales of the window sums:
    results agree to FP32 rounding.  The autotuner keeps a valid setting."""
    import ctypes
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances()
    b = D.Batch([(i.width, i.height) for i in insts])
    b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], [i.target for i in insts],
             [i.confidence for i in insts])
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    op = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=4))
    hp = D.HFBSGridParams(**dict(W.CFG1_HFBS, optim_iter_max=8))
    outs = {}
    for tile in (64, 32):
        for group in (0, 30000):
            b.set_tuning(D.TUNE_DTS_TILE, tile)
            b.set_tuning(D.TUNE_HFBS_GROUP_VOXELS, group)
            assert b.get_tuning(D.TUNE_DTS_TILE) == tile
            b.solve_dts(fp, op)
            b.solve_hfbs(hp)
            outs[(tile, group)] = (b.download(0), b.download(1))
    ref_d, ref_h = outs[(64, 0)]
    for (tile, group), (d, h) in outs.items():
        for a, r in zip(h, ref_h):
            assert np.array_equal(a, r, equal_nan=True)
        for a, r, inst in zip(d, ref_d, insts):
            assert np.abs(a - r).max() <= 1e-6 * max(P.target_range(inst.target), 1.0)
    # the window-bound walk's segment length changes nothing
    b.set_tuning(D.TUNE_DTS_TILE, 64)
    for seg in (4, 16, 8):
        b.set_tuning(D.TUNE_BOUNDS_SEGMENT, seg)
        b.solve_dts(fp, op)
        for a, r in zip(b.download(0), ref_d):
            assert np.array_equal(a, r)
    # one heavy-ball step per launch: the same solve to FP32 rounding
    b.set_tuning(D.TUNE_HFBS_SOLVE_STEPS, 1)
    b.solve_hfbs(hp)
    for a, r, inst in zip(b.download(1), ref_h, insts):
        fin = np.isfinite(r)
        assert np.array_equal(np.isfinite(a), fin)
        assert np.abs(a[fin] - r[fin]).max() <= 1e-5 * max(P.target_range(inst.target), 1.0)
    b.set_tuning(D.TUNE_HFBS_SOLVE_STEPS, 4)
    b.autotune(fp, op, hp, reps=1)
    assert b.get_tuning(D.TUNE_DTS_TILE) in (64, 32)
    assert b.get_tuning(D.TUNE_BOUNDS_SEGMENT) in (4, 8, 16)
    assert b.get_tuning(D.TUNE_HFBS_SOLVE_STEPS) in (1, 4)
    assert b.get_tuning(D.TUNE_HFBS_GROUP_VOXELS) in (0, 1000000, 2000000, 4000000, 8000000)
    if b.get_tuning(D.TUNE_HFBS_SOLVE_STEPS) == 4:
        for a, r in zip(b.download(1), ref_h):
            assert np.array_equal(a, r, equal_nan=True)


def test_autotune_cache_file(gpu_ready, tmp_path):
    """The first tuning of a case is timed and written to the cache file; a
    second batch of the same sizes and parameters reads the same choice."""
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances(SIZES[:3])
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    op = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=3))
    hp = D.HFBSGridParams(**dict(W.CFG1_HFBS, optim_iter_max=8))
    cache = tmp_path / "autotune.txt"
    choices = []
    for k in range(2):
        b = D.Batch([(i.width, i.height) for i in insts])
        b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], [i.target for i in insts],
                 [i.confidence for i in insts])
        hit = b.autotune(fp, op, hp, reps=1, cache_path=cache)
        assert hit == (k == 1)
        choices.append(b.tuning())
        b.close()
    assert choices[0] == choices[1]
    assert len(cache.read_text().splitlines()) == 1


def test_video_frames_reuse_guide_state(gpu_ready):
    """Frames that change only the target (upload_targets) keep the window
    bounds and the HFBS normalisation: results equal a fresh batch's bitwise,
    and a changed sigma or a new guide recomputes them."""
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances(SIZES[:4])
    sizes = [(i.width, i.height) for i in insts]
    rng = np.random.default_rng(5)
    frames = [[(i.target * (1.0 + 0.1 * k) + rng.normal(0, 0.01, i.target.shape))
               .astype(np.float32) for i in insts] for k in range(3)]
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    hp = D.HFBSGridParams(**dict(W.CFG1_HFBS, optim_iter_max=8))
    b = D.Batch(sizes)
    b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], frames[0],
             [i.confidence for i in insts])
    for k, frame in enumerate(frames):
        sz = 8.0 if k < 2 else 6.0  # the last frame changes sigma_z
        op = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=4, sigma_z=sz))
        if k:
            b.upload_targets(frame, [i.confidence for i in insts])
        b.solve_dts(fp, op)
        b.solve_hfbs(hp)
        fresh = D.Batch(sizes, use_graphs=False)
        fresh.set_tuning(D.TUNE_REUSE_GUIDE_STATE, 0)
        fresh.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], frame,
                     [i.confidence for i in insts])
        fresh.solve_dts(fp, op)
        fresh.solve_hfbs(hp)
        for a, r in zip(b.download(0), fresh.download(0)):
            assert np.array_equal(a, r)
        for a, r in zip(b.download(1), fresh.download(1)):
            assert np.array_equal(a, r, equal_nan=True)
    # a new guide invalidates the kept state
    rgba2 = [np.ascontiguousarray(i.rgba[::-1]) for i in insts]
    b.upload(D.COLOR_SPACE.YCbCr, rgba2, frames[0], [i.confidence for i in insts])
    op = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=4))
    b.solve_dts(fp, op)
    fresh = D.Batch(sizes)
    fresh.upload(D.COLOR_SPACE.YCbCr, rgba2, frames[0], [i.confidence for i in insts])
    fresh.solve_dts(fp, op)
    for a, r in zip(b.download(0), fresh.download(0)):
        assert np.array_equal(a, r)


def test_large_halos(gpu_ready):
    """sigma_z = 100 exceeds the tile-staged kernel's shared memory on 64 x 128
    tiles (the large-halo kernel runs instead); sigma_z = 200 exceeds both
    kernels there and runs on 32 x 32 tiles.  Class API and batch agree
    bitwise on the same tiles; the tile shapes agree to FP32 rounding."""
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    inst = W.depth_sr_instance(77, 2560, 1024, n_poly=12, sample_frac=0.05)
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    rng_t = float(inst.target.max() - inst.target.min())
    for sz in (100.0, 200.0):
        op = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=2, sigma_z=sz))
        s = D.DomainTransformSolver(D.ImageDim(2560, 1024))
        s.InitFrame(D.COLOR_SPACE.YCbCr, inst.rgba, inst.target, inst.confidence)
        s.ComputeColorSpaceDifferential(fp)
        s.IntegrateColorDifferentials()
        s.Optimize(op)
        v = s.Download(D.ImageType.OPTIMIZED_QUANTITY)
        assert np.isfinite(v).all()
        outs = {}
        for tile in (64, 32):
            b = D.Batch([(2560, 1024)])
            assert b.get_tuning(D.TUNE_DTS_TILE) == 64
            b.set_tuning(D.TUNE_DTS_TILE, tile)
            b.upload(D.COLOR_SPACE.YCbCr, [inst.rgba], [inst.target], [inst.confidence])
            b.solve_dts(fp, op)
            outs[tile] = b.download(0)[0]
        assert np.array_equal(v, outs[64])
        assert np.abs(outs[64] - outs[32]).max() <= 1e-6 * rng_t
        if sz == 200.0:
            assert np.array_equal(outs[64], outs[32])


@pytest.mark.parametrize("chunks", [1, 3, 10])
def test_pipeline_matches_batch(gpu_ready, chunks):
    """dtsgb_pipeline_run (chunks of instances on their own streams, copies
    overlapping solves) gives the batch's results bitwise, for both solvers
    and for one solver alone."""
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances()
    sizes = [(i.width, i.height) for i in insts]
    rgba = [i.rgba for i in insts]
    tgt = [i.target for i in insts]
    conf = [i.confidence for i in insts]
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    opt = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=5))
    hp = D.HFBSGridParams(**dict(W.CFG1_HFBS, optim_iter_max=13))
    b = D.Batch(sizes, flags=D.FLAG_BF16_STORAGE)
    b.upload(D.COLOR_SPACE.YCbCr, rgba, tgt, conf)
    b.solve_dts(fp, opt)
    b.solve_hfbs(hp)
    ref_d, ref_h = b.download(0), b.download(1)
    p = D.Pipeline(sizes, flags=D.FLAG_BF16_STORAGE, n_chunks=chunks)
    assert p.n_chunks == min(chunks, len(sizes))
    for _ in range(2):  # the second run replays each chunk's graphs
        od, oh = p.run(D.COLOR_SPACE.YCbCr, rgba, tgt, conf, fp, opt, hp)
        for a, r in zip(od, ref_d):
            assert np.array_equal(a, r)
        for a, r in zip(oh, ref_h):
            assert np.array_equal(a, r, equal_nan=True)
    od, oh = p.run(D.COLOR_SPACE.YCbCr, rgba, tgt, conf, fp, opt, None)
    assert oh is None and all(np.array_equal(a, r) for a, r in zip(od, ref_d))
    od, oh = p.run(D.COLOR_SPACE.YCbCr, rgba, tgt, conf, grid_params=hp)
    assert od is None and all(np.array_equal(a, r, equal_nan=True) for a, r in zip(oh, ref_h))
    p.close()


def test_pipeline_pinned_buffers(gpu_ready):
    """The asynchronous path of dtsgb_pipeline_run (pinned host buffers passed
    as raw pointers) gives the pageable path's results bitwise."""
    torch = pytest.importorskip("torch")
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances()
    sizes = [(i.width, i.height) for i in insts]
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    opt = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=4))
    hp = D.HFBSGridParams(**dict(W.CFG1_HFBS, optim_iter_max=9))
    p = D.Pipeline(sizes, flags=D.FLAG_BF16_STORAGE, n_chunks=3)
    ref_d, ref_h = p.run(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts],
                         [i.target for i in insts], [i.confidence for i in insts], fp, opt, hp)

    def pin(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory()

    rg = [pin(i.rgba) for i in insts]
    tg = [pin(i.target) for i in insts]
    cf = [pin(i.confidence) for i in insts]
    od = [torch.empty((h, w), dtype=torch.float32).pin_memory() for w, h in sizes]
    oh = [torch.empty((h, w), dtype=torch.float32).pin_memory() for w, h in sizes]
    ptrs = lambda ts: [t.data_ptr() for t in ts]  # noqa: E731
    p.run_ptrs(D.COLOR_SPACE.YCbCr, ptrs(rg), ptrs(tg), ptrs(cf), fp, opt, hp, ptrs(od),
               ptrs(oh))
    for a, r in zip(od, ref_d):
        assert np.array_equal(a.numpy(), r)
    for a, r in zip(oh, ref_h):
        assert np.array_equal(a.numpy(), r, equal_nan=True)
    p.close()


@pytest.mark.parametrize("flags", [0, 1])
def test_missing_confidences_are_ones(gpu_ready, flags):
    """A host upload without confidences, or with None entries, solves as
    with explicit ones (the staged upload fills them on the device), for FP32
    and BF16 storage."""
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances()
    sizes = [(i.width, i.height) for i in insts]
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    opt = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=3))
    ones = [np.ones((h, w), np.float32) for w, h in sizes]
    outs = []
    for conf in (ones, None, [None if k % 2 else o for k, o in enumerate(ones)]):
        b = D.Batch(sizes, flags=flags)
        b.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], [i.target for i in insts], conf)
        b.solve_dts(fp, opt)
        outs.append(b.download(0))
    for res in outs[1:]:
        for a, r in zip(res, outs[0]):
            assert np.array_equal(a, r)


@pytest.mark.parametrize("flags", [0, 1])
def test_device_uploads_match_host_uploads(gpu_ready, flags):
    """Uploads from device pointers (FP32 and BF16 storage, some confidences
    missing) solve exactly as the same images uploaded from the host."""
    torch = pytest.importorskip("torch")
    D = gpu_ready
    from domain_transform_solver_gb300 import workloads as W
    insts = _instances()
    sizes = [(i.width, i.height) for i in insts]
    fp = D.DomainFilterParams(**W.CFG0_FILTER)
    opt = D.DomainOptimizeParams(**dict(W.CFG0_OPT, num_iterations=3))
    conf = [None if k % 2 else i.confidence for k, i in enumerate(insts)]
    ref = D.Batch(sizes, flags=flags)
    ref.upload(D.COLOR_SPACE.YCbCr, [i.rgba for i in insts], [i.target for i in insts], conf)
    ref.solve_dts(fp, opt)
    dev = torch.device("cuda:0")
    rg = [torch.from_numpy(np.ascontiguousarray(i.rgba)).to(dev) for i in insts]
    tg = [torch.from_numpy(i.target).to(dev) for i in insts]
    cf = [None if c is None else torch.from_numpy(c).to(dev) for c in conf]
    torch.cuda.synchronize()
    b = D.Batch(sizes, flags=flags)
    b.upload_device(D.COLOR_SPACE.YCbCr, [x.data_ptr() for x in rg],
                    [x.data_ptr() for x in tg], [0 if x is None else x.data_ptr() for x in cf])
    b.solve_dts(fp, opt)
    for a, r in zip(b.download(0), ref.download(0)):
        assert np.array_equal(a, r)
