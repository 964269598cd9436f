"""The benchmark drivers (cli.py) end to end on small synthetic datasets laid
out like the reference CLIs' inputs: outputs written, RMSE lines printed, and
a DTS result equal to the class API's own solve of the same inputs."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _depth_dataset(root, w=96, h=72):
    from domain_transform_solver_gb300 import imageio as IO
    from domain_transform_solver_gb300 import workloads as W
    from domain_transform_solver_gb300.cli import FOLDERS, OUTPUTS, WEIGHTS
    rng = np.random.default_rng(11)
    for k, folder in enumerate(FOLDERS):
        inst = W.depth_sr_instance(300 + k, w, h, n_poly=5)
        for sub in ("_input/" + folder, "bicubic/" + folder, "weights/" + folder, "_gth"):
            os.makedirs(os.path.join(root, sub), exist_ok=True)
        IO.write_png(os.path.join(root, "_input", folder, folder + "_color.png"),
                     np.ascontiguousarray(inst.rgba[..., :3]))
        depth = (inst.target / 10.0).clip(0, 1)
        gt = (rng.random((h, w)) * 255).astype(np.uint8)
        IO.write_png(os.path.join(root, "_gth", folder + ".png"), gt)
        for o, wn in zip(OUTPUTS, WEIGHTS):
            IO.write_png(os.path.join(root, "bicubic", folder, o + ".png"),
                         (depth * 65535).astype(np.uint16))
            IO.write_png(os.path.join(root, "weights", folder, wn + ".png"),
                         (rng.random((h, w)) * 65535).astype(np.uint16))


@pytest.mark.parametrize("algo", ["dts", "hfbs"])
def test_depth_super_res_driver(gpu_ready, tmp_path, capsys, algo):
    D = gpu_ready
    from domain_transform_solver_gb300 import cli
    from domain_transform_solver_gb300 import imageio as IO
    root = str(tmp_path)
    _depth_dataset(root)
    assert cli.main(["depth_super_res", "--path_to_data_top_dir", root,
                     "--algorithm_name", algo]) == 0
    io = capsys.readouterr()
    assert f"Using {algo} algorithm." in io.out
    line = [l for l in io.err.splitlines() if l.startswith("RMSE ")][-1]
    assert np.isfinite(float(line.split()[1].rstrip(",")))
    for folder in cli.FOLDERS:
        for o in cli.OUTPUTS:
            assert IO.read_png(os.path.join(root, algo, folder, o + ".png")).dtype == np.uint8
    if algo == "dts":
        # the first image (art_big, x2) by the class API directly
        folder, o, wn = cli.FOLDERS[0], cli.OUTPUTS[0], cli.WEIGHTS[0]
        rgba = IO.read_rgba(os.path.join(root, "_input", folder, folder + "_color.png"))
        t = IO.read_float_16bit(os.path.join(root, "bicubic", folder, o + ".png"), cli._SCALE16)
        bump = IO.read_float_16bit(os.path.join(root, "weights", folder, wn + ".png"),
                                   cli._SCALE16)
        c = (bump / bump.max()).astype(np.float32)
        h, w = t.shape
        s = D.DomainTransformSolver(D.ImageDim(w, h))
        s.InitFrame(D.COLOR_SPACE.YCbCr, rgba, t, c)
        s.ComputeColorSpaceDifferential(D.DomainFilterParams(16.0, 16.0, 0.1))
        s.IntegrateColorDifferentials()
        s.Optimize(D.DomainOptimizeParams(num_iterations=10, loss=D.RobustLoss.L2,
                                          lambda_=0.99, sigma_z=16.0 / 1.8, step_size=0.99))
        v8 = cli._to_uint8(s.Download(D.ImageType.OPTIMIZED_QUANTITY), 255.0)
        assert np.array_equal(IO.read_png(os.path.join(root, "dts", folder, o + ".png")), v8)


def test_stereo_driver(gpu_ready, tmp_path, capsys):
    from domain_transform_solver_gb300 import cli
    from domain_transform_solver_gb300 import imageio as IO
    from domain_transform_solver_gb300 import workloads as W
    d = tmp_path / "Art"
    d.mkdir()
    inst = W.stereo_instance(7, 120, 80, n_poly=6)
    left = inst.rgba[..., :3]
    right = np.roll(left, -4, axis=1)
    IO.write_png(d / "im0.png", np.ascontiguousarray(left))
    IO.write_png(d / "im1.png", np.ascontiguousarray(right))
    IO.write_disparity_bin(d / "im0.png_disp.bin", inst.target)
    (d / "calib.txt").write_text("cam0=[1 0 0]\ncam1=[1 0 0]\ndoff=2\nbaseline=1\n")
    IO.write_pfm(d / "disp0GT.pfm", inst.target[::-1])
    assert cli._read_doff(str(d / "calib.txt")) == 2
    assert cli.main(["stereo", "--path_to_data_top_dir", str(tmp_path)]) == 0
    io = capsys.readouterr()
    assert "Using DTS algorithm." in io.out
    line = [l for l in io.err.splitlines() if l.startswith("RMSE ")][-1]
    assert np.isfinite(float(line.split()[1].rstrip(",")))
    assert IO.read_png(tmp_path / "dts_Art.png").shape == inst.target.shape


@pytest.mark.parametrize("algo", ["dts", "hfbs"])
def test_colorization_driver(gpu_ready, tmp_path, capsys, algo):
    from domain_transform_solver_gb300 import cli
    from domain_transform_solver_gb300 import imageio as IO
    from domain_transform_solver_gb300 import workloads as W
    rng = np.random.default_rng(12)
    for k, name in enumerate(cli.COLOR_IMAGES):
        inst, _ = W.colorization_instance(500 + k, 88, 64, n_poly=6)
        grey = inst.rgba[..., 0]
        color = np.stack([grey, np.roll(grey, 3, 1), np.roll(grey, 5, 0)], -1).astype(np.uint8)
        strokes = np.repeat(grey[..., None], 3, -1).copy()
        mask = rng.random(grey.shape) < 0.05
        strokes[mask] = color[mask]
        IO.write_bmp(tmp_path / f"{name}.bmp", np.repeat(grey[..., None], 3, -1))
        IO.write_bmp(tmp_path / f"{name}_strokes.bmp", strokes)
        IO.write_bmp(tmp_path / f"{name}_gt.bmp", color)
    assert cli.main(["colorization", "--path_to_data_top_dir", str(tmp_path),
                     "--algorithm_name", algo]) == 0
    io = capsys.readouterr()
    assert f"Using {algo} algorithm." in io.out
    assert sum(l.count("SSIM:") for l in io.out.splitlines()) == 2
    assert any(l.startswith("RMSE ") for l in io.err.splitlines())
    for name in cli.COLOR_IMAGES:
        assert IO.read_bmp(tmp_path / f"{algo}_{name}.bmp").shape == (64, 88, 3)
