"""Host-side formats and drivers of the benchmark CLIs (PNG, PFM, raw float
disparity; RMSE bookkeeping).  CPU only: the PNG row filters are undone by
libdtsgb's host helper, checked here against a Python restatement."""
import io
import zlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def IO(dts):
    from domain_transform_solver_gb300 import imageio
    return imageio


@pytest.mark.parametrize("shape,dtype", [((7, 9), np.uint8), ((5, 4, 3), np.uint8),
                                         ((6, 3, 4), np.uint8), ((4, 5), np.uint16),
                                         ((3, 3, 3), np.uint16)])
def test_png_round_trip(IO, tmp_path, shape, dtype):
    rng = np.random.default_rng(1)
    a = rng.integers(0, np.iinfo(dtype).max + 1, shape).astype(dtype)
    p = tmp_path / "x.png"
    IO.write_png(p, a)
    assert np.array_equal(IO.read_png(p), a)


def _filtered(rows: np.ndarray, bpp: int, rng) -> bytes:
    """Encode rows with random PNG filter types (the inverse of unfiltering)."""
    h, stride = rows.shape
    out = bytearray()
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        cur = rows[y].astype(np.int32)
        t = int(rng.integers(0, 5))
        f = np.zeros(stride, np.int32)
        for i in range(stride):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if t == 0:
                pred = 0
            elif t == 1:
                pred = a
            elif t == 2:
                pred = b
            elif t == 3:
                pred = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            f[i] = (cur[i] - pred) & 0xFF
        out += bytes([t]) + f.astype(np.uint8).tobytes()
        prev = cur
    return bytes(out)


@pytest.mark.parametrize("bpp", [1, 2, 3, 4, 6])
def test_png_unfilter_library_matches_python(IO, bpp):
    rng = np.random.default_rng(bpp)
    rows = rng.integers(0, 256, (9, 5 * bpp)).astype(np.uint8)
    raw = _filtered(rows, bpp, rng)
    assert np.array_equal(IO._unfilter(raw, 9, 5 * bpp, bpp), rows)
    assert np.array_equal(IO._unfilter_py(raw, 9, 5 * bpp, bpp), rows)


def test_png_with_filters_and_palette(IO, tmp_path):
    import struct
    rng = np.random.default_rng(3)
    idx = rng.integers(0, 4, (6, 7)).astype(np.uint8)
    pal = np.array([[0, 0, 0], [255, 0, 0], [0, 255, 0], [10, 20, 30]], np.uint8)
    raw = _filtered(idx, 1, rng)

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body))

    data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 7, 6, 8, 3, 0, 0, 0)) +
            chunk(b"PLTE", pal.tobytes()) + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))
    p = tmp_path / "p.png"
    p.write_bytes(data)
    assert np.array_equal(IO.read_png(p), pal[idx])
    rgba = IO.read_rgba(p)
    assert rgba.shape == (6, 7, 4) and (rgba[..., 3] == 0).all()
    assert np.array_equal(rgba[..., :3], pal[idx])


def test_pfm_and_disparity_bin(IO, tmp_path):
    rng = np.random.default_rng(4)
    a = rng.normal(size=(5, 8)).astype(np.float32)
    IO.write_pfm(tmp_path / "a.pfm", a)
    assert np.array_equal(IO.read_pfm(tmp_path / "a.pfm"), a)
    c = rng.normal(size=(3, 4, 3)).astype(np.float32)
    IO.write_pfm(tmp_path / "c.pfm", c)
    assert np.array_equal(IO.read_pfm(tmp_path / "c.pfm"), c)
    # big-endian files (positive scale)
    (tmp_path / "b.pfm").write_bytes(b"Pf\n8 5\n1.0\n" + a.astype(">f4").tobytes())
    assert np.array_equal(IO.read_pfm(tmp_path / "b.pfm"), a)
    IO.write_disparity_bin(tmp_path / "d.bin", a)
    assert np.array_equal(IO.read_disparity_bin(tmp_path / "d.bin", 8, 5), a)
    with pytest.raises(ValueError):
        IO.read_disparity_bin(tmp_path / "d.bin", 9, 5)


def test_16bit_scaling_and_rmse_bookkeeping(IO, tmp_path):
    from domain_transform_solver_gb300 import cli
    v = np.array([[0, 65535], [32768, 1]], np.uint16)
    IO.write_png(tmp_path / "d.png", v)
    f = IO.read_float_16bit(tmp_path / "d.png", 1.0 / (256.0 * 256.0 - 1))
    assert f.dtype == np.float32 and f[0, 1] == np.float32(1.0) and f[0, 0] == 0
    assert cli.rms_error(np.zeros((2, 2)), np.full((2, 2), 3.0)) == 3.0
    r = cli.Result(2)
    r.add(0, 2.0, 10.0, 100)
    r.add(1, 8.0, 30.0, 300)
    assert r.line() == "RMSE 4, time 20 ms, num_pixels 200"
    assert np.array_equal(cli._to_uint8(np.array([0.5 / 255, 1.5 / 255, 2.0]), 255.0),
                          np.array([0, 2, 255], np.uint8))


def test_cli_rejects_missing_inputs(dts, capsys):
    from domain_transform_solver_gb300 import cli
    assert cli.main(["stereo"]) == -1
    assert "Invalid command line inputs." in capsys.readouterr().err


def test_bmp_and_colour_helpers(IO, tmp_path):
    from domain_transform_solver_gb300 import cli
    rng = np.random.default_rng(6)
    a = rng.integers(0, 256, (9, 11, 3)).astype(np.uint8)
    IO.write_bmp(tmp_path / "a.bmp", a)
    assert np.array_equal(IO.read_bmp(tmp_path / "a.bmp"), a)
    # YCbCr round trip of grey stays grey; truncating conversion
    g = np.full((4, 4, 3), 100, np.uint8)
    y, cb, cr = cli.bgr_to_ycbcr_planes(g)
    assert np.allclose(y, 100, atol=1e-4) and np.allclose(cb, 128, atol=1e-4)
    assert np.array_equal(cli.ycbcr_to_bgr(y, cb, cr), g)
    assert cli.ssim(a, a) == pytest.approx([1.0, 1.0, 1.0], abs=1e-6)
    assert cli.bgr_to_ycbcr_u8(g).dtype == np.uint8
