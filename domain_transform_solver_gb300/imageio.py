"""Image and raster formats of the reference's benchmark drivers, without
OpenCV: PNG (8/16-bit grey, grey+alpha, RGB, RGBA, palette; non-interlaced),
PFM and raw float32 disparity files.

The reference reads its inputs with OpenCV (src/domain_transform_image_io.h:
ReadRGBAImageFrom, ReadFloatImageFrom16bit, ReadFloatImageFromUchar), its PFM
files with src/pfm_image.cpp and its stereo initialisation as raw float32
(src/benchmark_stereo_cli.cpp: LoadTargetImage).  This module gives the same
arrays:

* ``read_rgba``: a colour PNG as RGBA uint8 with A = 0 (OpenCV loads BGR and
  the reference mixes it to RGBA; its -1 source channel fills alpha with 0);
* ``read_float_16bit(path, scale)``: a 16-bit (or 8-bit) PNG times scale;
* ``read_pfm``: a PFM image as float32 (rows in file order, as the
  reference's reader keeps them; byte order from the scale's sign);
* ``read_disparity_bin``: W*H little-endian float32 values;
* ``read_bmp`` / ``write_bmp``: uncompressed BMP (8-bit paletted, 24- and
  32-bit) as BGR uint8, the channel order OpenCV's imread gives the
  reference's colorization driver.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_PNG_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    """PNG filter types 0-4 (None, Sub, Up, Average, Paeth), row by row, in
    libdtsgb (dtsgb_png_unfilter)."""
    from ._lib import check, load
    src = np.frombuffer(raw, np.uint8)
    if src.size < h * (stride + 1):
        raise ValueError("truncated PNG image data")
    out = np.empty((h, stride), np.uint8)
    check(load().dtsgb_png_unfilter(src.ctypes.data, h, stride, bpp, out.ctypes.data))
    return out


def _unfilter_py(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    """The same in Python (tests check the library against it)."""
    out = np.zeros((h, stride), np.uint8)
    data = np.frombuffer(raw, np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(h):
        ftype = int(data[pos])
        line = data[pos + 1:pos + 1 + stride].astype(np.int32)
        pos += 1 + stride
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 0xFF
        elif ftype == 1:
            cur = line.copy()
            for i in range(bpp, stride):
                cur[i] = (cur[i] + cur[i - bpp]) & 0xFF
        elif ftype == 3:
            cur = line.copy()
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                cur[i] = (cur[i] + ((a + prev[i]) >> 1)) & 0xFF
        elif ftype == 4:
            cur = line.copy()
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[i] = (cur[i] + pred) & 0xFF
        else:
            raise ValueError(f"bad PNG filter type {ftype}")
        out[y] = cur
        prev = cur
    return out


def read_png(path) -> np.ndarray:
    """(H, W) or (H, W, C) array, uint8 or uint16 (native byte order)."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != _PNG_SIG:
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, palette = 8, [], None
    w = h = depth = ctype = interlace = None
    while pos < len(buf):
        (n,) = struct.unpack(">I", buf[pos:pos + 4])
        kind = buf[pos + 4:pos + 8]
        body = buf[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if w is None:
        raise ValueError(f"{path}: no IHDR chunk")
    if interlace:
        raise ValueError(f"{path}: interlaced PNG is not supported")
    if ctype not in _CHANNELS or depth not in (8, 16) and not (ctype == 3 and depth == 8):
        raise ValueError(f"{path}: unsupported PNG (colour type {ctype}, depth {depth})")
    ch = _CHANNELS[ctype]
    bpp = ch * depth // 8
    rows = _unfilter(zlib.decompress(b"".join(idat)), h, w * bpp, bpp)
    if depth == 16:
        img = rows.reshape(h, w * ch, 2)
        img = (img[..., 0].astype(np.uint16) << 8) | img[..., 1].astype(np.uint16)
        img = img.reshape(h, w, ch)
    else:
        img = rows.reshape(h, w, ch)
    if ctype == 3:
        if palette is None:
            raise ValueError(f"{path}: palette image without PLTE")
        img = palette[img[..., 0]]
    return img[..., 0] if img.shape[-1] == 1 else img


def write_png(path, img: np.ndarray) -> None:
    """uint8 or uint16 image, (H, W), (H, W, 3) or (H, W, 4); no filtering."""
    a = np.asarray(img)
    if a.dtype not in (np.uint8, np.uint16):
        raise ValueError("write_png wants uint8 or uint16")
    if a.ndim == 2:
        a = a[..., None]
    h, w, ch = a.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[ch]
    depth = 16 if a.dtype == np.uint16 else 8
    if depth == 16:
        rows = a.astype(">u2").reshape(h, w * ch).view(np.uint8)
    else:
        rows = a.reshape(h, w * ch)
    raw = b"".join(b"\x00" + rows[y].tobytes() for y in range(h))

    def chunk(kind, body):
        return (struct.pack(">I", len(body)) + kind + body +
                struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF))

    with open(path, "wb") as f:
        f.write(_PNG_SIG)
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def read_rgba(path) -> np.ndarray:
    """ReadRGBAImageFrom: a colour image as (H, W, 4) RGBA uint8, alpha 0
    (grey images are replicated to RGB, as OpenCV's IMREAD_COLOR does)."""
    img = read_png(path)
    if img.dtype == np.uint16:
        img = (img >> 8).astype(np.uint8)
    if img.ndim == 2:
        img = np.repeat(img[..., None], 3, axis=2)
    elif img.shape[2] == 2:
        img = np.repeat(img[..., :1], 3, axis=2)
    out = np.empty(img.shape[:2] + (4,), np.uint8)
    out[..., :3] = img[..., :3]
    out[..., 3] = 0
    return out


def read_gray(path) -> np.ndarray:
    """IMREAD_GRAYSCALE of a grey image (uint8)."""
    img = read_png(path)
    if img.ndim != 2:
        raise ValueError(f"{path}: expected a grey image")
    return (img >> 8).astype(np.uint8) if img.dtype == np.uint16 else img


def read_float_16bit(path, scale: float) -> np.ndarray:
    """ReadFloatImageFrom16bit / ReadFloatImageFromUchar: the image's integer
    values (any depth) times scale, float32."""
    img = read_png(path)
    if img.ndim != 2:
        img = img[..., 0]
    return (img.astype(np.float32) * np.float32(scale)).astype(np.float32)


def read_pfm(path) -> np.ndarray:
    """(H, W) or (H, W, 3) float32; rows in file order."""
    with open(path, "rb") as f:
        tokens = []
        while len(tokens) < 4:
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: truncated PFM header")
            tokens += line.split()
        kind, w, h, scale = tokens[0], int(tokens[1]), int(tokens[2]), float(tokens[3])
        ch = {b"Pf": 1, b"PF": 3}.get(kind)
        if ch is None:
            raise ValueError(f"{path}: not a PFM file")
        dt = np.dtype("<f4") if scale < 0 else np.dtype(">f4")
        data = np.frombuffer(f.read(4 * w * h * ch), dt)
    if data.size != w * h * ch:
        raise ValueError(f"{path}: truncated PFM data")
    img = data.astype(np.float32).reshape(h, w, ch)
    return img[..., 0] if ch == 1 else img


def write_pfm(path, img: np.ndarray) -> None:
    a = np.asarray(img, np.float32)
    ch = 1 if a.ndim == 2 else a.shape[2]
    if ch not in (1, 3):
        raise ValueError("PFM holds 1 or 3 channels")
    h, w = a.shape[:2]
    with open(path, "wb") as f:
        f.write(b"Pf\n" if ch == 1 else b"PF\n")
        f.write(f"{w} {h}\n-1\n".encode())
        f.write(a.astype("<f4").tobytes())


def read_disparity_bin(path, width: int, height: int) -> np.ndarray:
    """LoadTargetImage: width*height little-endian float32 values, row-major."""
    data = np.fromfile(path, "<f4", count=width * height)
    if data.size != width * height:
        raise ValueError(f"{path}: expected {width * height} float32 values")
    return data.astype(np.float32).reshape(height, width)


def write_disparity_bin(path, img: np.ndarray) -> None:
    np.asarray(img, "<f4").tofile(path)


def read_bmp(path) -> np.ndarray:
    """(H, W, 3) BGR uint8 of an uncompressed BMP (BI_RGB, 8/24/32 bits)."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:2] != b"BM":
        raise ValueError(f"{path}: not a BMP file")
    (off,) = struct.unpack("<I", buf[10:14])
    (hsize,) = struct.unpack("<I", buf[14:18])
    w, h = struct.unpack("<ii", buf[18:26])
    (bits,) = struct.unpack("<H", buf[28:30])
    (comp,) = struct.unpack("<I", buf[30:34])
    if comp not in (0, 3) or bits not in (8, 24, 32):
        raise ValueError(f"{path}: unsupported BMP (bits {bits}, compression {comp})")
    top_down = h < 0
    h = abs(h)
    stride = (w * bits // 8 + 3) & ~3
    rows = np.frombuffer(buf, np.uint8, count=stride * h, offset=off).reshape(h, stride)
    if bits == 8:
        (ncol,) = struct.unpack("<I", buf[46:50])
        ncol = ncol or 256
        pal = np.frombuffer(buf, np.uint8, count=4 * ncol, offset=14 + hsize).reshape(ncol, 4)
        img = pal[rows[:, :w]][..., :3]
    else:
        img = rows[:, :w * (bits // 8)].reshape(h, w, bits // 8)[..., :3]
    if not top_down:
        img = img[::-1]
    return np.ascontiguousarray(img)


def write_bmp(path, bgr: np.ndarray) -> None:
    """(H, W, 3) BGR uint8 as a 24-bit bottom-up BMP."""
    a = np.asarray(bgr, np.uint8)
    h, w = a.shape[:2]
    stride = (w * 3 + 3) & ~3
    rows = np.zeros((h, stride), np.uint8)
    rows[:, :w * 3] = a[::-1].reshape(h, w * 3)
    size = 54 + rows.size
    hdr = (b"BM" + struct.pack("<IHHI", size, 0, 0, 54) +
           struct.pack("<IiiHHIIiiII", 40, w, h, 1, 24, 0, rows.size, 2835, 2835, 0, 0))
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(rows.tobytes())
