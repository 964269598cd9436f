"""A second, independent restatement of the reference algorithms in numpy /
pure Python loops, for small images only.  It cross-checks the C oracle
(oracle/oracle.c) so that the oracle does not rest on a single transcription.

Written from the reference sources directly, in a different style from the
C oracle: global prefix sums and the literal linear window search of
src/domain_transform_filter.cuh:7-28, HFBS with explicit padded grids.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

KINV255SQ = float(np.float32(0.0000153787))  # common_kernels.cuh:10


def _fma(a: float, b: float, c: float) -> float:
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def convert_pixel(r, g, b, cs, order=1):
    """src/color_space.cuh:11-40 with nvcc's fma contraction."""
    R, G, B = float(r), float(g), float(b)
    if order == 1:
        y = _fma(0.114, B, _fma(R, 0.299, 0.587 * G))
    else:
        y = _fma(0.114, B, _fma(0.587, G, R * 0.299))
    if cs == 2:
        return (int(y),) * 3
    cb = _fma(0.5, B, _fma(-0.331264, G, _fma(-R, 0.168736, 128.0)))
    cr = _fma(-0.081312, B, _fma(-0.418688, G, _fma(R, 0.5, 128.0)))
    return int(y), int(cb), int(cr)


def differentials(guide: np.ndarray, sx, sy, sr):
    g = guide.astype(np.int64)
    px = np.zeros_like(g)
    px[:, 1:] = g[:, :-1]
    py = np.zeros_like(g)
    py[1:, :] = g[:-1, :]
    rx = float(np.float32(np.float32(sx) / np.float32(sr)))
    ry = float(np.float32(np.float32(sy) / np.float32(sr)))
    ssdx = ((g - px) ** 2).sum(-1).astype(np.float64)
    ssdy = ((g - py) ** 2).sum(-1).astype(np.float64)
    dH = np.sqrt(ssdx * KINV255SQ * rx * rx + 1.0)
    dV = np.sqrt(ssdy * KINV255SQ * ry * ry + 1.0)
    return dH, dV


def search(ct: np.ndarray, p: int, limit: int, sigma: float):
    """LinearSearchLowerAndUpperBound2DX, literally."""
    val = ct[p]
    lower = p - 1
    upper = lower + 1
    for i in range(p, -1, -1):
        if val - sigma > ct[i]:
            lower = i
            break
    for i in range(p, min(limit, len(ct))):
        if val + sigma < ct[i]:
            upper = i - 1
            break
    return lower, upper


def all_bounds(ct2d: np.ndarray, axis: int, sigma: float, limit: int):
    H, W = ct2d.shape
    L = np.zeros((H, W), np.int64)
    U = np.zeros((H, W), np.int64)
    if axis == 0:
        for y in range(H):
            for x in range(W):
                L[y, x], U[y, x] = search(ct2d[y], x, limit, sigma)
    else:
        for x in range(W):
            col = ct2d[:, x]
            for y in range(H):
                L[y, x], U[y, x] = search(col, y, limit, sigma)
    return L, U


def box(v: np.ndarray, L, U, axis: int):
    S = np.cumsum(v, axis=1 if axis == 0 else 0)
    H, W = v.shape
    out = np.empty_like(v)
    for y in range(H):
        for x in range(W):
            l, u = L[y, x], U[y, x]
            if axis == 0:
                su = S[y, u]
                sl = S[y, l] if l >= 0 else 0.0
            else:
                su = S[u, x]
                sl = S[l, x] if l >= 0 else 0.0
            out[y, x] = (su - sl) / (u - l)
    return out


def photometric(guide, right, right_dH, v, offset, photo, filt):
    """PhotometricL2LossTerm::operator() for every pixel
    (src/domain_transform_loss_term.cuh:20-39)."""
    H, W = v.shape
    sxr = np.float32(np.float32(filt["sigma_r"]) / np.float32(filt["sigma_x"]))
    alpha = float(np.float32(sxr * sxr))
    inv255 = float(np.float32(0.00392156863))
    out = np.zeros((H, W))
    for y in range(H):
        for x in range(W):
            xr = float(np.float32(offset)) + x - v[y, x]
            if 0 <= xr < W:
                xi = int(xr)
                sad = int(np.abs(guide[y, x].astype(int) - right[y, xi].astype(int)).sum())
                g = right_dH[y, xi]
                out[y, x] = float(np.float32(photo)) * 2 * (sad * inv255) * ((g * g - 1) * alpha)
    return out


def dts_solve(guide, t, c, filt, opt, overwrite=-1.0, ref_y_limit=True, stereo=None):
    """ComputeColorSpaceDifferential -> Integrate -> Optimize on a converted
    guide (H, W, 4).  stereo = (converted right guide, centre offset,
    photo_consis_lambda) adds DomainTransformStereo's photometric term."""
    H, W = t.shape
    dH, dV = differentials(guide, filt["sigma_x"], filt["sigma_y"], filt["sigma_r"])
    right_dH = None
    if stereo is not None:
        right_dH, _ = differentials(stereo[0], filt["sigma_x"], filt["sigma_y"],
                                    filt["sigma_r"])
    ctH, ctV = np.cumsum(dH, 1), np.cumsum(dV, 0)
    sz = float(np.float32(opt["sigma_z"]))
    Lx, Ux = all_bounds(ctH, 0, sz, W)
    Ly, Uy = all_bounds(ctV, 1, sz, W if ref_y_limit else H)
    t = t.astype(np.float64)
    c = c.astype(np.float64)
    v = t.copy()
    lam = float(np.float32(opt["lambda_"]))
    st = float(np.float32(opt["step_size"]))
    over = 0 < overwrite < 1
    for _ in range(opt["num_iterations"]):
        if over:
            v = np.where(c > overwrite, t, v)
        B = box(v, Lx, Ux, 0)
        n = (Ux - Lx).astype(np.float64)
        cn = c / n
        d = v - t
        if opt["loss"] == 1:
            g = 2 * cn * d
        else:
            g = cn * d / np.sqrt(d * d + 1e-6)
        if stereo is not None:
            g = g + photometric(guide, stereo[0], right_dH, v, stereo[1], stereo[2], filt)
        v = v + st * (-(lam * (v - B) + 0.5 * g))
        if over:
            v = np.where(c > overwrite, t, v)
        B = box(v, Ly, Uy, 1)
        v = v + st * (-(lam * (v - B)))
    return v


def dt_filter(guide, inp, sx, sy, sr, num_iter, ref_y_limit=True):
    H, W = inp.shape
    dH, dV = differentials(guide, sx, sy, sr)
    ctH, ctV = np.cumsum(dH, 1), np.cumsum(dV, 0)
    v = inp.astype(np.float64)
    for it in range(num_iter):
        sxi, syi = np.float32(sx), np.float32(sy)
        if it:
            m = np.float32(3 * 2.0 ** (num_iter - (it + 1)) / math.sqrt(4.0 ** num_iter - 1))
            sxi, syi = np.float32(sxi * m), np.float32(syi * m)
        L, U = all_bounds(ctH, 0, float(sxi), W)
        v = box(v, L, U, 0)
        L, U = all_bounds(ctV, 1, float(syi), W if ref_y_limit else H)
        v = box(v, L, U, 1)
    return v


# ---- HFBS ------------------------------------------------------------------
def hfbs_solve(guide, t, c, p, max_grid):
    """HFBS::Optimize (src/hfbs.cu:586-743) on explicit grids padded with the
    reference's pad planes: index 0 of each padded axis is the -1 plane
    (always 0), index g+1 the pad plane."""
    H, W = t.shape
    f32 = np.float32
    gx = int(math.ceil(f32(W) / f32(p["sigma_x"])))
    gy = int(math.ceil(f32(H) / f32(p["sigma_y"])))
    gl = int(math.ceil(255.0 / float(f32(p["sigma_l"]))))
    mgx, mgy, mgl = max_grid
    if gx > mgx or gy > mgy or gl > mgl:
        return t.astype(np.float64), None
    shp = (gl + 3, gy + 2, gx + 2)  # z has the pad plane gl and one more
    cnt = np.zeros(shp)
    csum = np.zeros(shp)
    b = np.zeros(shp)
    sxf, syf, slf = f32(p["sigma_x"]), f32(p["sigma_y"]), f32(p["sigma_l"])
    for y in range(H):
        for x in range(W):
            bx = int(np.floor(f32(x) / sxf))
            by = int(np.floor(f32(y) / syf))
            bl = int(np.floor(f32(guide[y, x, 0]) / slf))
            if bl == gl and not gl < mgl:
                continue
            cnt[bl + 1, by + 1, bx + 1] += 1
            csum[bl + 1, by + 1, bx + 1] += float(c[y, x])
            b[bl + 1, by + 1, bx + 1] += float(c[y, x]) * float(t[y, x])
    I = (slice(1, gl + 1), slice(1, gy + 1), slice(1, gx + 1))
    cov = [(g % 8 != 0) and (g < m) for g, m in ((gx, mgx), (gy, mgy), (gl, mgl))]

    def set_pads(a, value):
        # FillGrid covers the face g on an axis when g % 8 != 0 and the face
        # is inside the allocation
        if cov[0]:
            a[1:gl + 1, 1:gy + 1, gx + 1] = value
        if cov[1]:
            a[1:gl + 1, gy + 1, 1:gx + 1] = value
        if cov[2]:
            a[gl + 1, 1:gy + 1, 1:gx + 1] = value

    def nb6(a):
        return (a[1:gl + 1, 1:gy + 1, 0:gx] + a[1:gl + 1, 1:gy + 1, 2:gx + 2] +
                a[1:gl + 1, 0:gy, 1:gx + 1] + a[1:gl + 1, 2:gy + 2, 1:gx + 1] +
                a[0:gl, 1:gy + 1, 1:gx + 1] + a[2:gl + 2, 1:gy + 1, 1:gx + 1])

    scratch = np.zeros(shp)
    scratch[I] = 1.0
    set_pads(scratch, 1.0)
    norm = np.zeros(shp)
    src, dst = scratch, norm
    e = float(f32(0.00001))
    for _ in range(p["bistoch_iter_max"]):
        v = src[I]
        dst[I] = np.sqrt(v * (cnt[I] + e) / (2 * v + nb6(src) + e))
        src, dst = dst, src
    n = np.zeros(shp)
    n[I] = src[I]
    lam = float(f32(p["lambda_"]))
    diag = lam * (cnt[I] - 2 * n[I] ** 2) + csum[I]
    invA = 1.0 / np.maximum(1e-3, diag)

    def blur(a):
        beta = float(f32(p["neg_exp_beta"]))
        out = a[I].copy()
        for axis in (2, 1, 0):
            L = out.shape[axis]
            idx = np.arange(L)
            K = beta ** np.abs(idx[:, None] - idx[None, :])
            out = np.moveaxis(np.tensordot(K, np.moveaxis(out, axis, 0), axes=(1, 0)), 0, axis)
        return out

    z = np.zeros(shp)
    z[I] = blur(b) / (blur(csum) + 1e-7)
    h = np.zeros(shp)
    alpha, beta = float(f32(p["alpha"])), float(f32(p["beta"]))
    zs, zd = z, np.zeros(shp)
    for _ in range(p["optim_iter_max"]):
        q = (b[I] + lam * n[I] * nb6(zs * n)) * invA
        grad = zs[I] - q
        gc = np.where(np.abs(grad) > 1.345, np.sign(grad), grad)
        h[I] = beta * h[I] + gc
        zd[I] = zs[I] - alpha * h[I]
        zs, zd = zd, zs
    out = np.empty((H, W))
    for y in range(H):
        for x in range(W):
            fx = f32(x) / sxf
            fy = f32(y) / syf
            fz = f32(guide[y, x, 0]) / slf
            x0, y0, z0 = np.floor(fx), np.floor(fy), np.floor(fz)
            wx, wy, wz = float(fx - x0), float(fy - y0), float(fz - z0)
            num = den = 0.0
            for dz in (0, 1):
                for dy in (0, 1):
                    for dx in (0, 1):
                        ix, iy, iz = int(x0) + dx, int(y0) + dy, int(z0) + dz
                        w = ((wx if dx else 1 - wx) * (wy if dy else 1 - wy) *
                             (wz if dz else 1 - wz))
                        cc = cnt[iz + 1, iy + 1, ix + 1]
                        zz = zs[iz + 1, iy + 1, ix + 1] if iz < gl else 0.0
                        num += cc * zz * w
                        den += cc * w
            with np.errstate(invalid="ignore", divide="ignore"):  # 0/0: NaN, as the reference
                out[y, x] = num / den
    return out, dict(count=cnt[I], norm=n[I], invA=invA, z=zs[I], dims=(gx, gy, gl))
