// DTS kernels for sm_103a: guide ingest, window-bound search, the fused
// X+Y half-step iteration, the domain-transform filter pass with the
// confidence epilogue, and small helpers for downloads.
//
// Key fact used throughout: the edge weights dH, dV are >= 1
// (sqrt(1 + nonnegative)), so a window of the reference's linear search
// (src/domain_transform_filter.cuh:7-28) never reaches further than
// floor(sigma)+1 pixels from its centre.  Every pass is therefore a
// bounded-radius stencil over a tile plus halo held in shared memory: no
// global prefix sums, no transposes, no long-row cancellation.
#include "../../include/dtsgb.h"
#include "color.cuh"
#include "dtsgb_internal.cuh"

namespace dtsgb {

namespace {

constexpr int kThreads = 256;
// kINV255Sq, src/domain_transform_common_kernels.cuh:10 (a float constant).
__device__ __constant__ float c_inv255sq = (float)0.0000153787;

// dH / dV integrand of src/domain_transform_common_kernels.cuh:71-116:
// sqrt(SSD4(a-b) * kINV255Sq * r * r + 1) with r = sigma_{x|y} / sigma_r,
// evaluated in the order nvcc compiles the reference expression.
__device__ __forceinline__ float edge_weight(uchar4 a, uchar4 b, float ratio) {
  const int d0 = (int)a.x - (int)b.x, d1 = (int)a.y - (int)b.y;
  const int d2 = (int)a.z - (int)b.z, d3 = (int)a.w - (int)b.w;
  const float ssd = (float)(d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3);
  float t = __fmul_rn(ssd, c_inv255sq);
  t = __fmul_rn(t, ratio);
  return __fsqrt_rn(__fmaf_rn(t, ratio, 1.0f));
}

__global__ void k_color_convert_flat(uchar4* __restrict__ g, long long n,
                                     int cs) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    g[i] = convert_pixel(g[i], cs);
}

// ---------------------------------------------------------------------------
// Window bounds (a4).  One CTA per TWxTH tile.  Shared memory holds dH for
// the tile rows over columns [x0-rx+1, x0+TW+rx-1) and dV for the tile
// columns over rows [y0-ry+1, y0+TH+ry-1), rx = floor(sigma_x)+1.
// Lower bound: the largest i < p with sum_{j=i+1..p} w(j) > sigma, else p-1.
// Upper bound: (the smallest i > p, i < limit, with sum_{j=p+1..i} w(j) >
// sigma) - 1, else p.  limit is W for X and min(W,H) (reference quirk) or H
// for Y.  A negative ratio stands for an all-zero domain transform (no
// differential computed yet): every window is the pixel itself.
// ---------------------------------------------------------------------------
template <int TW, int TH>
__global__ void __launch_bounds__(kThreads)
    k_bounds(const Inst* __restrict__ insts, const Tile* __restrict__ tiles,
             const uchar4* __restrict__ guide, uint32_t* __restrict__ bounds,
             float ratio_x, float ratio_y, float sig_x, float sig_y, int rx,
             int ry, int ref_y_limit) {
  extern __shared__ float sm[];
  const Tile t = tiles[blockIdx.x];
  const Inst in = insts[t.inst];
  const int W = in.w, H = in.h, P = in.pitch;
  const uchar4* g = guide + in.off;
  const int DW = TW + 2 * rx - 1;
  const int DR = TH + 2 * ry - 1;
  float* sH = sm;            // TH x DW
  float* sV = sm + TH * DW;  // DR x TW
  const uchar4 zero = make_uchar4(0, 0, 0, 0);
  for (int i = threadIdx.x; i < TH * DW; i += blockDim.x) {
    const int r = i / DW, c = i - r * DW;
    const int x = t.x0 - rx + 1 + c, y = t.y0 + r;
    float w = 0.f;
    if (x >= 0 && x < W && y < H) {
      const uchar4 cur = g[(long long)y * P + x];
      const uchar4 prev = x > 0 ? g[(long long)y * P + x - 1] : zero;
      w = ratio_x < 0.f ? 0.f : edge_weight(cur, prev, ratio_x);
    }
    sH[i] = w;
  }
  for (int i = threadIdx.x; i < DR * TW; i += blockDim.x) {
    const int r = i / TW, c = i - r * TW;
    const int x = t.x0 + c, y = t.y0 - ry + 1 + r;
    float w = 0.f;
    if (x < W && y >= 0 && y < H) {
      const uchar4 cur = g[(long long)y * P + x];
      const uchar4 prev = y > 0 ? g[(long long)(y - 1) * P + x] : zero;
      w = ratio_y < 0.f ? 0.f : edge_weight(cur, prev, ratio_y);
    }
    sV[i] = w;
  }
  __syncthreads();
  const int ylim = ref_y_limit ? min(W, H) : H;
  uint32_t* bo = bounds + in.off;
  for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
    const int r = i / TW, c = i - r * TW;
    const int x = t.x0 + c, y = t.y0 + r;
    if (x >= W || y >= H) continue;
    const float* row = sH + r * DW + (c + rx - 1);  // row[0] = dH(x)
    int dlx = 1, dux = 0, dly = 1, duy = 0;
    float acc = 0.f;
    for (int k = 1; k <= rx && x - k >= 0; ++k) {
      acc += row[1 - k];
      if (acc > sig_x) {
        dlx = k;
        break;
      }
    }
    acc = 0.f;
    for (int k = 1; k <= rx && x + k < W; ++k) {
      acc += row[k];
      if (acc > sig_x) {
        dux = k - 1;
        break;
      }
    }
    const float* col = sV + (r + ry - 1) * TW + c;  // col[0] = dV(y)
    acc = 0.f;
    for (int k = 1; k <= ry && y - k >= 0; ++k) {
      acc += col[(1 - k) * TW];
      if (acc > sig_y) {
        dly = k;
        break;
      }
    }
    acc = 0.f;
    for (int k = 1; k <= ry && y + k < ylim; ++k) {
      acc += col[k * TW];
      if (acc > sig_y) {
        duy = k - 1;
        break;
      }
    }
    bo[(long long)y * P + x] = pack_bounds(dlx, dux, dly, duy);
  }
}

// ---------------------------------------------------------------------------
// One solver iteration (a6/a7): the X half-step followed by the Y half-step
// in one kernel.  A CTA owns a TWxTH output tile and stages the previous
// iterate over the tile plus a halo of floor(sigma) on all sides.  The X
// half-step is evaluated for the tile columns over the tile rows plus the
// vertical halo (those rows feed the Y windows), kept in shared memory, and
// the Y half-step writes the tile.  HBM traffic per pixel and iteration:
// read v, t, c, bounds; write v.
//   X: v' = v - s*(lambda*(v - B_x) + 0.5*g),
//      g = 2*(c/n)*(v - t) (L2) or (c/n)*(v-t)/sqrt((v-t)^2 + 1e-6)
//   Y: v' = v - s*lambda*(v - B_y)
// (src/domain_transform_solver.cuh:12-116).  With overwrite in (0,1), the
// target replaces v where c > overwrite before each half-step
// (src/domain_transform_solver.cu:126-130, 160-164).
// ---------------------------------------------------------------------------
// Window sums are direct sums over the window, first element to last, never
// a difference of running or prefix sums: a subtraction leaves an error of
// about one ulp of the larger sum, and the Charbonnier gradient
// x/sqrt(x^2+1e-6) magnifies errors in a near-zero residual about 1000-fold
// (a one-pixel window must give back the pixel exactly).  Each thread
// handles runs of kSeg consecutive pixels of a row so that the per-pixel
// inputs come in as 16-byte vector loads.
constexpr int kSeg = 8;

__device__ __forceinline__ float window_sum(const float* __restrict__ s,
                                            int stride, int lo, int hi) {
  float acc = 0.f;
  for (int k = lo; k <= hi; ++k) acc += s[k * stride];
  return acc;
}

// Eight consecutive values starting at an 8-element-aligned address; `full`
// means all eight are inside the row, otherwise only the first n are read.
__device__ __forceinline__ void load8(const float* __restrict__ p, bool full,
                                      int n, float (&o)[kSeg]) {
  if (full) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(p));
    const float4 b = __ldg(reinterpret_cast<const float4*>(p) + 1);
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
  } else {
#pragma unroll
    for (int j = 0; j < kSeg; ++j) o[j] = j < n ? __ldg(p + j) : 0.f;
  }
}
__device__ __forceinline__ void load8(const __nv_bfloat16* __restrict__ p,
                                      bool full, int n, float (&o)[kSeg]) {
  if (full) {
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
    const uint32_t w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      o[2 * j] = __uint_as_float(w[j] << 16);
      o[2 * j + 1] = __uint_as_float(w[j] & 0xffff0000u);
    }
  } else {
#pragma unroll
    for (int j = 0; j < kSeg; ++j) o[j] = j < n ? __bfloat162float(p[j]) : 0.f;
  }
}
__device__ __forceinline__ void load8(const uint32_t* __restrict__ p, bool full,
                                      int n, uint32_t (&o)[kSeg]) {
  if (full) {
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
    const uint4 b = __ldg(reinterpret_cast<const uint4*>(p) + 1);
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
  } else {
#pragma unroll
    for (int j = 0; j < kSeg; ++j) o[j] = j < n ? __ldg(p + j) : 0u;
  }
}

// X half-step update of one pixel (src/domain_transform_solver.cuh:37-86);
// rn = 1/n correctly rounded.
template <int MODE, bool STEREO = false>
__device__ __forceinline__ float x_update(float v, float B, float tv, float cv,
                                          float rn, float lambda, float step,
                                          float extra = 0.f) {
  const float cn = cv * rn;
  const float d = v - tv;
  float g;
  if (MODE == 0) {
    g = 2.f * cn * d;
  } else {
    g = __fdiv_rn(cn * d, __fsqrt_rn(__fmaf_rn(d, d, 1e-6f)));
  }
  if (STEREO) g += extra;
  return __fmaf_rn(step, -__fmaf_rn(lambda, v - B, 0.5f * g), v);
}

// PhotometricL2LossTerm::operator() (src/domain_transform_loss_term.cuh:
// 20-39) at pixel (x, y) of an image with row pitch P, for disparity d:
//   lambda_p * 2 * SAD4(left(x), right(xi)) / 255
//     * ((dH_right(xi)^2 - 1) * alpha),   xi = (int)(offset + x - d),
// zero when offset + x - d falls outside [0, W).  dH_right is the right
// image's dHdx, evaluated here from the right guide.
__device__ __forceinline__ float photometric(const StereoArgs& sa, long long row,
                                             int x, int W, float d) {
  const float xr = (sa.offset + (float)x) - d;
  if (!(xr >= 0.f && xr < (float)W)) return 0.f;
  const int xi = (int)xr;
  const uchar4 a = sa.left[row + x], b = sa.right[row + xi];
  const float sad = ((float)abs((int)a.x - (int)b.x) + (float)abs((int)a.y - (int)b.y) +
                     (float)abs((int)a.z - (int)b.z) + (float)abs((int)a.w - (int)b.w)) *
                    (float)0.00392156863;
  float gr = 0.f;
  if (sa.ratio >= 0.f)
    gr = edge_weight(b, xi > 0 ? sa.right[row + xi - 1] : make_uchar4(0, 0, 0, 0),
                     sa.ratio);
  return sa.lam_p * 2.f * sad * (__fmaf_rn(gr, gr, -1.f) * sa.alpha);
}

template <typename TS, int MODE, int TW, int TH, bool STEREO = false>
__global__ void __launch_bounds__(kThreads)
    k_dts_iter(const Inst* __restrict__ insts, const Tile* __restrict__ tiles,
               const float* __restrict__ vin, float* __restrict__ vout,
               const TS* __restrict__ tgt, const TS* __restrict__ cnf,
               const uint32_t* __restrict__ bnd, float lambda, float step,
               float overwrite, int hx, int hy, StereoArgs sa) {
  static_assert(TW % kSeg == 0 && TH % kSeg == 0, "tile must hold whole runs");
  static_assert(TW % 32 == 0, "tile width must be whole warps");
  extern __shared__ float sm[];
  const Tile t = tiles[blockIdx.x];
  const Inst in = insts[t.inst];
  const int W = in.w, H = in.h, P = in.pitch;
  const int SW = TW + 2 * hx, SR = TH + 2 * hy;
  // odd row strides: one row per lane is bank-conflict free
  const int SWp = SW | 1;
  constexpr int TXp = TW + 1;
  float* sv = sm;             // SR x SWp previous iterate (tile + halo)
  float* sx = sm + SR * SWp;  // SR x TXp after the X half-step
  const bool over = overwrite > 0.f && overwrite < 1.f;
  const int gx0 = t.x0 - hx, gy0 = t.y0 - hy;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = kThreads / 32;
  const float* vin_i = vin + in.off;
  const TS* tgt_i = tgt + in.off;
  const TS* cnf_i = cnf + in.off;
  const uint32_t* bnd_i = bnd + in.off;
  // stage the iterate: one warp per row, lanes along x (coalesced)
  for (int r = warp; r < SR; r += NW) {
    const int y = gy0 + r;
    const bool yok = y >= 0 && y < H;
    const float* src = vin_i + (long long)y * P;
    for (int c = lane; c < SW; c += 32) {
      const int x = gx0 + c;
      float v = 0.f;
      if (yok && x >= 0 && x < W) {
        v = __ldg(src + x);
        if (over && load_f(cnf_i + (long long)y * P + x) > overwrite)
          v = load_f(tgt_i + (long long)y * P + x);
      }
      sv[r * SWp + c] = v;
    }
  }
  __syncthreads();
  // X half-step: a run of kSeg pixels of one row per lane; the lanes of a
  // warp take 32 consecutive rows of the same run.
  constexpr int NSX = TW / kSeg;
  const int row_blocks = (SR + 31) >> 5;
  for (int item = warp; item < row_blocks * NSX; item += NW) {
    const int sg = item % NSX;  // constant divisor
    const int r = (item / NSX) * 32 + lane;
    const int y = gy0 + r;
    const int xs = t.x0 + sg * kSeg;
    if (r >= SR || y < 0 || y >= H || xs >= W) continue;
    const int n = min(kSeg, W - xs);
    const bool full = n == kSeg;
    const long long p = (long long)y * P + xs;
    uint32_t b[kSeg];
    float tv[kSeg], cv[kSeg];
    load8(bnd_i + p, full, n, b);
    load8(tgt_i + p, full, n, tv);
    load8(cnf_i + p, full, n, cv);
    const float* row = sv + r * SWp + hx + sg * kSeg;  // row[j] = v(xs + j)
    float* out = sx + r * TXp + sg * kSeg;
#pragma unroll
    for (int j = 0; j < kSeg; ++j) {
      if (j < n) {
        // radii clamped to the staged halo: a window never reads outside it
        const int dl = min((int)(b[j] & 0xff), hx + 1);
        const int du = min((int)((b[j] >> 8) & 0xff), hx);
        const float s = window_sum(row, 1, j + 1 - dl, j + du);
        const float rn = __frcp_rn((float)(dl + du));
        float extra = 0.f;
        if (STEREO)
          extra = photometric(sa, in.off + (long long)y * P, xs + j, W, row[j]);
        float o = x_update<MODE, STEREO>(row[j], s * rn, tv[j], cv[j], rn, lambda,
                                         step, extra);
        if (over && cv[j] > overwrite) o = tv[j];
        out[j] = o;
      }
    }
  }
  __syncthreads();
  // Y half-step: a run of kSeg rows of one column per lane; the lanes of a
  // warp take 32 consecutive columns (coalesced bounds loads and stores).
  const float slam = step * lambda;
  constexpr int NSY = TH / kSeg;
  constexpr int CB = TW / 32;
  float* vout_i = vout + in.off;
  for (int item = warp; item < CB * NSY; item += NW) {
    const int c = (item % CB) * 32 + lane;  // constant divisor
    const int sg = item / CB;
    const int x = t.x0 + c, ys = t.y0 + sg * kSeg;
    if (x >= W || ys >= H) continue;
    const int n = min(kSeg, H - ys);
    const float* col = sx + (hy + sg * kSeg) * TXp + c;  // col[j*TXp] = vx(ys + j)
    const uint32_t* bp = bnd_i + (long long)ys * P + x;
    float* op = vout_i + (long long)ys * P + x;
    for (int j = 0; j < n; ++j) {
      const uint32_t b = __ldg(bp + j * P);
      const int dl = min((int)((b >> 16) & 0xff), hy + 1), du = min((int)(b >> 24), hy);
      const float s = window_sum(col, TXp, j + 1 - dl, j + du);
      const float v = col[j * TXp];
      op[j * P] = __fmaf_rn(-slam, v - s * __frcp_rn((float)(dl + du)), v);
    }
  }
}

// ---------------------------------------------------------------------------
// Filter pass (a5): X box mean then Y box mean over NCH channels sharing the
// windows (src/domain_transform_filter.cuh:30-71).  With CONF the Y result
// is not stored; instead the confidence epilogue of
// src/domain_transform_solver.cu:21-44 is applied to (ch0, ch1) =
// (DT(t), DT(t^2)).
// ---------------------------------------------------------------------------
template <int NCH, bool CONF, typename TS, int TW, int TH>
__global__ void __launch_bounds__(kThreads)
    k_filter(const Inst* __restrict__ insts, const Tile* __restrict__ tiles,
             const float* __restrict__ in0, const float* __restrict__ in1,
             float* __restrict__ out0, float* __restrict__ out1,
             const uint32_t* __restrict__ bnd, int hx, int hy,
             TS* __restrict__ conf_out, float scale, int left_clear) {
  extern __shared__ float sm[];
  const Tile t = tiles[blockIdx.x];
  const Inst in = insts[t.inst];
  const int W = in.w, H = in.h, P = in.pitch;
  const long long off = in.off;
  const int SW = TW + 2 * hx, SR = TH + 2 * hy;
  float* sv[NCH];
  float* sx[NCH];
  for (int ch = 0; ch < NCH; ++ch) {
    sv[ch] = sm + ch * (SR * SW + SR * TW);
    sx[ch] = sv[ch] + SR * SW;
  }
  const float* src[2] = {in0, in1};
  const int gx0 = t.x0 - hx, gy0 = t.y0 - hy;
  for (int i = threadIdx.x; i < SR * SW; i += blockDim.x) {
    const int r = i / SW, c = i - r * SW;
    const int x = gx0 + c, y = gy0 + r;
    const bool ok = x >= 0 && x < W && y >= 0 && y < H;
    const long long p = off + (long long)y * P + x;
#pragma unroll
    for (int ch = 0; ch < NCH; ++ch) sv[ch][i] = ok ? __ldg(src[ch] + p) : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < SR * TW; i += blockDim.x) {
    const int r = i / TW, c = i - r * TW;
    const int x = t.x0 + c, y = gy0 + r;
    float res[NCH];
#pragma unroll
    for (int ch = 0; ch < NCH; ++ch) res[ch] = 0.f;
    if (x < W && y >= 0 && y < H) {
      const long long p = off + (long long)y * P + x;
      const uint32_t b = __ldg(bnd + p);
      // radii clamped to the staged halo: a window never reads outside it
      const int dl = min((int)(b & 0xff), hx + 1), du = min((int)((b >> 8) & 0xff), hx);
      const float nf = (float)(dl + du);
#pragma unroll
      for (int ch = 0; ch < NCH; ++ch) {
        const float* row = sv[ch] + r * SW + (c + hx);
        float s = 0.f;
        for (int k = 1 - dl; k <= du; ++k) s += row[k];
        res[ch] = __fdiv_rn(s, nf);
      }
    }
#pragma unroll
    for (int ch = 0; ch < NCH; ++ch) sx[ch][i] = res[ch];
  }
  __syncthreads();
  float* dst[2] = {out0, out1};
  for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
    const int r = i / TW, c = i - r * TW;
    const int x = t.x0 + c, y = t.y0 + r;
    if (x >= W || y >= H) continue;
    const long long p = off + (long long)y * P + x;
    const uint32_t b = __ldg(bnd + p);
    const int dl = min((int)((b >> 16) & 0xff), hy + 1), du = min((int)(b >> 24), hy);
    const float nf = (float)(dl + du);
    float res[NCH];
#pragma unroll
    for (int ch = 0; ch < NCH; ++ch) {
      const float* col = sx[ch] + (r + hy) * TW + c;
      float s = 0.f;
      for (int k = 1 - dl; k <= du; ++k) s += col[k * TW];
      res[ch] = __fdiv_rn(s, nf);
    }
    if (CONF) {
      float cv = 0.f;
      if (x > left_clear) {
        const float var = res[1] - res[0] * res[0];
        cv = (var < 0.f || !isfinite(var)) ? 0.f : expf(-var * scale);
      }
      conf_out[p] = store_cast<TS>(cv);
      // keep DT(t^2) as the filter's last result (the reference leaves it in
      // its var buffer)
      dst[1][p] = res[1];
      dst[0][p] = res[0];
    } else {
#pragma unroll
      for (int ch = 0; ch < NCH; ++ch) dst[ch][p] = res[ch];
    }
  }
}

template <typename TS>
__global__ void k_to_float(const Inst* __restrict__ insts, int n_inst,
                           const TS* __restrict__ src, float* __restrict__ dst,
                           float* __restrict__ dst_sq) {
  const Inst in = insts[blockIdx.y];
  const long long n = (long long)in.pitch * in.h;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = load_f(src + in.off + i);
    dst[in.off + i] = v;
    if (dst_sq) dst_sq[in.off + i] = v * v;
  }
}

template <typename TS>
__global__ void k_from_float(const float* __restrict__ src, TS* __restrict__ dst,
                             long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = store_cast<TS>(src[i]);
}

template <typename TS>
__global__ void k_fill(TS* __restrict__ dst, long long n, float v) {
  const TS val = store_cast<TS>(v);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = val;
}

__global__ void k_differential(const Inst* __restrict__ insts,
                               const uchar4* __restrict__ guide, float ratio,
                               int axis, float* __restrict__ out) {
  const Inst in = insts[blockIdx.y];
  const long long n = (long long)in.w * in.h;
  const uchar4 zero = make_uchar4(0, 0, 0, 0);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / in.w), x = (int)(i - (long long)y * in.w);
    const long long p = in.off + (long long)y * in.pitch + x;
    const uchar4 cur = guide[p];
    uchar4 prev = zero;
    if (axis == 0 && x > 0) prev = guide[p - 1];
    if (axis == 1 && y > 0) prev = guide[p - in.pitch];
    out[p] = edge_weight(cur, prev, ratio);
  }
}

// Row-wise inclusive prefix sum, one warp per row, Kahan-compensated carry
// between 32-element chunks.
__global__ void k_row_prefix(const Inst* __restrict__ insts,
                             const float* __restrict__ in,
                             float* __restrict__ out) {
  const Inst I = insts[blockIdx.y];
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= I.h) return;
  const float* src = in + I.off + (long long)warp * I.pitch;
  float* dst = out + I.off + (long long)warp * I.pitch;
  float carry = 0.f, comp = 0.f;
  for (int x0 = 0; x0 < I.w; x0 += 32) {
    const int x = x0 + lane;
    float v = x < I.w ? src[x] : 0.f;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float n = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += n;
    }
    if (x < I.w) dst[x] = carry + v;
    const float total = __shfl_sync(0xffffffffu, v, 31);
    const float yk = total - comp;
    const float tk = carry + yk;
    comp = (tk - carry) - yk;
    carry = tk;
  }
}

__global__ void k_unpack_bounds(const Inst* __restrict__ insts,
                                const uint32_t* __restrict__ bnd, int axis,
                                int32_t* __restrict__ l, int32_t* __restrict__ u) {
  const Inst in = insts[blockIdx.y];
  const long long n = (long long)in.w * in.h;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / in.w), x = (int)(i - (long long)y * in.w);
    const uint32_t b = bnd[in.off + (long long)y * in.pitch + x];
    const int pos = axis == 0 ? x : y;
    const int dl = axis == 0 ? (b & 0xff) : ((b >> 16) & 0xff);
    const int du = axis == 0 ? ((b >> 8) & 0xff) : (b >> 24);
    l[i] = pos - dl;
    u[i] = pos + du;
  }
}

int grid_for(long long n, int threads = kThreads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int)b;
}

template <typename F>
int set_smem(F* f, size_t bytes) {
  if (bytes > 48 * 1024) {
    DTSGB_CUDA(cudaFuncSetAttribute(
        f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  }
  return DTSGB_OK;
}

constexpr size_t kMaxSmem = 227 * 1024;

}  // namespace

int launch_color_convert_flat(uchar4* guide, long long n, int color_space,
                              cudaStream_t s) {
  if (color_space == DTSGB_RGB || n <= 0) return DTSGB_OK;
  k_color_convert_flat<<<grid_for(n), kThreads, 0, s>>>(guide, n, color_space);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

int launch_bounds(const DtsLaunch& L, const uchar4* guide, uint32_t* bounds,
                  float ratio_x, float ratio_y, float sigma_x, float sigma_y,
                  int ref_y_limit, cudaStream_t s) {
  const int rx = (int)floorf(sigma_x) + 1, ry = (int)floorf(sigma_y) + 1;
  if (rx > 255 || ry > 255)
    return fail(DTSGB_ERR_UNSUPPORTED, "sigma >= 255 is not supported");
  const int TW = kBoundsTW, TH = kBoundsTH;
  const size_t smem =
      sizeof(float) * ((size_t)TH * (TW + 2 * rx - 1) + (size_t)(TH + 2 * ry - 1) * TW);
  if (smem > kMaxSmem) return fail(DTSGB_ERR_UNSUPPORTED, "sigma too large");
  int st = set_smem(k_bounds<TW, TH>, smem);
  if (st) return st;
  ProfScope ps(s, DTSGB_K_BOUNDS);
  k_bounds<TW, TH><<<L.n_tiles, kThreads, smem, s>>>(
      L.d_inst, L.d_tiles, guide, bounds, ratio_x, ratio_y, sigma_x, sigma_y,
      rx, ry, ref_y_limit);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

template <typename TS, int MODE, int TW, int TH, bool STEREO>
static int launch_iter_shape(const DtsLaunch& L, const float* vin, float* vout,
                             const void* target, const void* conf,
                             const uint32_t* bounds, float lambda, float step,
                             float overwrite, int hx, int hy, cudaStream_t s,
                             const StereoArgs& sa) {
  const size_t smem = sizeof(float) * ((size_t)(TH + 2 * hy) * ((TW + 2 * hx) | 1) +
                                       (size_t)(TH + 2 * hy) * (TW + 1));
  if (smem > kMaxSmem) return fail(DTSGB_ERR_UNSUPPORTED, "sigma_z too large");
  int st = set_smem(k_dts_iter<TS, MODE, TW, TH, STEREO>, smem);
  if (st) return st;
  ProfScope ps(s, DTSGB_K_DTS_ITER);
  k_dts_iter<TS, MODE, TW, TH, STEREO><<<L.n_tiles, kThreads, smem, s>>>(
      L.d_inst, L.d_tiles, vin, vout, (const TS*)target, (const TS*)conf,
      bounds, lambda, step, overwrite, hx, hy, sa);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

template <typename TS, int MODE, bool STEREO>
static int launch_iter_t(const DtsLaunch& L, const float* vin, float* vout,
                         const void* target, const void* conf,
                         const uint32_t* bounds, float lambda, float step,
                         float overwrite, int hx, int hy, cudaStream_t s,
                         const StereoArgs& sa) {
  if (L.small)
    return launch_iter_shape<TS, MODE, kIterSmallTW, kIterSmallTH, STEREO>(
        L, vin, vout, target, conf, bounds, lambda, step, overwrite, hx, hy, s, sa);
  return launch_iter_shape<TS, MODE, kIterTW, kIterTH, STEREO>(
      L, vin, vout, target, conf, bounds, lambda, step, overwrite, hx, hy, s, sa);
}

template <typename TS, bool STEREO>
static int launch_iter_mode(const DtsLaunch& L, IterMode mode, const float* vin,
                            float* vout, const void* target, const void* conf,
                            const uint32_t* bounds, float lambda, float step,
                            float overwrite, int hx, int hy, cudaStream_t s,
                            const StereoArgs& sa) {
  if (mode == IterMode::L2)
    return launch_iter_t<TS, 0, STEREO>(L, vin, vout, target, conf, bounds, lambda,
                                        step, overwrite, hx, hy, s, sa);
  return launch_iter_t<TS, 1, STEREO>(L, vin, vout, target, conf, bounds, lambda,
                                      step, overwrite, hx, hy, s, sa);
}

int launch_dts_iter(const DtsLaunch& L, Storage st, IterMode mode,
                    const float* vin, float* vout, const void* target,
                    const void* conf, const uint32_t* bounds, float lambda,
                    float step, float overwrite, int hx, int hy,
                    cudaStream_t s, const StereoArgs* stereo) {
  const StereoArgs none{nullptr, nullptr, 0.f, 0.f, 0.f, -1.f};
  if (st == Storage::F32) {
    if (stereo)
      return launch_iter_mode<float, true>(L, mode, vin, vout, target, conf, bounds,
                                           lambda, step, overwrite, hx, hy, s, *stereo);
    return launch_iter_mode<float, false>(L, mode, vin, vout, target, conf, bounds,
                                          lambda, step, overwrite, hx, hy, s, none);
  }
  if (stereo)
    return launch_iter_mode<__nv_bfloat16, true>(L, mode, vin, vout, target, conf,
                                                 bounds, lambda, step, overwrite, hx,
                                                 hy, s, *stereo);
  return launch_iter_mode<__nv_bfloat16, false>(L, mode, vin, vout, target, conf,
                                                bounds, lambda, step, overwrite, hx,
                                                hy, s, none);
}

int launch_target_to_float(const DtsLaunch& L, Storage st, const void* src,
                           float* dst, float* dst_sq, cudaStream_t s) {
  dim3 grid(64, L.n_inst);
  ProfScope ps(s, DTSGB_K_DTS_OTHER);
  if (st == Storage::F32)
    k_to_float<float><<<grid, kThreads, 0, s>>>(L.d_inst, L.n_inst,
                                                 (const float*)src, dst, dst_sq);
  else
    k_to_float<__nv_bfloat16><<<grid, kThreads, 0, s>>>(
        L.d_inst, L.n_inst, (const __nv_bfloat16*)src, dst, dst_sq);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

int launch_init_var(const DtsLaunch& L, Storage st, const void* target,
                    float* v, cudaStream_t s) {
  return launch_target_to_float(L, st, target, v, nullptr, s);
}

int launch_storage_from_float(const Inst*, int, Storage st, const float* src,
                              void* dst, long long n, cudaStream_t s) {
  if (st == Storage::F32) {
    DTSGB_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(float),
                               cudaMemcpyDeviceToDevice, s));
    return DTSGB_OK;
  }
  k_from_float<__nv_bfloat16><<<grid_for(n), kThreads, 0, s>>>(
      src, (__nv_bfloat16*)dst, n);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

int launch_fill_storage(Storage st, void* dst, long long n, float value,
                        cudaStream_t s) {
  if (st == Storage::F32)
    k_fill<float><<<grid_for(n), kThreads, 0, s>>>((float*)dst, n, value);
  else
    k_fill<__nv_bfloat16><<<grid_for(n), kThreads, 0, s>>>(
        (__nv_bfloat16*)dst, n, value);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

template <int NCH, bool CONF, typename TS, int TW, int TH>
static int launch_filter_shape(const DtsLaunch& L, const float* in0,
                               const float* in1, float* out0, float* out1,
                               const uint32_t* bounds, int hx, int hy,
                               void* conf_out, float scale, int left_clear,
                               cudaStream_t s) {
  const size_t smem = NCH * sizeof(float) *
                      ((size_t)(TH + 2 * hy) * (TW + 2 * hx) + (size_t)(TH + 2 * hy) * TW);
  if (smem > kMaxSmem) return fail(DTSGB_ERR_UNSUPPORTED, "filter sigma too large");
  int st = set_smem(k_filter<NCH, CONF, TS, TW, TH>, smem);
  if (st) return st;
  ProfScope ps(s, DTSGB_K_FILTER);
  k_filter<NCH, CONF, TS, TW, TH><<<L.n_tiles, kThreads, smem, s>>>(
      L.d_inst, L.d_tiles, in0, in1, out0, out1, bounds, hx, hy, (TS*)conf_out,
      scale, left_clear);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

template <int NCH, bool CONF, typename TS>
static int launch_filter_t(const DtsLaunch& L, const float* in0,
                           const float* in1, float* out0, float* out1,
                           const uint32_t* bounds, int hx, int hy,
                           void* conf_out, float scale, int left_clear,
                           cudaStream_t s) {
  if (L.small)
    return launch_filter_shape<NCH, CONF, TS, kIterSmallTW, kIterSmallTH>(
        L, in0, in1, out0, out1, bounds, hx, hy, conf_out, scale, left_clear, s);
  return launch_filter_shape<NCH, CONF, TS, kIterTW, kIterTH>(
      L, in0, in1, out0, out1, bounds, hx, hy, conf_out, scale, left_clear, s);
}

int launch_filter_pass(const DtsLaunch& L, int nch, const float* in0,
                       const float* in1, float* out0, float* out1,
                       const uint32_t* bounds, int hx, int hy, Storage st,
                       void* conf_out, float scale, int left_clear,
                       cudaStream_t s) {
  if (conf_out) {
    if (st == Storage::F32)
      return launch_filter_t<2, true, float>(L, in0, in1, out0, out1, bounds, hx,
                                             hy, conf_out, scale, left_clear, s);
    return launch_filter_t<2, true, __nv_bfloat16>(L, in0, in1, out0, out1,
                                                   bounds, hx, hy, conf_out,
                                                   scale, left_clear, s);
  }
  if (nch == 2)
    return launch_filter_t<2, false, float>(L, in0, in1, out0, out1, bounds, hx,
                                            hy, nullptr, 0.f, 0, s);
  return launch_filter_t<1, false, float>(L, in0, nullptr, out0, nullptr, bounds,
                                          hx, hy, nullptr, 0.f, 0, s);
}

int launch_differential(const DtsLaunch& L, const uchar4* guide, float ratio,
                        int axis, float* out, cudaStream_t s) {
  k_differential<<<dim3(64, L.n_inst), kThreads, 0, s>>>(L.d_inst, guide, ratio,
                                                         axis, out);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

int launch_row_prefix(const Inst* h_inst, const Inst* d_inst, int n_inst,
                      const float* in, float* out, cudaStream_t s) {
  int max_h = 1;
  for (int i = 0; i < n_inst; ++i) max_h = max_h > h_inst[i].h ? max_h : h_inst[i].h;
  const int warps_per_block = kThreads / 32;
  dim3 grid((max_h + warps_per_block - 1) / warps_per_block, n_inst);
  k_row_prefix<<<grid, kThreads, 0, s>>>(d_inst, in, out);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

int launch_unpack_bounds(const DtsLaunch& L, const uint32_t* bounds, int axis,
                         int32_t* l, int32_t* u, cudaStream_t s) {
  k_unpack_bounds<<<dim3(64, L.n_inst), kThreads, 0, s>>>(L.d_inst, bounds, axis,
                                                          l, u);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

}  // namespace dtsgb
