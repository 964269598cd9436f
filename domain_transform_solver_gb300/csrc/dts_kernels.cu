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
#include <algorithm>
#include <cmath>

#include "../../include/dtsgb.h"
#include "color.cuh"
#include "dtsgb_internal.cuh"
#include "fixed_point.cuh"
#include "tma.cuh"

namespace dtsgb {

namespace {

constexpr int kThreads = 256;

// CTAs of this file's kernels that gave up waiting for their TMA staging.
__device__ unsigned long long g_wait_timeouts = 0;

__global__ void k_color_convert_flat(uchar4* __restrict__ g, long long n,
                                     int cs) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    g[i] = convert_pixel(g[i], cs);
}

// ---------------------------------------------------------------------------
// Window bounds (a4).  One CTA per TWxTH tile, 256 threads.
// Lower bound: the largest i < p with sum_{j=i+1..p} w(j) > sigma, else p-1.
// Upper bound: (the smallest i > p, i < limit, with sum_{j=p+1..i} w(j) >
// sigma) - 1, else p.  limit is W for X and min(W,H) (reference quirk) or H
// for Y.  A negative ratio stands for an all-zero domain transform (no
// differential computed yet): every window is the pixel itself.
//
// The weights are clamped to sigma + 1 (a window holding a larger one
// exceeds sigma either way) and converted to fixed point at 2^F with
// r * (sigma + 1) * 2^F <= 2^30, so a window sum is the exact difference of
// two wrapping 32-bit prefixes of the converted weights (each within 2^-F-1
// of the float weight: decisions differ from float sums only within about
// r * 2^-F of the threshold).  Shared memory holds the prefix of dH along
// each tile row over [x0 - r, x0 + TW + r) and of dV along each tile column
// over [y0 - r, y0 + TH + r).  As p moves forward, both window ends move
// forward, so a thread walks a segment of 8 pixels with two pointers that
// only advance: about two prefix reads per end and pixel instead of a search
// over the whole radius.
// ---------------------------------------------------------------------------
// Pixels per thread and axis of the two-pointer walks (a launch knob:
// DTSGB_TUNE_BOUNDS_SEGMENT selects 4, 8 or 16).
constexpr int kBoundsSegDefault = 8;

// Lower and upper window ends along one axis for the n pixels starting at
// prefix index j0 (S[j0 + k] for pixel p0 + k), coordinates p0.., axis length
// `len` (lower limit 0), upper limit `lim`; stride between prefix entries s.
// Writes dl | du << 8 to out[k * os].
__device__ __forceinline__ void bounds_walk(const unsigned* __restrict__ S, int s, int j0,
                                            int p0, int n, int r, int lim, int T,
                                            uint16_t* out, int os) {
  int q = 0, u = 0;
  for (int k = 0; k < n; ++k) {
    const int j = j0 + k, p = p0 + k;
    const unsigned Sj = S[j * s];
    // lower: the largest q in [j - K, j - 1] with S[j] - S[q] > T (K = min(r, p)),
    // advanced from the previous pixel's (both only move forward)
    const int qmin = j - min(r, p);
    q = k == 0 ? qmin - 1 : max(q, qmin - 1);
    while (q + 1 <= j - 1 && (int)(Sj - S[(q + 1) * s]) > T) ++q;
    const int dl = q >= qmin ? j - q : 1;
    // upper: the smallest u in [j + 1, j + K'] with S[u] - S[j] > T
    // (K' = min(r, lim - 1 - p)); the first pixel starts from the far end
    const int umax = j + min(r, lim - 1 - p);
    if (k == 0) {
      u = umax + 1;
      while (u - 1 > j && (int)(S[(u - 1) * s] - Sj) > T) --u;
    } else {
      u = max(u, j + 1);
      while (u <= umax && (int)(S[u * s] - Sj) <= T) ++u;
    }
    const int du = u <= umax ? u - j - 1 : 0;
    out[k * os] = (uint16_t)(dl | (du << 8));
  }
}

template <int TW, int TH, int SEG>
__global__ void __launch_bounds__(kThreads)
    k_bounds(const Inst* __restrict__ insts, const Tile* __restrict__ tiles,
             const uchar4* __restrict__ guide, uint32_t* __restrict__ bounds,
             float ratio_x, float ratio_y, int rx, int ry, int ref_y_limit,
             float cap_x, float cap_y, float scale_x, float scale_y, int Tx, int Ty) {
  static_assert(TW == 32 && TH == 32 && kThreads == 256, "bounds tile shape");
  static_assert(SEG == 4 || SEG == 8 || SEG == 16, "walk segment");
  constexpr int NW = kThreads / 32;
  extern __shared__ unsigned smu[];
  const Tile t = tiles[blockIdx.x];
  const Inst in = insts[t.inst];
  const int W = in.w, H = in.h, P = in.pitch;
  const uchar4* g = guide + in.off;
  const int DW = TW + 2 * rx, DWp = DW | 1;  // odd row stride: lanes on rows
  const int DR = TH + 2 * ry;
  unsigned* SH = smu;             // TH x DWp: prefix of dH, entry 0 = 0 at x0 - rx
  unsigned* SV = SH + TH * DWp;   // DR x TW: prefix of dV, entry 0 = 0 at y0 - ry
  uint16_t* BX = reinterpret_cast<uint16_t*>(SV + DR * TW);  // TH x TW
  uint16_t* BY = BX + TH * TW;                               // TH x TW
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // ---- 1. weights in fixed point.  dH: a warp per row, lanes on columns; a
  // lane's left neighbour comes from the lane before it (one load per pixel).
  // dV: eight threads per column, each down a run of rows, the pixel above
  // carried in a register.  Pixels outside the image read as zero.
  auto load_g = [&](int x, int y) -> unsigned {
    return (x >= 0 && x < W && y >= 0 && y < H)
               ? *reinterpret_cast<const unsigned*>(g + (long long)y * P + x)
               : 0u;
  };
  auto as_px = [](unsigned v) { return *reinterpret_cast<const uchar4*>(&v); };
  for (int r = warp; r < TH; r += NW) {
    const int y = t.y0 + r;
    for (int j0 = 0; j0 < DW; j0 += 32) {
      const int j = j0 + lane, x = t.x0 - rx + j;
      const unsigned cur = j < DW ? load_g(x, y) : 0u;
      unsigned prev = __shfl_up_sync(0xffffffffu, cur, 1);
      if (lane == 0) prev = load_g(x - 1, y);
      unsigned q = 0u;
      if (j > 0 && x >= 0 && x < W && y < H && ratio_x >= 0.f)
        q = (unsigned)__float2int_rn(
            fminf(edge_weight(as_px(cur), as_px(prev), ratio_x), cap_x) * scale_x);
      if (j < DW) SH[r * DWp + j] = q;
    }
  }
  {
    const int c = tid % TW, sgi = tid / TW, nsg = kThreads / TW;
    const int seg = (DR + nsg - 1) / nsg;
    const int j0 = sgi * seg, j1 = min(DR, j0 + seg);
    const int x = t.x0 + c;
    unsigned prev = load_g(x, t.y0 - ry + j0 - 1);
    for (int j = j0; j < j1; ++j) {
      const int y = t.y0 - ry + j;
      const unsigned cur = load_g(x, y);
      unsigned q = 0u;
      if (j > 0 && x < W && y >= 0 && y < H && ratio_y >= 0.f)
        q = (unsigned)__float2int_rn(
            fminf(edge_weight(as_px(cur), as_px(prev), ratio_y), cap_y) * scale_y);
      SV[j * TW + c] = q;
      prev = cur;
    }
  }
  __syncthreads();
  // ---- 2. inclusive prefixes: a thread per row of SH, a thread per column of SV
  // (a segmented scan over all warps was slower: its extra pass costs more
  // issue slots than the serial chains, which the other resident blocks hide)
  if (tid < TH) {
    unsigned* row = SH + tid * DWp;
    unsigned acc = 0u;
    for (int j = 0; j < DW; ++j) row[j] = acc += row[j];
  } else if (tid >= 32 && tid < 32 + TW) {
    unsigned* col = SV + (tid - 32);
    unsigned acc = 0u;
    for (int j = 0; j < DR; ++j) col[j * TW] = acc += col[j * TW];
  }
  __syncthreads();
  // ---- 3. two-pointer walks: warps 0-3 rows (X), warps 4-7 columns (Y), each
  // taking the SEG-pixel segments sg = warp, warp + 4, ... of its lines
  const int ylim = ref_y_limit ? min(W, H) : H;
  constexpr int NSEG = TW / SEG;
  if (tid < 4 * 32) {
    const int r = lane, y = t.y0 + r;  // lanes on rows
    for (int sg = warp; sg < NSEG; sg += 4) {
      const int xs = t.x0 + sg * SEG;
      const int n = min(SEG, W - xs);
      if (y < H && n > 0)
        bounds_walk(SH + r * DWp, 1, xs - t.x0 + rx, xs, n, rx, W, Tx,
                    BX + r * TW + sg * SEG, 1);
    }
  } else {
    const int c = lane, x = t.x0 + c;  // lanes on columns
    for (int sg = warp - 4; sg < NSEG; sg += 4) {
      const int ys = t.y0 + sg * SEG;
      const int n = min(SEG, H - ys);
      if (x < W && n > 0)
        bounds_walk(SV + c, TW, ys - t.y0 + ry, ys, n, ry, ylim, Ty, BY + sg * SEG * TW + c,
                    TW);
    }
  }
  __syncthreads();
  // ---- 4. packed bounds, rows written coalesced
  uint32_t* bo = bounds + in.off;
  for (int i = tid; i < TH * TW; i += kThreads) {
    const int r = i / TW, c = i % TW;
    const int x = t.x0 + c, y = t.y0 + r;
    if (x < W && y < H) bo[y * P + x] = (uint32_t)BX[i] | ((uint32_t)BY[i] << 16);
  }
}

// ---------------------------------------------------------------------------
// One solver iteration (a6/a7): the X half-step followed by the Y half-step
// in one kernel (k_dts_iter_vec below).  A CTA owns a TWxTH output tile;
// the X half-step is evaluated for the tile columns over the tile rows plus
// a vertical halo of floor(sigma) (those rows feed the Y windows), kept in
// shared memory, and the Y half-step writes the tile.  HBM traffic per pixel
// and iteration: read v, t, c, bounds; write v.
//   X: v' = v - s*(lambda*(v - B_x) + 0.5*g),
//      g = 2*(c/n)*(v - t) (L2) or (c/n)*(v-t)/sqrt((v-t)^2 + 1e-6)
//   Y: v' = v - s*lambda*(v - B_y)
// (src/domain_transform_solver.cuh:12-116).  With overwrite in (0,1), the
// target replaces v where c > overwrite before each half-step
// (src/domain_transform_solver.cu:126-130, 160-164).
// ---------------------------------------------------------------------------

// X half-step update of one pixel (src/domain_transform_solver.cuh:37-86);
// rn = 1/n correctly rounded.
template <int MODE, bool STEREO = false>
__device__ __forceinline__ float x_update(float v, float B, float tv, float cv,
                                          float rn, float lambda, float step,
                                          float extra = 0.f) {
  const float cn = cv * rn;
  const float d = v - tv;
  // L2: 0.5 * (2 (c/n) d) is (c/n) d exactly (scaling by 2 is exact)
  if (MODE == 0 && !STEREO) return __fmaf_rn(step, -__fmaf_rn(lambda, v - B, cn * d), v);
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

// v = t where c > overwrite, in place (DomainTransformSolver::Optimize's
// overwrite before the X half-step, src/domain_transform_solver.cu:126-130).
template <typename TS>
__global__ void k_overwrite(const Inst* __restrict__ insts, float* __restrict__ v,
                            const TS* __restrict__ tgt, const TS* __restrict__ cnf,
                            float overwrite) {
  const Inst in = insts[blockIdx.y];
  const long long n = (long long)in.pitch * in.h;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    if (load_f(cnf + in.off + i) > overwrite) v[in.off + i] = load_f(tgt + in.off + i);
}

// ---------------------------------------------------------------------------
// The fused X+Y iteration with four adjacent pixels per thread
// (k_dts_iter_vec): every global access is a 16-byte (f32) or 8-byte (bf16)
// vector.  Tiles start at
// multiples of 4 pixels and planes at multiples of 32 elements with a pitch
// of a multiple of 32, so every group of four is aligned and lies inside
// its row's pitch.  Phases of one CTA (TW x TH tile, halos hx, hy; SR = TH +
// 2hy rows):
//  1. stage the iterate over SR rows x SW columns, from HA >= hx + 1
//     columns left of the tile (SW and HA multiples of 4), and reduce its
//     largest magnitude (the X scale).  With a tensor-map table the whole
//     box arrives by one TMA load (cp.async.bulk.tensor; zeros past the
//     image) while the threads fetch their first X-step operands; without
//     one, by 16-byte loads;
//  2. the rows are converted to fixed point and scanned: a thread per
//     16-entry segment, then the segment offsets are added;
//  3. X half-step for the tile columns over all SR rows, four pixels per
//     thread, the next group's loads in flight while one is computed;
//     results and the Y bounds kept in shared memory with their largest
//     magnitude (the Y scale);
//  4. Y prefix: one warp per group of four columns, one lane per segment of
//     rows, segment offsets from a warp scan;
//  5. Y half-step for the tile, four pixels per thread, vector stores.
// ---------------------------------------------------------------------------
// i / d for 0 <= i < 2^16 and 2 <= d < 2^16 with m = ceil(2^32 / d): the
// error term i * (m * d - 2^32) / (d * 2^32) stays below 1 / d.
__host__ __forceinline__ unsigned fast_div_magic(unsigned d) {
  return (unsigned)((0x100000000ull + d - 1) / d);
}
__device__ __forceinline__ int fast_div(int i, unsigned m) {
  return (int)__umulhi((unsigned)i, m);
}

template <int TW, int TH, int NT>
struct VecIterSmem {
  int ha, sw, sws, sr, nsx, seg, sx_off, sby_off, rt_off, ry_off, mx_off, total;
  unsigned sw4_magic, sr_magic;  // fast_div_magic(sw / 4), fast_div_magic(sr)
  __host__ VecIterSmem(int hx, int hy) {
    constexpr int TQ = TW + 4;  // sx / Py row stride: 16 bytes mod 128
    ha = (hx + 4) & ~3;
    sw = ha + TW + ((hx + 3) & ~3);
    // X row stride: an odd number of 16-byte chunks, so that 8 consecutive
    // rows start in 8 different chunks of the banks
    sws = ((sw >> 2) & 1) ? sw : sw + 4;
    nsx = (sw + 15) / 16;  // 16-entry scan segments per row
    sr = TH + 2 * hy;
    // rows per lane in the Y scan; odd, so that the 32 lanes' rows spread
    // over all banks
    seg = ((sr + 1 + 31) / 32) | 1;
    sx_off = max(sr * sws, (sr + 1) * TQ) * 4;  // X prefix, later the Y prefix
    sby_off = sx_off + sr * TQ * 4;
    rt_off = sby_off + sr * TW * 2;  // (1/n, 1/n 2^-F) for X
    const int nrt = 2 * max(hx, hy) + 2;
    ry_off = rt_off + (nrt * 8 + 15) / 16 * 16;  // 1/n 2^-Fy for Y
    mx_off = ry_off + (nrt * 4 + 15) / 16 * 16;
    total = mx_off + 16;
    sw4_magic = fast_div_magic((unsigned)(sw >> 2));
    sr_magic = fast_div_magic((unsigned)sr);
  }
};

// Four consecutive storage values, kept packed until they are used.
template <typename TS>
struct Raw4;
template <>
struct Raw4<float> {
  float4 v;
  __device__ __forceinline__ void load(const float* p) {
    v = __ldg(reinterpret_cast<const float4*>(p));
  }
  __device__ __forceinline__ void zero() { v = make_float4(0.f, 0.f, 0.f, 0.f); }
  __device__ __forceinline__ float operator[](int k) const {
    return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
  }
};
template <>
struct Raw4<__nv_bfloat16> {
  uint2 v;
  __device__ __forceinline__ void load(const __nv_bfloat16* p) {
    v = __ldg(reinterpret_cast<const uint2*>(p));
  }
  __device__ __forceinline__ void zero() { v = make_uint2(0u, 0u); }
  // bf16 -> f32 is exact: the 16 bits become the high half
  __device__ __forceinline__ float operator[](int k) const {
    const unsigned w = k < 2 ? v.x : v.y;
    return __uint_as_float((k & 1) ? (w & 0xffff0000u) : (w << 16));
  }
};

__device__ __forceinline__ float f4_get(const float4& v, int k) {
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}
__device__ __forceinline__ unsigned u4_get(const uint4& v, int k) {
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

template <typename TS, int MODE, int TW, int TH, int NT, bool STEREO = false>
__global__ void __launch_bounds__(NT, 1024 / NT)
    k_dts_iter_vec(const Inst* __restrict__ insts, const Tile* __restrict__ tiles,
                   const float* __restrict__ vin, float* __restrict__ vout,
                   const TS* __restrict__ tgt, const TS* __restrict__ cnf,
                   const uint32_t* __restrict__ bnd, float lambda, float step,
                   float overwrite, int hx, int hy, StereoArgs sa, VecIterSmem<TW, TH, NT> L,
                   const CUtensorMap* __restrict__ tmaps) {
  constexpr int QW = TW / 4, TQ = TW + 4, RPP = NT / QW, NW = NT / 32;
  static_assert(TW % 32 == 0 && NT % TW == 0 && NW >= QW, "tile shape");
  pdl_wait_then_release();  // launched as a dependent of the previous iteration
  extern __shared__ __align__(128) unsigned char smraw[];
  const Tile t = tiles[blockIdx.x];
  const Inst in = insts[t.inst];
  const int W = in.w, H = in.h, P = in.pitch;
  const float* vin_i = vin + in.off;
  float* vout_i = vout + in.off;
  const TS* tgt_i = tgt + in.off;
  const TS* cnf_i = cnf + in.off;
  const uint32_t* bnd_i = bnd + in.off;
  const int SR = L.sr, SW = L.sw, SWS = L.sws, HA = L.ha;
  float* Xf = reinterpret_cast<float*>(smraw);          // SR x SWS: iterate, then
  unsigned* XP = reinterpret_cast<unsigned*>(smraw);    // its X prefix
  unsigned* Py = XP;                                    // (SR + 1) x TQ, phase 4
  float* sx = reinterpret_cast<float*>(smraw + L.sx_off);          // SR x TQ
  uint16_t* sby = reinterpret_cast<uint16_t*>(smraw + L.sby_off);  // SR x TW
  float2* rtx = reinterpret_cast<float2*>(smraw + L.rt_off);  // (1/n, 1/n 2^-F)
  float* rsy = reinterpret_cast<float*>(smraw + L.ry_off);     // 1/n 2^-Fy
  unsigned* smax = reinterpret_cast<unsigned*>(smraw + L.mx_off);  // [0] X, [1] Y
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smraw + L.mx_off + 8);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nrt = 2 * max(hx, hy) + 2;
  for (int i = tid; i < nrt; i += NT) rtx[i].x = i ? __frcp_rn((float)i) : 0.f;
  if (tid < 2) smax[tid] = 0u;
  const bool over = overwrite > 0.f && overwrite < 1.f;  // v itself is already
                                                          // overwritten
  const int xs = t.x0 - HA;   // image x of staged column 0
  const int gy0 = t.y0 - hy;  // image y of row 0
  // TMA staging: the box is SWS x SR (its row stride in shared memory is
  // the staging stride); the destination must be 128-byte aligned
  const bool use_tma = tmaps != nullptr && (smem_u32(Xf) & 127u) == 0;
  if (use_tma) {
    if (tid == 0) {
      mbar_init(bar, 1);
      mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0) {
      mbar_arrive_expect_tx(bar, (unsigned)(L.sws * SR * 4));
      tma_load_2d(Xf, tmaps + t.inst, xs, gy0, bar);
    }
  }
  const int lgx = ceil_log2(2 * hx + 1), lgy = ceil_log2(2 * hy + 1);
  // ---- 3'. the X half-step's loads for this thread's first group ------------
  const int cq = tid % QW, r3 = tid / QW;  // group of columns x3 .. x3 + 3
  const int x3 = t.x0 + 4 * cq;
  struct Quad {
    uint4 b;  // 0 outside the image
    Raw4<TS> tv, cv;
    float4 vv;
  };
  auto fetch = [&](int r, Quad& Q) {
    const int y = gy0 + r;
    if (r < SR && x3 < W && (unsigned)y < (unsigned)H) {
      const int p = y * P + x3;
      Q.b = __ldg(reinterpret_cast<const uint4*>(bnd_i + p));
      Q.tv.load(tgt_i + p);
      Q.cv.load(cnf_i + p);
      Q.vv = __ldg(reinterpret_cast<const float4*>(vin_i + p));
      if (x3 + 4 > W) {  // columns past the width hold the pitch's padding
        if (x3 + 1 >= W) Q.b.y = 0u;
        if (x3 + 2 >= W) Q.b.z = 0u;
        Q.b.w = 0u;
      }
    } else {
      Q.b = make_uint4(0u, 0u, 0u, 0u);
      Q.tv.zero();
      Q.cv.zero();
      Q.vv = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  Quad QA, QB;
  fetch(r3, QA);
  __syncthreads();  // smax initialised
  // A non-finite value in the staged box (or among the X results) has no
  // fixed-point form: the tile's outputs are then NaN, as every pixel of it
  // can reach that value within the iteration (the reference's float prefix
  // sums carry it along rows and columns likewise).  Never finite garbage.
  auto poison = [&]() {
    if (x3 >= W) return;
    const int jmax = min(TH, H - t.y0);
    for (int j = r3; j < jmax; j += RPP) {
      float* dst = vout_i + (t.y0 + j) * P + x3;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (x3 + k < W) dst[k] = __int_as_float(0x7fc00000);
    }
  };
  // ---- 1. stage the iterate, four columns per item, four items in flight -------
  unsigned mb = 0u;  // magnitude bits (mag_bits)
  if (use_tma) {
    // every thread waits for the box; a CTA whose wait ran out (all of its
    // threads agree through the barrier) records it and leaves its tile
    const bool ok = mbar_wait_bounded(bar, 0, kTmaWaitPolls);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicAdd(&g_wait_timeouts, 1ull);
      (void)mbar_wait_bounded(bar, 0, kTmaWaitPolls);  // the copy may still land
      return;
    }
    const int SW4 = SW >> 2, n = SR * SW4;
    const unsigned mg = L.sw4_magic;
    for (int i = tid; i < n; i += NT) {
      const int r = fast_div(i, mg), q = i - r * SW4;
      const float4 v = *reinterpret_cast<const float4*>(Xf + r * SWS + 4 * q);
      mb = max(mb, max(max(mag_bits(v.x), mag_bits(v.y)), max(mag_bits(v.z), mag_bits(v.w))));
    }
  } else {
    constexpr int U = 4;
    const int SW4 = SW >> 2, n = SR * SW4;
    const unsigned mg = L.sw4_magic;
    for (int i0 = tid; i0 < n; i0 += U * NT) {
      float4 v[U];
      int dst[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * NT;
        const int r = fast_div(i, mg), q = i - r * SW4;
        const int y = gy0 + r, x = xs + 4 * q;
        dst[u] = i < n ? r * SWS + 4 * q : -1;
        v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < n && (unsigned)y < (unsigned)H && x >= 0 && x < W)
          v[u] = __ldg(reinterpret_cast<const float4*>(vin_i + y * P + x));
        if (x + 4 > W) {  // columns past the width hold the pitch's padding
          if (x + 1 >= W) v[u].y = 0.f;
          if (x + 2 >= W) v[u].z = 0.f;
          v[u].w = 0.f;
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (dst[u] >= 0) *reinterpret_cast<float4*>(Xf + dst[u]) = v[u];
        mb = max(mb, max(max(mag_bits(v[u].x), mag_bits(v[u].y)),
                         max(mag_bits(v[u].z), mag_bits(v[u].w))));
      }
    }
  }
  mb = __reduce_max_sync(0xffffffffu, mb);
  if (lane == 0) atomicMax(&smax[0], mb);
  __syncthreads();
  if (smax[0] >= kNonFiniteBits) {
    poison();
    return;
  }
  // ---- 2. X prefix: a thread per 16-entry segment of a row, then offsets -------
  {
    const float sF = pow2f(fx_shift(__uint_as_float(smax[0]), lgx));
    const float isF = pow2f(-fx_shift(__uint_as_float(smax[0]), lgx));
    for (int i = tid; i < nrt; i += NT) rtx[i].y = rtx[i].x * isF;
    const int NSX = L.nsx, n = SR * NSX, SW4 = SW >> 2;
    unsigned* segx = reinterpret_cast<unsigned*>(sx);  // SR x NSX totals (sx is free)
    for (int i = tid; i < n; i += NT) {
      const int sg = fast_div(i, L.sr_magic), r = i - sg * SR;  // lanes on rows
      uint4* e = reinterpret_cast<uint4*>(XP + r * SWS) + 4 * sg;
      const float4* f = reinterpret_cast<const float4*>(Xf + r * SWS) + 4 * sg;
      const int nq = min(4, SW4 - 4 * sg);
      unsigned acc = 0u;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (q < nq) {
          const float4 v = f[q];
          uint4 w;
          w.x = acc += fx_from(v.x, sF);
          w.y = acc += fx_from(v.y, sF);
          w.z = acc += fx_from(v.z, sF);
          w.w = acc += fx_from(v.w, sF);
          e[q] = w;
        }
      }
      segx[r * NSX + sg] = acc;
    }
    __syncthreads();
    for (int i = tid; i < n; i += NT) {
      const int sg = fast_div(i, L.sr_magic), r = i - sg * SR;
      if (sg == 0) continue;
      unsigned off = 0u;
      for (int s2 = 0; s2 < sg; ++s2) off += segx[r * NSX + s2];
      uint4* e = reinterpret_cast<uint4*>(XP + r * SWS) + 4 * sg;
      const int nq = min(4, SW4 - 4 * sg);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (q < nq) {
          uint4 w = e[q];
          w.x += off;
          w.y += off;
          w.z += off;
          w.w += off;
          e[q] = w;
        }
      }
    }
  }
  __syncthreads();
  // ---- 3. X half-step for the tile columns over all rows -----------------------
  {
    unsigned mloc = 0u;  // magnitude bits of the X results
    auto compute = [&](int r, const Quad& Q) {
      const unsigned* e0 = XP + r * SWS + HA + 4 * cq;  // e0[k]: prefix at x3 + k
      float o[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        o[k] = 0.f;
        const uint32_t b = u4_get(Q.b, k);
        if (b) {  // inside the image (a window always holds its own pixel)
          const int dl = min((int)(b & 0xff), hx + 1);
          const int du = min((int)((b >> 8) & 0xff), hx);
          const float2 rr = rtx[dl + du];
          const float rn = rr.x;
          const float B = fx_window(e0[k + du], e0[k - dl], rr.y);
          const float vv = f4_get(Q.vv, k), tv = Q.tv[k], cv = Q.cv[k];
          float extra = 0.f;
          if (STEREO)
            extra = photometric(sa, in.off + (long long)(gy0 + r) * P, x3 + k, W, vv);
          o[k] = x_update<MODE, STEREO>(vv, B, tv, cv, rn, lambda, step, extra);
          if (over && cv > overwrite) o[k] = tv;
        }
        mloc = max(mloc, mag_bits(o[k]));
      }
      *reinterpret_cast<float4*>(sx + r * TQ + 4 * cq) = make_float4(o[0], o[1], o[2], o[3]);
      // the Y bytes (b >> 16) of the four pixels as four u16
      *reinterpret_cast<uint2*>(sby + r * TW + 4 * cq) =
          make_uint2((Q.b.x >> 16) | (Q.b.y & 0xffff0000u), (Q.b.z >> 16) | (Q.b.w & 0xffff0000u));
    };
    int r = r3;
    while (r < SR) {
      if (r + RPP < SR) fetch(r + RPP, QB);
      compute(r, QA);
      r += RPP;
      if (r >= SR) break;
      if (r + RPP < SR) fetch(r + RPP, QA);
      compute(r, QB);
      r += RPP;
    }
    mloc = __reduce_max_sync(0xffffffffu, mloc);
    if (lane == 0) atomicMax(&smax[1], mloc);
  }
  __syncthreads();
  if (smax[1] >= kNonFiniteBits) {
    poison();
    return;
  }
  // ---- 4. Y prefix: a warp per group of four columns, a lane per segment ---------
  const int Fy = fx_shift(__uint_as_float(smax[1]), lgy);
  const float sFy = pow2f(Fy), isFy = pow2f(-Fy);
  for (int i = tid; i < nrt; i += NT) rsy[i] = rtx[i].x * isFy;
  {
    const int RY = SR + 1;
    const int k0 = min(lane * L.seg, RY), k1 = min(k0 + L.seg, RY);
    for (int q = warp; q < QW; q += NW) {
      uint4 acc = make_uint4(0u, 0u, 0u, 0u);
      for (int k = k0; k < k1; ++k) {
        if (k > 0) {
          const float4 v = *reinterpret_cast<const float4*>(sx + (k - 1) * TQ + 4 * q);
          acc.x += fx_from(v.x, sFy);
          acc.y += fx_from(v.y, sFy);
          acc.z += fx_from(v.z, sFy);
          acc.w += fx_from(v.w, sFy);
        }
        *reinterpret_cast<uint4*>(Py + k * TQ + 4 * q) = acc;
      }
      uint4 off;
      off.x = warp_incl_scan(acc.x, lane) - acc.x;
      off.y = warp_incl_scan(acc.y, lane) - acc.y;
      off.z = warp_incl_scan(acc.z, lane) - acc.z;
      off.w = warp_incl_scan(acc.w, lane) - acc.w;
      for (int k = k0; k < k1; ++k) {
        uint4* pk = reinterpret_cast<uint4*>(Py + k * TQ + 4 * q);
        uint4 w = *pk;
        w.x += off.x;
        w.y += off.y;
        w.z += off.z;
        w.w += off.w;
        *pk = w;
      }
    }
  }
  __syncthreads();
  // ---- 5. Y half-step, four pixels per thread, vector stores --------------------
  const float slam = step * lambda;
  if (x3 >= W) return;
  const int jmax = min(TH, H - t.y0);
  for (int j = r3; j < jmax; j += RPP) {
    const uint2 bq = *reinterpret_cast<const uint2*>(sby + (j + hy) * TW + 4 * cq);
    const float4 v4 = *reinterpret_cast<const float4*>(sx + (j + hy) * TQ + 4 * cq);
    const unsigned* c0 = Py + (j + hy + 1) * TQ + 4 * cq;
    float o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const unsigned b = ((k < 2 ? bq.x : bq.y) >> (16 * (k & 1))) & 0xffffu;
      const int dl = min((int)(b & 0xff), hy + 1), du = min((int)(b >> 8), hy);
      const float Bv = fx_window(c0[du * TQ + k], c0[-dl * TQ + k], rsy[dl + du]);
      const float v = f4_get(v4, k);
      o[k] = __fmaf_rn(-slam, v - Bv, v);
    }
    float* dst = vout_i + (t.y0 + j) * P + x3;
    if (x3 + 4 <= W) {
      *reinterpret_cast<float4*>(dst) = make_float4(o[0], o[1], o[2], o[3]);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (x3 + k < W) dst[k] = o[k];
    }
  }
}

// ---------------------------------------------------------------------------
// The same iteration for large halos (k_dts_iter_rows): shared memory grows
// linearly with the halo instead of with its square, so every sigma_z below
// 254 fits the 32 x 32 tiles.  Window sums from fixed-point prefix sums
// (fixed_point.cuh) as in k_dts_iter_vec; the X scale comes from the
// largest magnitude in the row (X) or among the tile's X results (Y).
//
// X half-step: one warp per row of the tile plus the vertical halo; each
// lane scans four consecutive values, a warp shuffle scan joins the lanes,
// and the row's prefix sits in a per-warp shared buffer.  A warp issues the
// global loads of its next row before working on the current one.  Y
// half-step: the X results stay in shared memory; each thread scans a
// segment of one column, segment offsets are added in a second pass, and
// the tile's output rows are written coalesced.  Reciprocals 1/n come from
// a per-block table of correctly rounded values.
// ---------------------------------------------------------------------------
template <int TW, int TH, int NT>
struct PrefixIterSmem {
  // bytes of shared memory for halos hx, hy
  static size_t bytes(int hx, int hy) {
    const size_t SR = TH + 2 * hy, SWX = TW + 2 * hx + 1;
    const size_t py = std::max((SR + 1) * TW, (size_t)(NT / 32) * SWX) * 4;
    const size_t seg = (size_t)(NT / TW) * TW * 4;
    const size_t sx = SR * (TW + 1) * 4;
    const size_t sby = (size_t)TH * TW * 2;
    const size_t rt = (size_t)(2 * std::max(hx, hy) + 2) * 4;
    return py + seg + sx + sby + rt + 16;
  }
};

template <typename TS, int MODE, int TW, int TH, int NT, bool STEREO = false>
__global__ void __launch_bounds__(NT, 1024 / NT)
    k_dts_iter_rows(const Inst* __restrict__ insts, const Tile* __restrict__ tiles,
                      const float* __restrict__ vin, float* __restrict__ vout,
                      const TS* __restrict__ tgt, const TS* __restrict__ cnf,
                      const uint32_t* __restrict__ bnd, float lambda, float step,
                      float overwrite, int hx, int hy, StereoArgs sa) {
  static_assert(TW % 32 == 0 && NT % TW == 0, "tile width: whole warps");
  constexpr int NW = NT / 32, NSEG = NT / TW, TWp = TW + 1;
  extern __shared__ __align__(128) unsigned char smraw[];
  const Tile t = tiles[blockIdx.x];
  const Inst in = insts[t.inst];
  const int W = in.w, H = in.h, P = in.pitch;
  const int SR = TH + 2 * hy, SWX = TW + 2 * hx + 1, RY = SR + 1;
  const int pyn = max(RY * TW, NW * SWX);
  unsigned* Py = reinterpret_cast<unsigned*>(smraw);  // RY x TW (Y phase)
  unsigned* Xb = Py;                                  // NW x SWX (X phase)
  unsigned* segtot = Py + pyn;                        // NSEG x TW
  float* sx = reinterpret_cast<float*>(segtot + NSEG * TW);   // SR x TWp
  uint16_t* sby = reinterpret_cast<uint16_t*>(sx + SR * TWp);  // TH x TW
  float* rtab = reinterpret_cast<float*>(sby + TH * TW);
  const int nrt = 2 * max(hx, hy) + 2;
  unsigned* smax = reinterpret_cast<unsigned*>(rtab + nrt);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < nrt; i += NT) rtab[i] = i ? __frcp_rn((float)i) : 0.f;
  if (tid == 0) *smax = 0u;
  __syncthreads();
  const bool over = overwrite > 0.f && overwrite < 1.f;
  const int gx0 = t.x0 - hx - 1;  // image x of X prefix entry 0 (a zero entry)
  const int gy0 = t.y0 - hy;      // image y of sx row 0
  const int lgx = ceil_log2(2 * hx + 1), lgy = ceil_log2(2 * hy + 1);
  // ---- X half-step ----------------------------------------------------------
  constexpr int CPL = TW / 32;  // tile columns per lane
  struct RowIn {
    float v4[4];  // prefix entries 4*lane .. 4*lane+3
    uint32_t b[CPL];  // tile columns lane + 32k
    float tv[CPL], cv[CPL], vc[CPL];
  };
  auto load_v = [&](bool yok, long long row, int cc) -> float {  // prefix entry cc
    const int x = gx0 + cc;
    if (cc < 1 || cc >= SWX || !yok || (unsigned)x >= (unsigned)W) return 0.f;
    float v = __ldg(vin + row + x);
    if (over && load_f(cnf + row + x) > overwrite) v = load_f(tgt + row + x);
    return v;
  };
  auto fetch = [&](int r, RowIn& R) {
    const int y = gy0 + r;
    const bool yok = (unsigned)y < (unsigned)H;
    const long long row = in.off + (long long)y * P;
#pragma unroll
    for (int j = 0; j < 4; ++j) R.v4[j] = load_v(yok, row, 4 * lane + j);
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
      const int x = t.x0 + lane + 32 * k;
      R.b[k] = 0u;
      R.tv[k] = R.cv[k] = R.vc[k] = 0.f;
      if (yok && x < W) {
        const long long p = row + x;
        R.b[k] = __ldg(bnd + p);
        R.tv[k] = load_f(tgt + p);
        R.cv[k] = load_f(cnf + p);
        R.vc[k] = __ldg(vin + p);
      }
    }
  };
  unsigned mloc = 0u;  // magnitude bits of the X results
  unsigned* xb = Xb + warp * SWX;
  RowIn cur, nxt;
  if (warp < SR) fetch(warp, cur);
  for (int r = warp; r < SR; r += NW) {
    if (r + NW < SR) fetch(r + NW, nxt);
    const int y = gy0 + r;
    const bool yok = (unsigned)y < (unsigned)H;
    const long long row = in.off + (long long)y * P;
    unsigned mb = max(max(mag_bits(cur.v4[0]), mag_bits(cur.v4[1])),
                      max(mag_bits(cur.v4[2]), mag_bits(cur.v4[3])));
    for (int base = 128; base < SWX; base += 128)
#pragma unroll
      for (int j = 0; j < 4; ++j) mb = max(mb, mag_bits(load_v(yok, row, base + 4 * lane + j)));
    mb = __reduce_max_sync(0xffffffffu, mb);
    // a non-finite value in the row: its X results are NaN (see below)
    const bool row_bad = mb >= kNonFiniteBits;
    const int F = fx_shift(__uint_as_float(row_bad ? 0u : mb), lgx);
    const float sF = pow2f(F), isF = pow2f(-F);
    unsigned carry = 0;
    for (int base = 0; base < SWX; base += 128) {
      unsigned s4[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float v = base == 0 ? cur.v4[j] : load_v(yok, row, base + 4 * lane + j);
        s4[j] = fx_from(v, sF) + (j ? s4[j - 1] : 0u);
      }
      const unsigned incl = warp_incl_scan(s4[3], lane);
      const unsigned off = carry + incl - s4[3];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int cc = base + 4 * lane + j;
        if (cc < SWX) xb[cc] = off + s4[j];
      }
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
      const int c = lane + 32 * k;
      const int x = t.x0 + c;
      float o = 0.f;
      if (yok && x < W) {
        const uint32_t b = cur.b[k];
        const float tv = cur.tv[k], cv = cur.cv[k];
        float v = cur.vc[k];
        if (over && cv > overwrite) v = tv;
        const int dl = min((int)(b & 0xff), hx + 1);
        const int du = min((int)((b >> 8) & 0xff), hx);
        const float rn = rtab[dl + du];
        const int i = c + hx + 1;
        const float B = fx_window(xb[i + du], xb[i - dl], rn * isF);
        float extra = 0.f;
        if (STEREO) extra = photometric(sa, row, x, W, v);
        o = x_update<MODE, STEREO>(v, B, tv, cv, rn, lambda, step, extra);
        if (over && cv > overwrite) o = tv;
        if (row_bad) o = __int_as_float(0x7fc00000);
        if (r >= hy && r < hy + TH) sby[(r - hy) * TW + c] = (uint16_t)(b >> 16);
      }
      sx[r * TWp + c] = o;
      mloc = max(mloc, mag_bits(o));
    }
    __syncwarp();  // the warp's prefix buffer is rewritten for its next row
    cur = nxt;
  }
  mloc = __reduce_max_sync(0xffffffffu, mloc);
  if (lane == 0) atomicMax(smax, mloc);
  __syncthreads();
  if (*smax >= kNonFiniteBits) {
    // a non-finite value reached the X results: the tile's outputs are NaN
    // (every pixel of it can reach that value), never finite garbage
    const int x = t.x0 + tid % TW;
    for (int j = tid / TW; j < TH; j += NT / TW)
      if (t.y0 + j < H && x < W)
        vout[in.off + (long long)(t.y0 + j) * P + x] = __int_as_float(0x7fc00000);
    return;
  }
  // ---- Y half-step ----------------------------------------------------------
  const int Fy = fx_shift(__uint_as_float(*smax), lgy);
  const float sFy = pow2f(Fy), isFy = pow2f(-Fy);
  const int c = tid % TW, sgi = tid / TW;
  const int seg = (RY + NSEG - 1) / NSEG;
  const int k0 = min(sgi * seg, RY), k1 = min(k0 + seg, RY);
  unsigned acc = 0;
  for (int k = k0; k < k1; ++k) {
    if (k > 0) acc += fx_from(sx[(k - 1) * TWp + c], sFy);
    Py[k * TW + c] = acc;
  }
  segtot[sgi * TW + c] = acc;
  __syncthreads();
  unsigned off = 0;
  for (int s2 = 0; s2 < sgi; ++s2) off += segtot[s2 * TW + c];
  for (int k = k0; k < k1; ++k) Py[k * TW + c] += off;
  __syncthreads();
  const float slam = step * lambda;
  const int x = t.x0 + c;
  for (int j = sgi; j < TH; j += NSEG) {
    const int y = t.y0 + j;
    if (y >= H || x >= W) continue;
    const uint32_t b = sby[j * TW + c];
    const int dl = min((int)(b & 0xff), hy + 1), du = min((int)(b >> 8), hy);
    const int k = j + hy + 1;
    const float B = fx_window(Py[(k + du) * TW + c], Py[(k - dl) * TW + c],
                              rtab[dl + du] * isFy);
    const float v = sx[(j + hy) * TWp + c];
    vout[in.off + (long long)y * P + x] = __fmaf_rn(-slam, v - B, v);
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
  const size_t smem = sizeof(unsigned) * ((size_t)TH * ((TW + 2 * rx) | 1) +
                                          (size_t)(TH + 2 * ry) * TW) +
                      2 * sizeof(uint16_t) * TH * TW;
  if (smem > kMaxSmem) return fail(DTSGB_ERR_UNSUPPORTED, "sigma too large");
  // fixed point per axis: r * (sigma + 1) * 2^F <= 2^30; threshold floor(sigma 2^F)
  auto fx = [](int r, float sigma, float* cap, float* scale, int* T) {
    *cap = sigma + 1.f;
    const int F = 30 - (int)std::ceil(std::log2((double)r * (double)*cap));
    *scale = std::ldexp(1.f, F);
    *T = (int)std::floor((double)sigma * std::ldexp(1.0, F));
  };
  float cap_x, cap_y, scale_x, scale_y;
  int Tx, Ty;
  fx(rx, sigma_x, &cap_x, &scale_x, &Tx);
  fx(ry, sigma_y, &cap_y, &scale_y, &Ty);
  auto go = [&](auto kern) -> int {
    int st = set_smem(kern, smem);
    if (st) return st;
    ProfScope ps(s, DTSGB_K_BOUNDS);
    kern<<<L.n_tiles, kThreads, smem, s>>>(L.d_inst, L.d_tiles, guide, bounds, ratio_x,
                                           ratio_y, rx, ry, ref_y_limit, cap_x, cap_y,
                                           scale_x, scale_y, Tx, Ty);
    DTSGB_CUDA(cudaGetLastError());
    return DTSGB_OK;
  };
  if (L.bounds_seg == 4) return go(k_bounds<kBoundsTW, kBoundsTH, 4>);
  if (L.bounds_seg == 16) return go(k_bounds<kBoundsTW, kBoundsTH, 16>);
  return go(k_bounds<kBoundsTW, kBoundsTH, kBoundsSegDefault>);
}

template <typename TS, int MODE, int TW, int TH, bool STEREO>
static int launch_iter_shape(const DtsLaunch& L, const float* vin, float* vout,
                             const void* target, const void* conf,
                             const uint32_t* bounds, float lambda, float step,
                             float overwrite, int hx, int hy, cudaStream_t s,
                             const StereoArgs& sa) {
  constexpr int NT = TW >= 64 ? 512 : 256;
  const VecIterSmem<TW, TH, NT> lay(hx, hy);
  const size_t smem = (size_t)lay.total;
  const size_t smem_rows = PrefixIterSmem<TW, TH, NT>::bytes(hx, hy);
  if (smem > kMaxSmem && smem_rows > kMaxSmem)
    return fail(DTSGB_ERR_UNSUPPORTED, "sigma_z too large");
  if (overwrite > 0.f && overwrite < 1.f) {
    // the input iterate is overwritten in place, as the reference does
    k_overwrite<TS><<<dim3(64, L.n_inst), kThreads, 0, s>>>(
        L.d_inst, const_cast<float*>(vin), (const TS*)target, (const TS*)conf, overwrite);
    DTSGB_CUDA(cudaGetLastError());
  }
  if (smem > kMaxSmem) {  // halo too large for the tile-staged kernel
    int st = set_smem(k_dts_iter_rows<TS, MODE, TW, TH, NT, STEREO>, smem_rows);
    if (st) return st;
    ProfScope ps(s, DTSGB_K_DTS_ITER);
    k_dts_iter_rows<TS, MODE, TW, TH, NT, STEREO><<<L.n_tiles, NT, smem_rows, s>>>(
        L.d_inst, L.d_tiles, vin, vout, (const TS*)target, (const TS*)conf,
        bounds, lambda, step, overwrite, hx, hy, sa);
    DTSGB_CUDA(cudaGetLastError());
    return DTSGB_OK;
  }
  int st = set_smem(k_dts_iter_vec<TS, MODE, TW, TH, NT, STEREO>, smem);
  if (st) return st;
  // TMA staging of the iterate box (SWS x SR, both within the 256-element
  // box limit) from the owner's tensor-map cache, when it has one
  const CUtensorMap* tm = nullptr;
  if (L.tma && L.h_inst && lay.sws <= 256 && lay.sr <= 256)
    tm = L.tma->get(L.h_inst, L.n_inst, vin, lay.sws, lay.sr, s);
  ProfScope ps(s, DTSGB_K_DTS_ITER);
  DTSGB_CUDA(launch_dependent(k_dts_iter_vec<TS, MODE, TW, TH, NT, STEREO>, dim3(L.n_tiles),
                              dim3(NT), smem, s, L.d_inst, L.d_tiles, vin, vout,
                              (const TS*)target, (const TS*)conf, bounds, lambda, step,
                              overwrite, hx, hy, sa, lay, tm));
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
  if (L.d_tiles_small &&
      (size_t)VecIterSmem<kIterTW, kIterTH, 512>(hx, hy).total > kMaxSmem &&
      PrefixIterSmem<kIterTW, kIterTH, 512>::bytes(hx, hy) > kMaxSmem)
    return launch_iter_shape<TS, MODE, kIterSmallTW, kIterSmallTH, STEREO>(
        L.as_small(), vin, vout, target, conf, bounds, lambda, step, overwrite, hx, hy,
        s, sa);
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
  if (L.d_tiles_small &&
      NCH * sizeof(float) * ((size_t)(kIterTH + 2 * hy) * (kIterTW + 2 * hx) +
                             (size_t)(kIterTH + 2 * hy) * kIterTW) > kMaxSmem)
    return launch_filter_shape<NCH, CONF, TS, kIterSmallTW, kIterSmallTH>(
        L.as_small(), in0, in1, out0, out1, bounds, hx, hy, conf_out, scale, left_clear, s);
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

unsigned long long dts_wait_timeouts() {
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_wait_timeouts, sizeof v) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return v;
}

// Tensor-map boxes the iteration kernel stages for halos hx, hy on the
// current tile shape (0 x 0: staged by loads).
void dts_iter_tma_box(const DtsLaunch& L, int hx, int hy, int* box_w, int* box_h) {
  *box_w = *box_h = 0;
  int sws = 0, sr = 0;
  // the tile shape launch_iter_t picks, then the staged kernel's box (the
  // large-halo kernel, taken when that box does not fit, stages by loads)
  const VecIterSmem<kIterTW, kIterTH, 512> big(hx, hy);
  const bool small =
      L.small || (L.d_tiles_small && (size_t)big.total > kMaxSmem &&
                  PrefixIterSmem<kIterTW, kIterTH, 512>::bytes(hx, hy) > kMaxSmem);
  if (small) {
    const VecIterSmem<kIterSmallTW, kIterSmallTH, 256> lay(hx, hy);
    if ((size_t)lay.total > kMaxSmem) return;
    sws = lay.sws;
    sr = lay.sr;
  } else {
    if ((size_t)big.total > kMaxSmem) return;
    sws = big.sws;
    sr = big.sr;
  }
  if (sws <= 256 && sr <= 256) {
    *box_w = sws;
    *box_h = sr;
  }
}

int launch_unpack_bounds(const DtsLaunch& L, const uint32_t* bounds, int axis,
                         int32_t* l, int32_t* u, cudaStream_t s) {
  k_unpack_bounds<<<dim3(64, L.n_inst), kThreads, 0, s>>>(L.d_inst, bounds, axis,
                                                          l, u);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

}  // namespace dtsgb
