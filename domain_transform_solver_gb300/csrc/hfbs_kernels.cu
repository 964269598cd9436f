// HFBS kernels for sm_103a (Mazumdar et al. bilateral-grid solver as the
// reference implements it, src/hfbs.cu:65-427).
//
// Every kernel handles a batch of independent instances: blockIdx.y selects
// the instance, blockIdx.x strides over its pixels / voxels / lines (CTAs
// past the end of a small instance exit at once).  Grids are dense
// gx*gy*gl float arrays, x fastest.  Reads outside the interior follow the
// reference's buffers (see hfbs_internal.cuh / the oracle): index -1 reads 0
// (zero boundary mode), index g reads the pad value of that buffer.
//
// The splat is atomic-free and deterministic: one thread per spatial cell
// walks the cell's pixels in row-major order and bins them into per-thread
// luma histograms held in shared memory.
#include <algorithm>
#include <vector>

#include "../../include/dtsgb.h"
#include "dtsgb_internal.cuh"
#include "hfbs_internal.cuh"
#include "tma.cuh"

namespace dtsgb {

namespace {

constexpr int kT = 256;

// CTAs of this file's kernels that gave up waiting for their TMA staging.
__device__ unsigned long long g_wait_timeouts = 0;

__device__ __forceinline__ long long gidx(const HInst& I, int x, int y, int z) {
  return I.grid_off + ((long long)z * I.gy + y) * I.px + x;
}

// a12: SplatBAndC + BistochastasizeSetup (src/hfbs.cu:72-120).  Bins
// (floor(x/sx), floor(y/sy), floor(L/sl)) with L the .x channel; sums of
// c*t, c and 1 per bin.  Luma bin == gl lands in the overflow plane.
template <typename TS>
__global__ void __launch_bounds__(64)
    k_splat(const HInst* __restrict__ insts, const uchar4* __restrict__ guide,
            const TS* __restrict__ tgt, const TS* __restrict__ cnf,
            float* __restrict__ count, float* __restrict__ csum,
            float* __restrict__ b, float* __restrict__ ovf, HParams p) {
  extern __shared__ float sh[];
  __shared__ int lbin[256];  // luma bin of each 8-bit luma value
  const HInst I = insts[blockIdx.y];
  const int ncell = I.gx * I.gy;
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  const int gl = I.gl;
  // per-thread histograms: [bin][3] strided by blockDim for conflict-free use
  float* hist = sh;
  const int T = blockDim.x;
  if (blockIdx.x * blockDim.x >= ncell) return;
  for (int l = threadIdx.x; l < 256; l += T)
    lbin[l] = (int)floorf((float)l * 1.0f / p.sigma_l);
  __syncthreads();
  for (int k = 0; k < 3 * gl; ++k) hist[k * T + threadIdx.x] = 0.f;
  float ovf_cnt = 0.f;
  if (cell < ncell) {
    const int bx = cell % I.gx, by = cell / I.gx;
    const int xs = cell_start(bx, p.sigma_x, I.w), xe = cell_start(bx + 1, p.sigma_x, I.w);
    const int ys = cell_start(by, p.sigma_y, I.h), ye = cell_start(by + 1, p.sigma_y, I.h);
    // a run of pixels in the same luma bin is summed in registers and added
    // to the cell's histogram when the bin changes (a fixed order: the
    // result is deterministic)
    int run = -1;
    float r_ct = 0.f, r_c = 0.f, r_n = 0.f;
    auto flush = [&]() {
      if (run < 0) return;
      if (run < gl) {
        hist[(3 * run + 0) * T + threadIdx.x] += r_ct;
        hist[(3 * run + 1) * T + threadIdx.x] += r_c;
        hist[(3 * run + 2) * T + threadIdx.x] += r_n;
      } else {
        ovf_cnt += r_n;
      }
    };
    constexpr int U = 8;  // pixels whose loads are issued together
    for (int y = ys; y < ye; ++y) {
      const long long row = I.pix_off + (long long)y * I.pitch;
      for (int x0 = xs; x0 < xe; x0 += U) {
        int lum[U];
        float cv[U], tv[U];
#pragma unroll
        for (int k = 0; k < U; ++k) {
          lum[k] = 0;
          cv[k] = tv[k] = 0.f;
          if (x0 + k < xe) {
            lum[k] = guide[row + x0 + k].x;
            cv[k] = load_f(cnf + row + x0 + k);
            tv[k] = load_f(tgt + row + x0 + k);
          }
        }
#pragma unroll
        for (int k = 0; k < U; ++k) {
          if (x0 + k >= xe) break;
          const int bl = lbin[lum[k]];
          const float ct = cv[k] * tv[k];
          if (bl != run) {
            flush();
            run = bl;
            r_ct = ct;
            r_c = cv[k];
            r_n = 1.f;
          } else {
            r_ct += ct;
            r_c += cv[k];
            r_n += 1.f;
          }
        }
      }
    }
    flush();
    for (int z = 0; z < gl; ++z) {
      const long long gi = gidx(I, bx, by, z);
      b[gi] = hist[(3 * z + 0) * T + threadIdx.x];
      csum[gi] = hist[(3 * z + 1) * T + threadIdx.x];
      count[gi] = hist[(3 * z + 2) * T + threadIdx.x];
    }
    ovf[I.plane_off + cell] = I.ovf_stored ? ovf_cnt : 0.f;
  }
}

// The elementwise kernels below run flat over the whole grid arena: the
// voxels in the gaps between instances are computed too and never read.
__global__ void k_fill_ones(float* __restrict__ a, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    a[i] = 1.f;
}

// a13: one BistochastasizeOptimize step (src/hfbs.cu:126-155):
// n' = sqrt(n * (count + 1e-5) / (2n + sum6 nbr n + 1e-5)).  Faces covered by
// FillGrid read `pad`, all other out-of-grid reads 0.
__global__ void k_bistoch(const HInst* __restrict__ insts,
                          const float* __restrict__ src, float* __restrict__ dst,
                          const float* __restrict__ count, float pad) {
  pdl_wait_then_release();  // launched as a dependent of the previous pass
  const HInst I = insts[blockIdx.y];
  const int gx = I.gx, gy = I.gy, gl = I.gl;
  const float px = I.cov_x ? pad : 0.f, py = I.cov_y ? pad : 0.f,
              pz = I.cov_l ? pad : 0.f;
  const float* s = src + I.grid_off;
  const float* cn = count + I.grid_off;
  float* d = dst + I.grid_off;
  const int sy = I.px, sz = I.px * gy;
  // one thread per (x, y) column, marching along l: the l-neighbours come
  // from registers, and the loads of level l+1 are issued before level l is
  // computed
  for (int cl = blockIdx.x * blockDim.x + threadIdx.x; cl < gx * gy;
       cl += gridDim.x * blockDim.x) {
    const int y = cl / gx, x = cl - y * gx;
    const int col = y * sy + x;
    const bool xm = x > 0, xp = x + 1 < gx, ym = y > 0, yp = y + 1 < gy;
    auto nb4 = [&](int i, float (&o)[5]) {  // x-1, x+1, y-1, y+1, count
      o[0] = xm ? s[i - 1] : 0.f;
      o[1] = xp ? s[i + 1] : px;
      o[2] = ym ? s[i - sy] : 0.f;
      o[3] = yp ? s[i + sy] : py;
      o[4] = cn[i];
    };
    float vprev = 0.f, vcur = s[col];
    float cur[5], nxt[5];
    nb4(col, cur);
    for (int l = 0; l < gl; ++l) {
      const int i = l * sz + col;
      const bool more = l + 1 < gl;
      const float vnext = more ? s[i + sz] : pz;
      if (more) nb4(i + sz, nxt);
      float a = cur[0];
      a += cur[1];
      a += cur[2];
      a += cur[3];
      a += l > 0 ? vprev : 0.f;
      a += vnext;
      const float blurred = 2.f * vcur + a;
      d[i] = __fsqrt_rn(__fdiv_rn(vcur * (cur[4] + 0.00001f), blurred + 0.00001f));
      vprev = vcur;
      vcur = vnext;
#pragma unroll
      for (int k = 0; k < 5; ++k) cur[k] = nxt[k];
    }
  }
}

// a14: CalcInvDiagA (src/hfbs.cu:159-195):
// invA = 1 / max(1e-3, lambda*(count - 2 n^2) + sum c), evaluated by the
// reference in double and stored as float.  For a float d, rounding 1/d to
// double and then to float gives the correctly rounded float reciprocal (a
// product of a 24-bit and a 25-bit significand cannot come within 2^-53 of 1
// without equalling it, so 1/d never lands within a double ulp of a float
// midpoint), so the FP64 division is replaced by __frcp_rn.  d >= 1e-3f is
// the float form of (double)d > 1e-3, and 1/1e-3 rounds to 1000 (NaN too,
// as fmax returns the other operand).
__global__ void k_inv_diag(const float* __restrict__ count, const float* __restrict__ csum,
                           const float* __restrict__ norm, float* __restrict__ invA,
                           float lambda, long long n) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x) {
    const float nv = norm[g];
    const float diag = lambda * (count[g] - 2.f * nv * nv) + csum[g];
    invA[g] = diag >= 1e-3f ? __frcp_rn(diag) : 1000.f;
  }
}

// a15 along x (contiguous lines): one warp per line.  The forward recursion
// F(i) = s(i) + beta*F(i-1) and the backward one S(i) = s(i) + beta*S(i+1)
// are decayed scans over 32-element chunks (Hillis-Steele with beta^o weights,
// carry scaled by beta^(lane+1) between chunks); d(i) = F(i) + beta*S(i+1).
__global__ void k_laplace_x(const HInst* __restrict__ insts,
                            const float* __restrict__ s0, float* __restrict__ d0,
                            const float* __restrict__ s1, float* __restrict__ d1,
                            float beta) {
  const HInst I = insts[blockIdx.y];
  const int gx = I.gx, nlines = I.gy * I.gl;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  float bo[5];  // beta^1, beta^2, beta^4, beta^8, beta^16
  bo[0] = beta;
#pragma unroll
  for (int k = 1; k < 5; ++k) bo[k] = bo[k - 1] * bo[k - 1];
  float blane = 1.f;  // beta^(lane+1)
  for (int k = 0; k <= lane; ++k) blane *= beta;
  float brev = 1.f;  // beta^(32-lane)
  for (int k = lane; k < 32; ++k) brev *= beta;
  for (int line = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; line < nlines;
       line += nwarps) {
    const long long base = I.grid_off + (long long)line * I.px;
    for (int f = 0; f < 2; ++f) {
      const float* s = (f ? s1 : s0) + base;
      float* d = (f ? d1 : d0) + base;
      // forward: F
      float carry = 0.f;
      for (int x0 = 0; x0 < gx; x0 += 32) {
        const int x = x0 + lane;
        float r = x < gx ? s[x] : 0.f;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const float t = __shfl_up_sync(0xffffffffu, r, 1 << k);
          if (lane >= (1 << k)) r = __fmaf_rn(bo[k], t, r);
        }
        r = __fmaf_rn(blane, carry, r);
        if (x < gx) d[x] = r;
        carry = __shfl_sync(0xffffffffu, r, 31);
      }
      // backward: S over reversed chunks, add beta * S(i+1)
      carry = 0.f;  // S of the first element after the chunk
      const int last0 = ((gx - 1) / 32) * 32;
      for (int x0 = last0; x0 >= 0; x0 -= 32) {
        const int x = x0 + lane;
        float r = x < gx ? s[x] : 0.f;  // suffix scan runs from lane 31 down
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const float t = __shfl_down_sync(0xffffffffu, r, 1 << k);
          if (lane + (1 << k) < 32) r = __fmaf_rn(bo[k], t, r);
        }
        // lanes past the end hold zeros, so the suffix needs no masking;
        // add the carried S of the next chunk, decayed by beta^(32-lane)
        r = __fmaf_rn(brev, carry, r);
        float next = __shfl_down_sync(0xffffffffu, r, 1);  // S(i+1)
        if (lane == 31) next = carry;
        if (x < gx) d[x] = __fmaf_rn(beta, next, d[x]);
        carry = __shfl_sync(0xffffffffu, r, 0);
      }
    }
  }
}

// a15: Laplace sweep along one axis for two fields at once (src/hfbs.cu:
// 355-427): d(i) = sum_j beta^|i-j| s(j), forward then backward recursion,
// one thread per grid line (used along y and l, where consecutive threads
// take consecutive x and the accesses coalesce).  The recursions are serial,
// their loads are not: each thread loads kLapChunk elements of a line before
// it runs the recursion over them, so that a chunk's loads are in flight
// together instead of one load latency per element.
constexpr int kLapChunk = 8;
__global__ void k_laplace(const HInst* __restrict__ insts, int axis,
                          const float* __restrict__ s0, float* __restrict__ d0,
                          const float* __restrict__ s1, float* __restrict__ d1,
                          float beta) {
  constexpr int U = kLapChunk;
  const HInst I = insts[blockIdx.y];
  const int gx = I.gx, gy = I.gy, gl = I.gl;
  int len, na, nlines;
  long long stride;
  const int px = I.px;
  if (axis == 0) {
    len = gx; stride = 1; na = gy; nlines = gy * gl;
  } else if (axis == 1) {
    len = gy; stride = px; na = gx; nlines = gx * gl;
  } else {
    len = gl; stride = (long long)px * gy; na = gx; nlines = gx * gy;
  }
  for (int line = blockIdx.x * blockDim.x + threadIdx.x; line < nlines;
       line += gridDim.x * blockDim.x) {
    const int a = line % na, bb = line / na;
    long long base;
    if (axis == 0) base = ((long long)bb * gy + a) * px;
    else if (axis == 1) base = (long long)bb * px * gy + a;
    else base = (long long)bb * px + a;
    base += I.grid_off;
    for (int f = 0; f < 2; ++f) {
      const float* s = (f ? s1 : s0) + base;
      float* d = (f ? d1 : d0) + base;
      // forward: d(0) = s(0), d(i) = beta * d(i-1) + s(i)
      float r = 0.f;
      for (int i0 = 0; i0 < len; i0 += U) {
        float v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = i0 + u < len ? s[(i0 + u) * stride] : 0.f;
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = i0 + u;
          if (i < len) {
            r = i == 0 ? v[u] : __fmaf_rn(beta, r, v[u]);
            d[i * stride] = r;
          }
        }
      }
      // backward: r(len-1) = s(len-1); for i < len-1: r = beta * r,
      // d(i) += r, r += s(i)
      r = s[(long long)(len - 1) * stride];
      for (int i0 = len - 2; i0 >= 0; i0 -= U) {
        float v[U], w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = i0 - u;
          v[u] = i >= 0 ? s[i * stride] : 0.f;
          w[u] = i >= 0 ? d[i * stride] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = i0 - u;
          if (i >= 0) {
            r = beta * r;
            d[i * stride] = w[u] + r;
            r = r + v[u];
          }
        }
      }
    }
  }
}

// (float)((double)b / ((double)c + 1e-7)) without double arithmetic, which
// is slow on this part.  The denominator c + 1e-7 is carried as floats
// dh + dl to about 2^-48 of itself: an exact two-sum of c and the float
// nearest 1e-7, plus the rest of the double 1e-7.  q0 = b / dh is correctly
// rounded, so b - q0 * dh is exact by FMA, and q0 + (b - q0 * d) / dh carries
// the quotient to about 2^-46 of itself before the final rounding: it can
// differ from the double quotient's rounding only when that lies within
// about 2^-22 ulp of a float rounding midpoint.
__device__ __forceinline__ float div_by_c_plus_eps(float b, float c) {
  constexpr float e_hi = 1e-7f;
  constexpr float e_lo = (float)(1e-7 - (double)1e-7f);
  const float s = c + e_hi;
  const float bb = s - c;
  const float err = (c - (s - bb)) + (e_hi - bb);  // c + e_hi == s + err exactly
  const float dl0 = err + e_lo;
  const float dh = s + dl0;
  const float dl = dl0 - (dh - s);
  const float q0 = __fdiv_rn(b, dh);
  float r = __fmaf_rn(-q0, dh, b);
  r = __fmaf_rn(-q0, dl, r);
  return q0 + __fdiv_rn(r, dh);
}

// InitZ<true> (src/hfbs.cu:337-353): z = blur(b) / (blur(c) + 1e-7), the
// division in double as the reference's double literal makes it; h = 0.
__global__ void k_init_z(const float* __restrict__ blur_b, const float* __restrict__ blur_c,
                         float* __restrict__ z, float* __restrict__ h, long long n) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x) {
    z[g] = div_by_c_plus_eps(blur_b[g], blur_c[g]);
    h[g] = 0.f;
  }
}

// a16: SolveHFBS heavy-ball step (src/hfbs.cu:201-239).
__global__ void k_solve(const HInst* __restrict__ insts,
                        const float* __restrict__ zs, float* __restrict__ zd,
                        float* __restrict__ h, const float* __restrict__ norm,
                        const float* __restrict__ b,
                        const float* __restrict__ invA, float lambda,
                        float alpha, float beta) {
  const HInst I = insts[blockIdx.y];
  const int gx = I.gx, gy = I.gy, gl = I.gl;
  const float* z = zs + I.grid_off;
  const float* nn = norm + I.grid_off;
  const float* bb = b + I.grid_off;
  const float* ia = invA + I.grid_off;
  float* hh = h + I.grid_off;
  float* zo = zd + I.grid_off;
  const int sy = I.px, sz = I.px * gy;
  // one warp per grid row (fixed y, l); lanes stride along x
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < gy * gl;
       row += nwarps) {
    const int zz = row / gy, y = row - zz * gy;
    const int base = row * sy;
    // two x positions per lane per pass: their 34 loads are issued before
    // either result is computed
    for (int x0 = lane; x0 < gx; x0 += 64) {
      float d[2], zc[2], nc[2], bc[2], ic[2], hc[2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int x = x0 + 32 * j;
        d[j] = zc[j] = nc[j] = bc[j] = ic[j] = hc[j] = 0.f;
        if (x < gx) {
          const int i = base + x;
          float a = 0.f;
          if (x > 0) a += z[i - 1] * nn[i - 1];
          if (x + 1 < gx) a += z[i + 1] * nn[i + 1];
          if (y > 0) a += z[i - sy] * nn[i - sy];
          if (y + 1 < gy) a += z[i + sy] * nn[i + sy];
          if (zz > 0) a += z[i - sz] * nn[i - sz];
          if (zz + 1 < gl) a += z[i + sz] * nn[i + sz];
          d[j] = a;
          zc[j] = z[i];
          nc[j] = nn[i];
          bc[j] = bb[i];
          ic[j] = ia[i];
          hc[j] = hh[i];
        }
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int x = x0 + 32 * j;
        if (x >= gx) break;
        const int i = base + x;
        const float q = (bc[j] + lambda * nc[j] * d[j]) * ic[j];
        const float grad = zc[j] - q;
        // |grad| > 1.345 with the double threshold of the reference: the
        // smallest float above 1.345 (double) is 1.345f
        const float gc = fabsf(grad) >= 1.345f ? copysignf(1.f, grad) : grad;
        const float hn = __fmaf_rn(beta, hc[j], gc);
        hh[i] = hn;
        zo[i] = zc[j] - alpha * hn;
      }
    }
  }
}

// a16, K steps per pass (temporal blocking).  A CTA loads a 24 x 24 block of
// (x, y) columns, a 16 x 16 tile plus a K = 4 column halo, with all l levels;
// each thread keeps the z, h and n of its column in registers (b and invA
// in shared memory) and the z * n products of a step go through shared
// memory to the x and y neighbours.  Step k updates the columns at least k
// inside the block, whose neighbours the previous step updated, so after K
// steps the tile is exact.  Outside the grid (and above level gl) z = n = 0,
// so z * n there adds zero to a neighbour sum without bounds tests.  The
// neighbour sum adds the six rounded products in the reference's order
// (x-1, x+1, y-1, y+1, l-1, l+1).  HBM traffic is about a quarter of four
// one-step passes: the halo comes from L2.  h ping-pongs between hs and hd
// because a neighbouring CTA reads the old h of this tile's columns as its
// halo.
//
// The block arrives by TMA: one cp.async.bulk.tensor load per plane of the
// 24 x 24 x 16 box (tensor maps of the pitched grids, zeros outside the
// grid and above level gl), issued by one thread and waited for on an
// mbarrier; without tensor maps, by 4-byte cp.async copies (zero-filled
// outside the grid).  z, h and n are staged in the space the z * n buffers
// use afterwards.  Every thread reads and writes only its own column there,
// so the reuse needs no barrier.
constexpr int kTBT = 16, kTBK = 4, kTBL = kTBT + 2 * kTBK;
static_assert(kTBK == kHfbsTBSteps, "steps per temporally blocked launch");
constexpr int kTBMaxGL = 16;
constexpr int kTBThreads = kTBL * kTBL;  // one thread per (x, y) column
constexpr int kTBPlane = kTBMaxGL * kTBThreads;  // floats per staged array
// b, invA, then z, h, n staged (later z * n, double-buffered), an mbarrier
constexpr size_t kTBSmem = sizeof(float) * 5 * kTBPlane + 16;
constexpr unsigned kTBBoxBytes = sizeof(float) * kTBPlane;  // one plane's box

// Tensor-map tables (one entry per instance of the launch) of the planes a
// temporally blocked launch stages; all null: staged by 4-byte copies.
struct TBMaps {
  const CUtensorMap *b, *a, *z, *h, *n;
};

// Issues the block's TMA loads (thread 0; the mbarrier initialised for one
// arrival) of np planes into consecutive kTBPlane regions from dst, and
// waits, bounded.  False (the same in every thread) when the wait ran out.
__device__ __forceinline__ bool tb_tma_stage(const CUtensorMap* const* maps, int np, float* dst,
                                             int x0, int y0, unsigned long long* bar) {
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(bar, (unsigned)np * kTBBoxBytes);
    for (int k = 0; k < np; ++k)
      tma_load_3d(dst + (size_t)k * kTBPlane, maps[k] + blockIdx.y, x0, y0, 0, bar);
  }
  const bool ok = mbar_wait_bounded(bar, 0, kTmaWaitPolls);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) atomicAdd(&g_wait_timeouts, 1ull);
    (void)mbar_wait_bounded(bar, 0, kTmaWaitPolls);  // copies may still land
    return false;
  }
  return true;
}

// True when column (xx, yy) of a temporally blocked block is updated at step
// k: it lies at least k columns inside the block.
__device__ __forceinline__ bool tb_active(int xx, int yy, int k) {
  return xx >= k && xx < kTBL - k && yy >= k && yy < kTBL - k;
}

// 4-byte global -> shared copy; copies zero bytes (the destination is
// zero-filled) when !valid, and src must then still be a mapped address.
__device__ __forceinline__ void cp_async_f32(float* dst, const float* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src),
               "r"(valid ? 4 : 0)
               : "memory");
}

// a13, up to K bistochastization iterations per pass (temporal blocking as
// in k_solve_tb): a thread per (x, y) column of a 24 x 24 block keeps its
// column's v in registers (its counts in shared memory), and v goes through
// shared memory to the x and y neighbours.  Columns past the grid hold what
// the one-step kernel reads there: the covered pad faces (x = gx, y = gy,
// and level gl when covered) the pad value of the iteration's parity (1 on
// even iterations, 0 on odd ones), everything else 0.  The neighbour order
// and the arithmetic are k_bistoch's, so the result is bitwise that of the
// one-step passes.  it0: the global index of the pass's first iteration.
// v x 2 (the first also the staged src), count, an mbarrier
constexpr size_t kTBBistochSmem = sizeof(float) * 3 * kTBPlane + 16;
// Small grids only: there one-step passes are launch-latency-bound (about
// 12 us each on GB300 whatever the size) and four iterations per pass win
// (a 640x480 colorization's two 80x60x16 grids: 0.097 against 0.246 ms).  At 11.7 M voxels
// the one-step kernel's 0.056 ms per iteration beats this kernel's 0.063 (one
// 576-thread CTA per SM, a division and a square root per voxel and
// iteration), and batches of a few hundred thousand voxels solved side by
// side on several streams (the pipeline's chunks) hide the one-step
// latency, where this kernel's large blocks only crowd the SMs.
constexpr long long kBistochTBMaxVoxels = 1ll << 18;

__global__ void __launch_bounds__(kTBThreads, 1)
    k_bistoch_tb(const HInst* __restrict__ insts, const float* __restrict__ src,
                 float* __restrict__ dst, const float* __restrict__ count, int it0,
                 int steps, const CUtensorMap* __restrict__ msrc,
                 const CUtensorMap* __restrict__ mcnt) {
  pdl_wait_then_release();  // launched as a dependent of the previous pass
  extern __shared__ __align__(128) float tb_s[];
  float* Cs = tb_s + 2 * kTBPlane;  // counts of the block's columns
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(tb_s + 3 * kTBPlane);
  const HInst I = insts[blockIdx.y];
  const int gx = I.gx, gy = I.gy, gl = I.gl;  // gl <= kTBMaxGL (host checks)
  const int tiles_x = (gx + kTBT - 1) / kTBT;
  if ((int)blockIdx.x >= tiles_x * ((gy + kTBT - 1) / kTBT)) return;
  const int ty = blockIdx.x / tiles_x, tx = blockIdx.x - ty * tiles_x;
  const int c = threadIdx.x, yy = c / kTBL, xx = c - yy * kTBL;
  const int x = tx * kTBT - kTBK + xx, y = ty * kTBT - kTBK + yy;
  const bool in = x >= 0 && x < gx && y >= 0 && y < gy;
  const bool face = (I.cov_x && x == gx && y >= 0 && y < gy) ||
                    (I.cov_y && y == gy && x >= 0 && x < gx);
  const int plane = I.px * gy, col = in ? y * I.px + x : 0;
  const long long g0 = I.grid_off + col;
  if (msrc && mcnt && (smem_u32(tb_s) & 127u) == 0) {
    // src into plane 0 (the first step's exchange then writes plane 1),
    // the counts into plane 2
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_arrive_expect_tx(bar, 2u * kTBBoxBytes);
      tma_load_3d(tb_s, msrc + blockIdx.y, tx * kTBT - kTBK, ty * kTBT - kTBK, 0, bar);
      tma_load_3d(Cs, mcnt + blockIdx.y, tx * kTBT - kTBK, ty * kTBT - kTBK, 0, bar);
    }
    const bool ok = mbar_wait_bounded(bar, 0, kTmaWaitPolls);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicAdd(&g_wait_timeouts, 1ull);
      (void)mbar_wait_bounded(bar, 0, kTmaWaitPolls);
      return;
    }
  } else {
#pragma unroll
    for (int l = 0; l < kTBMaxGL; ++l) {
      const bool v = in && l < gl;
      const long long i = g0 + (v ? (long long)l * plane : 0);
      cp_async_f32(tb_s + l * kTBThreads + c, src + i, v);
      cp_async_f32(Cs + l * kTBThreads + c, count + i, v);
    }
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
  }
  float v[kTBMaxGL];
#pragma unroll
  for (int l = 0; l < kTBMaxGL; ++l) v[l] = tb_s[l * kTBThreads + c];
  for (int k = 1; k <= steps; ++k) {
    const float pad = ((it0 + k - 1) & 1) ? 0.f : 1.f;
    const float pz = I.cov_l ? pad : 0.f;
    float* P = tb_s + (k & 1) * kTBPlane;
#pragma unroll
    for (int l = 0; l < kTBMaxGL; ++l)
      P[l * kTBThreads + c] = in ? v[l] : (face && l < gl ? pad : 0.f);
    __syncthreads();
    if (in && tb_active(xx, yy, k)) {
      float below = 0.f;
#pragma unroll
      for (int l = 0; l < kTBMaxGL; ++l) {
        if (l < gl) {
          const float* q = P + l * kTBThreads + c;
          const float vc = v[l];
          float a = q[-1];
          a += q[1];
          a += q[-kTBL];
          a += q[kTBL];
          a += below;
          a += l + 1 < gl ? v[l + 1] : pz;
          const float blurred = 2.f * vc + a;
          v[l] = __fsqrt_rn(
              __fdiv_rn(vc * (Cs[l * kTBThreads + c] + 0.00001f), blurred + 0.00001f));
          below = vc;
        }
      }
    }
  }
  if (in && xx >= kTBK && xx < kTBK + kTBT && yy >= kTBK && yy < kTBK + kTBT) {
    float* o = dst + g0;
#pragma unroll
    for (int l = 0; l < kTBMaxGL; ++l)
      if (l < gl) o[l * plane] = v[l];
  }
}

__global__ void __launch_bounds__(kTBThreads, 1)
    k_solve_tb(const HInst* __restrict__ insts, const float* __restrict__ zs,
               float* __restrict__ zd, const float* __restrict__ hs, float* __restrict__ hd,
               const float* __restrict__ norm, const float* __restrict__ b,
               const float* __restrict__ invA, float lambda, float alpha, float beta,
               int steps, float* __restrict__ rec, long long rec_stride, int rec_steps,
               TBMaps m) {
  pdl_wait_then_release();  // launched as a dependent of the previous pass
  extern __shared__ __align__(128) float tb_s[];
  float* Bs = tb_s;
  float* As = Bs + kTBPlane;
  float* R = As + kTBPlane;  // z, h, n staging; then z * n [2]
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(tb_s + 5 * kTBPlane);
  const HInst I = insts[blockIdx.y];
  const int gx = I.gx, gy = I.gy, gl = I.gl;  // gl <= kTBMaxGL (host checks)
  const int tiles_x = (gx + kTBT - 1) / kTBT;
  if ((int)blockIdx.x >= tiles_x * ((gy + kTBT - 1) / kTBT)) return;
  const int ty = blockIdx.x / tiles_x, tx = blockIdx.x - ty * tiles_x;
  const int c = threadIdx.x, yy = c / kTBL, xx = c - yy * kTBL;
  const int x = tx * kTBT - kTBK + xx, y = ty * kTBT - kTBK + yy;
  const bool in = x >= 0 && x < gx && y >= 0 && y < gy;
  const int plane = I.px * gy, col = in ? y * I.px + x : 0;
  const long long g0 = I.grid_off + col;
  if (m.b && (smem_u32(tb_s) & 127u) == 0) {
    // b, invA, z, h, n: the five consecutive plane regions from Bs
    const CUtensorMap* maps[5] = {m.b, m.a, m.z, m.h, m.n};
    if (!tb_tma_stage(maps, 5, Bs, tx * kTBT - kTBK, ty * kTBT - kTBK, bar)) return;
  } else {
#pragma unroll
    for (int l = 0; l < kTBMaxGL; ++l) {
      const bool v = in && l < gl;
      const long long i = g0 + (v ? (long long)l * plane : 0);
      cp_async_f32(R + l * kTBThreads + c, zs + i, v);
      cp_async_f32(R + kTBPlane + l * kTBThreads + c, hs + i, v);
      cp_async_f32(R + 2 * kTBPlane + l * kTBThreads + c, norm + i, v);
      cp_async_f32(Bs + l * kTBThreads + c, b + i, v);
      cp_async_f32(As + l * kTBThreads + c, invA + i, v);
    }
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
  }
  float z[kTBMaxGL], h[kTBMaxGL], n[kTBMaxGL];
#pragma unroll
  for (int l = 0; l < kTBMaxGL; ++l) {
    z[l] = R[l * kTBThreads + c];
    h[l] = R[kTBPlane + l * kTBThreads + c];
    n[l] = R[2 * kTBPlane + l * kTBThreads + c];
  }
  for (int k = 1; k <= steps; ++k) {
    float* P = R + (k & 1) * kTBPlane;
#pragma unroll
    for (int l = 0; l < kTBMaxGL; ++l) P[l * kTBThreads + c] = z[l] * n[l];
    __syncthreads();
    if (in && tb_active(xx, yy, k)) {
      float below = 0.f, cur = z[0] * n[0];
#pragma unroll
      for (int l = 0; l < kTBMaxGL; ++l) {
        const float above = l + 1 < kTBMaxGL ? z[l + 1] * n[l + 1] : 0.f;
        const float* q = P + l * kTBThreads + c;
        const float d = q[-1] + q[1] + q[-kTBL] + q[kTBL] + below + above;
        const float qb = (Bs[l * kTBThreads + c] + lambda * n[l] * d) * As[l * kTBThreads + c];
        const float grad = z[l] - qb;
        // |grad| > 1.345 with the double threshold of the reference: the
        // smallest float above 1.345 (double) is 1.345f
        const float gc = fabsf(grad) >= 1.345f ? copysignf(1.f, grad) : grad;
        h[l] = __fmaf_rn(beta, h[l], gc);
        z[l] = z[l] - alpha * h[l];
        below = cur;
        cur = above;
      }
    }
    // iterates kept for the adjoint: z after step k of the tile's columns
    if (k <= rec_steps && in && xx >= kTBK && xx < kTBK + kTBT && yy >= kTBK &&
        yy < kTBK + kTBT) {
      float* zr = rec + (long long)(k - 1) * rec_stride + g0;
#pragma unroll
      for (int l = 0; l < kTBMaxGL; ++l)
        if (l < gl) zr[l * plane] = z[l];
    }
  }
  if (in && xx >= kTBK && xx < kTBK + kTBT && yy >= kTBK && yy < kTBK + kTBT) {
    float* zo = zd + g0;
    float* ho = hd + g0;
#pragma unroll
    for (int l = 0; l < kTBMaxGL; ++l)
      if (l < gl) {
        zo[l * plane] = z[l];
        ho[l * plane] = h[l];
      }
  }
}

// a16 as k_solve_tb (the same K-step blocks, the same arithmetic in the
// same order: bitwise the same z and h), in a persistent form that keeps the
// SM busy while a block is staged.  One CTA per SM walks the launch's
// blocks L = blockIdx.x, + gridDim.x, ... (the blocks of the (tile,
// instance) grid that lie inside their instance).  Shared memory: the z, n
// staging area (two planes), the current block's b and invA (two planes)
// and the z * n exchange (two planes, alternating by step).  As soon as a
// block's z and n are in registers, the next block's are requested by TMA
// into the staging area, so that they arrive while this block is solved;
// the next b and invA are requested after this block's last step, and a
// block's h (read by its own column's thread only) comes straight from
// global memory into registers, in flight during the first exchange.  Each
// of the two mbarriers completes once per block, so both are waited for
// with the parity of the block's position in the CTA's walk.  A wait that
// runs out (bounded) is counted in g_wait_timeouts (as is a shared-memory
// base that TMA cannot write to); the CTA then waits, bounded, for its
// copies in flight and returns.
constexpr size_t kTBPSmem = sizeof(float) * 6 * kTBPlane + 32;
// registers a thread: warps take registers in groups of four, so the 18
// warps of a block count as 20 and 65536 / 640 leaves 96
constexpr int kTBPRegs = 96;
static_assert(kTBPRegs * 640 <= 65536, "one CTA per SM");

__global__ void __maxnreg__(kTBPRegs)
    k_solve_tbp(const HInst* __restrict__ insts, int n_inst, int tiles_max,
                float* __restrict__ zd, const float* __restrict__ hs, float* __restrict__ hd,
                float lambda, float alpha, float beta, int steps, TBMaps m) {
  pdl_wait_then_release();  // launched as a dependent of the previous pass
  extern __shared__ __align__(128) float tb_s[];
  float* ZS = tb_s;                 // z, n of the block being staged
  float* Bs = tb_s + 2 * kTBPlane;  // b, invA of the current block
  float* As = Bs + kTBPlane;
  float* PP = tb_s + 4 * kTBPlane;  // z * n of a step, two buffers
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(tb_s + 6 * kTBPlane);
  const int c = threadIdx.x, yy = c / kTBL, xx = c - yy * kTBL;
  const long long total = (long long)tiles_max * n_inst;
  // block L: instance and tile
  auto decode = [&](long long L, int& inst, int& tx, int& ty) -> bool {
    inst = (int)(L / tiles_max);
    const int t = (int)(L - (long long)inst * tiles_max);
    const int gx = insts[inst].gx, gy = insts[inst].gy;
    const int tiles_x = (gx + kTBT - 1) / kTBT;
    ty = t / tiles_x;
    tx = t - ty * tiles_x;
    return t < tiles_x * ((gy + kTBT - 1) / kTBT);
  };
  // the first block inside its instance at or after L in this CTA's walk
  auto next_block = [&](long long L) -> long long {
    int i, tx, ty;
    for (; L < total; L += gridDim.x)
      if (decode(L, i, tx, ty)) return L;
    return -1;
  };
  auto issue_zn = [&](long long L) {  // thread 0
    int i, tx, ty;
    decode(L, i, tx, ty);
    const int x0 = tx * kTBT - kTBK, y0 = ty * kTBT - kTBK;
    mbar_arrive_expect_tx(&bar[0], 2u * kTBBoxBytes);
    tma_load_3d(ZS, m.z + i, x0, y0, 0, &bar[0]);
    tma_load_3d(ZS + kTBPlane, m.n + i, x0, y0, 0, &bar[0]);
  };
  auto issue_ba = [&](long long L) {  // thread 0
    int i, tx, ty;
    decode(L, i, tx, ty);
    const int x0 = tx * kTBT - kTBK, y0 = ty * kTBT - kTBK;
    mbar_arrive_expect_tx(&bar[1], 2u * kTBBoxBytes);
    tma_load_3d(Bs, m.b + i, x0, y0, 0, &bar[1]);
    tma_load_3d(As, m.a + i, x0, y0, 0, &bar[1]);
  };
  long long L = next_block(blockIdx.x);
  if (L < 0) return;
  if ((smem_u32(tb_s) & 127u) != 0) {  // TMA destinations need 128-byte alignment
    if (c == 0) atomicAdd(&g_wait_timeouts, 1ull);
    return;
  }
  if (c == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (c == 0) {
    issue_zn(L);
    issue_ba(L);
  }
  unsigned ph = 0;  // parity of this block's phase of both barriers
  for (;;) {
    int inst, tx, ty;
    decode(L, inst, tx, ty);
    const HInst& I = insts[inst];
    const int gx = I.gx, gy = I.gy, gl = I.gl;
    const int x = tx * kTBT - kTBK + xx, y = ty * kTBT - kTBK + yy;
    const bool in = x >= 0 && x < gx && y >= 0 && y < gy;
    const int plane = I.px * gy, col = in ? y * I.px + x : 0;
    const long long g0 = I.grid_off + col;
    // h straight into registers (zero outside the grid and above level gl,
    // as the staged planes read there)
    float h[kTBMaxGL];
#pragma unroll
    for (int l = 0; l < kTBMaxGL; ++l) h[l] = in && l < gl ? hs[g0 + (long long)l * plane] : 0.f;
    // this block's z, n
    const bool ok0 = mbar_wait_bounded(&bar[0], ph, kTmaWaitPolls);
    if (__syncthreads_or(!ok0)) {
      if (c == 0) atomicAdd(&g_wait_timeouts, 1ull);
      (void)mbar_wait_bounded(&bar[0], ph, kTmaWaitPolls);  // copies may still land
      (void)mbar_wait_bounded(&bar[1], ph, kTmaWaitPolls);
      return;
    }
    float z[kTBMaxGL], n[kTBMaxGL];
#pragma unroll
    for (int l = 0; l < kTBMaxGL; ++l) {
      z[l] = ZS[l * kTBThreads + c];
      n[l] = ZS[kTBPlane + l * kTBThreads + c];
    }
    __syncthreads();  // the staging area is free
    const long long Ln = next_block(L + gridDim.x);
    if (c == 0 && Ln >= 0) {
      fence_proxy_async_shared();
      issue_zn(Ln);
    }
    // this block's b, invA
    const bool ok1 = mbar_wait_bounded(&bar[1], ph, kTmaWaitPolls);
    if (__syncthreads_or(!ok1)) {
      if (c == 0) atomicAdd(&g_wait_timeouts, 1ull);
      (void)mbar_wait_bounded(&bar[1], ph, kTmaWaitPolls);
      if (Ln >= 0) (void)mbar_wait_bounded(&bar[0], ph ^ 1u, kTmaWaitPolls);
      return;
    }
    for (int k = 1; k <= steps; ++k) {
      float* P = PP + (k & 1) * kTBPlane;
#pragma unroll
      for (int l = 0; l < kTBMaxGL; ++l) P[l * kTBThreads + c] = z[l] * n[l];
      __syncthreads();
      if (in && tb_active(xx, yy, k)) {
        float below = 0.f, cur = z[0] * n[0];
#pragma unroll
        for (int l = 0; l < kTBMaxGL; ++l) {
          const float above = l + 1 < kTBMaxGL ? z[l + 1] * n[l + 1] : 0.f;
          const float* q = P + l * kTBThreads + c;
          const float d = q[-1] + q[1] + q[-kTBL] + q[kTBL] + below + above;
          const float qb = (Bs[l * kTBThreads + c] + lambda * n[l] * d) * As[l * kTBThreads + c];
          const float grad = z[l] - qb;
          // |grad| > 1.345 with the double threshold of the reference: the
          // smallest float above 1.345 (double) is 1.345f
          const float gc = fabsf(grad) >= 1.345f ? copysignf(1.f, grad) : grad;
          h[l] = __fmaf_rn(beta, h[l], gc);
          z[l] = z[l] - alpha * h[l];
          below = cur;
          cur = above;
        }
      }
    }
    __syncthreads();  // b, invA and the exchange buffers read
    if (c == 0 && Ln >= 0) {
      fence_proxy_async_shared();
      issue_ba(Ln);
    }
    if (in && xx >= kTBK && xx < kTBK + kTBT && yy >= kTBK && yy < kTBK + kTBT) {
      float* zo = zd + g0;
      float* ho = hd + g0;
#pragma unroll
      for (int l = 0; l < kTBMaxGL; ++l)
        if (l < gl) {
          zo[l * plane] = z[l];
          ho[l * plane] = h[l];
        }
    }
    if (Ln < 0) return;
    L = Ln;
    ph ^= 1u;
  }
}

constexpr int kSliceXTable = 2048;

// The slice's corner values, once per solve: (count * z, count) at every
// voxel of (gx + 1) x (gy + 1) x (gl + 2), the overflow counts (times a zero
// z, as the reference's read past the grid gives) in plane gl and zeros on
// the faces past the grid, so that the slice reads its eight corners without
// tests.  count * z is the product the reference forms first.  One warp per
// (y, l) row of the padded grid.
__global__ void k_slice_pack(const HInst* __restrict__ insts, const float* __restrict__ count,
                             const float* __restrict__ ovf, const float* __restrict__ z,
                             float2* __restrict__ sgrid) {
  const HInst I = insts[blockIdx.y];
  const int PX = I.gx + 1, PY = I.gy + 1, rows = PY * (I.gl + 2);
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < rows; row += nwarps) {
    const int iz = row / PY, iy = row - iz * PY;
    float2* out = sgrid + I.slice_off + (long long)row * PX;
    for (int ix = lane; ix < PX; ix += 32) {
      float2 v = make_float2(0.f, 0.f);
      if (ix < I.gx && iy < I.gy) {
        if (iz < I.gl) {
          const long long g = gidx(I, ix, iy, iz);
          const float c = count[g];
          v = make_float2(c * z[g], c);
        } else if (iz == I.gl) {
          const float c = ovf[I.plane_off + (long long)iy * I.gx + ix];
          v = make_float2(c * 0.f, c);
        }
      }
      out[ix] = v;
    }
  }
}

__device__ __forceinline__ float slice_pixel(const HInst& I, const float2* __restrict__ sgrid,
                                             const HParams& p, int x, float fy, float fz,
                                             const float* fxt) {
  // x * 1.0f / sigma_x from the block's table where it covers x
  const float fx = x < kSliceXTable ? fxt[x] : (float)x * 1.0f / p.sigma_x;
  const float x0 = floorf(fx), y0 = floorf(fy), z0 = floorf(fz);
  const float wx = fx - x0, wy = fy - y0, wz = fz - z0;
  // x < W puts floor(x / sx) below gx (and likewise y, and L <= 255 puts
  // floor(L / sl) at most gl); the clamps only keep the reads inside the
  // padded grid
  const int ix = min((int)x0, I.gx - 1), iy = min((int)y0, I.gy - 1),
            iz = min((int)z0, I.gl);
  const int PX = I.gx + 1, PXY = PX * (I.gy + 1);
  const float2* c0 = sgrid + I.slice_off + (long long)iz * PXY + iy * PX + ix;
  float2 v[2][2][2];  // the eight corners' loads, all issued before the weighting
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) v[dz][dy][dx] = c0[dz * PXY + dy * PX + dx];
  float num[2][2], den[2][2];
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy) {
      float ns = 0.f, ds = 0.f;
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const float w = dx ? wx : 1.f - wx;
        ns += v[dz][dy][dx].x * w;
        ds += v[dz][dy][dx].y * w;
      }
      num[dz][dy] = ns;
      den[dz][dy] = ds;
    }
  const float c0y = num[0][0] * (1.f - wy) + num[0][1] * wy;
  const float c1y = num[1][0] * (1.f - wy) + num[1][1] * wy;
  const float c0m = den[0][0] * (1.f - wy) + den[0][1] * wy;
  const float c1m = den[1][0] * (1.f - wy) + den[1][1] * wy;
  return __fdiv_rn(c0y * (1.f - wz) + c1y * wz, c0m * (1.f - wz) + c1m * wz);
}

// a17: SliceSolution<true> (src/hfbs.cu:246-330): count-weighted trilinear
// interpolation of z at (x/sx, y/sy, L/sl).  One warp per image row, lanes
// along x, two pixels per lane per pass.
__global__ void k_slice(const HInst* __restrict__ insts,
                        const uchar4* __restrict__ guide,
                        const float2* __restrict__ sgrid, float* __restrict__ out,
                        HParams p) {
  // the reference's x/sx and L/sl (correctly rounded divisions) are the same
  // for every row: computed once per block into tables
  __shared__ float fxt[kSliceXTable];
  __shared__ float fzt[256];
  const HInst I = insts[blockIdx.y];
  for (int i = threadIdx.x; i < min(I.w, kSliceXTable); i += blockDim.x)
    fxt[i] = (float)i * 1.0f / p.sigma_x;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) fzt[i] = (float)i * 1.0f / p.sigma_l;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const uchar4* g = guide + I.pix_off;
  float* o = out + I.pix_off;
  for (int y = blockIdx.x * wpb + (threadIdx.x >> 5); y < I.h; y += gridDim.x * wpb) {
    const int row = y * I.pitch;
    const float fy = (float)y * 1.0f / p.sigma_y;
    // four pixels per lane per pass: their 32 corner loads are in flight
    // together
    for (int xb = lane; xb < I.w; xb += 128) {
      float zq[4], rq[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = xb + 32 * u;
        zq[u] = x < I.w ? fzt[g[row + x].x] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = min(xb + 32 * u, I.w - 1);  // past the width: a copy of the last
        rq[u] = slice_pixel(I, sgrid, p, x, fy, zq[u], fxt);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (xb + 32 * u < I.w) o[row + xb + 32 * u] = rq[u];
    }
  }
}

// The table of tensor maps of grid plane `plane` over B's instances (TMA
// boxes of the temporally blocked kernels), or null.
const CUtensorMap* grid_map(const HfbsBatch& B, const float* plane, cudaStream_t s) {
  if (!B.tma || !B.h_inst || B.max_gl > kTBMaxGL) return nullptr;
  std::vector<TmaGrid> g(B.n_inst);
  for (int i = 0; i < B.n_inst; ++i) {
    const HInst& H = B.h_inst[i];
    g[i] = TmaGrid{H.grid_off, H.gx, H.gy, H.gl, H.px};
  }
  return B.tma->get_grid(g.data(), B.n_inst, plane, kTBL, kTBL, kTBMaxGL, s);
}

// The five tables of a temporally blocked heavy-ball launch over the
// instances from `first`; all null when any is missing.
TBMaps tb_maps(const HfbsBatch& B, int first, const float* zs, const float* hs,
               const float* norm, cudaStream_t s) {
  const float* planes[5] = {B.b, B.invA, zs, hs, norm};
  const CUtensorMap* t[5];
  for (int k = 0; k < 5; ++k)
    if (!(t[k] = grid_map(B, planes[k], s))) return TBMaps{};
  return TBMaps{t[0] + first, t[1] + first, t[2] + first, t[3] + first, t[4] + first};
}

int blocks_for(long long n) {
  long long b = (n + kT - 1) / kT;
  if (b > 152 * 8) b = 152 * 8;
  return b < 1 ? 1 : (int)b;
}

}  // namespace

unsigned long long hfbs_wait_timeouts() {
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_wait_timeouts, sizeof v) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return v;
}

void hfbs_prepare_tma(const HfbsBatch& B, cudaStream_t s) {
  for (const float* p : {(const float*)B.b, (const float*)B.invA, (const float*)B.z0,
                         (const float*)B.z1, (const float*)B.h, (const float*)B.t2,
                         (const float*)B.n0, (const float*)B.n1, (const float*)B.count})
    (void)grid_map(B, p, s);
}

bool hfbs_uses_tb(const HfbsBatch& B) {
  return B.max_gl <= kTBMaxGL && B.h_inst && B.solve_steps != 1;
}

void hfbs_launch_steps(const HfbsBatch& B, const HParams& p, const float* norm,
                       const float* zs, float* zd, const float* hs, float* hd, int steps,
                       float* rec, int rec_steps, cudaStream_t s) {
  prof_begin(s, DTSGB_K_HFBS_SOLVE);
  if (hfbs_uses_tb(B)) {
    long long tiles = 1;
    for (int i = 0; i < B.n_inst; ++i) {
      const HInst& H = B.h_inst[i];
      tiles = std::max(tiles, (long long)((H.gx + kTBT - 1) / kTBT) * ((H.gy + kTBT - 1) / kTBT));
    }
    cudaFuncSetAttribute(k_solve_tb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTBSmem);
    k_solve_tb<<<dim3((unsigned)tiles, B.n_inst), kTBThreads, kTBSmem, s>>>(
        B.d_inst, zs, zd, hs, hd, norm, B.b, B.invA, p.lambda, p.alpha, p.beta, steps, rec,
        B.total_voxels, rec_steps, tb_maps(B, 0, zs, hs, norm, s));
  } else {
    // one step; h in place (hs == hd)
    const dim3 gr((unsigned)std::min<long long>((B.max_rows + 7) / 8, 4096), B.n_inst);
    k_solve<<<gr, kT, 0, s>>>(B.d_inst, zs, zd, hd, norm, B.b, B.invA, p.lambda, p.alpha,
                              p.beta);
  }
  prof_end(s, DTSGB_K_HFBS_SOLVE);
}

void hfbs_launch_blur_pair(const HfbsBatch& B, const HParams& p, const float* s0,
                           const float* s1, float* x0, float* x1, float* y0, float* y1,
                           cudaStream_t s) {
  const dim3 gr((unsigned)std::min<long long>((B.max_rows + 7) / 8, 4096), B.n_inst);
  const dim3 gl_lines(blocks_for(B.max_lines), B.n_inst);
  k_laplace_x<<<gr, kT, 0, s>>>(B.d_inst, s0, x0, s1, x1, p.neg_exp_beta);
  k_laplace<<<gl_lines, kT, 0, s>>>(B.d_inst, 1, x0, y0, x1, y1, p.neg_exp_beta);
  k_laplace<<<gl_lines, kT, 0, s>>>(B.d_inst, 2, y0, x0, y1, x1, p.neg_exp_beta);
}

int hfbs_enqueue_solve(const HfbsBatch& B, const HParams& p, cudaStream_t s) {
  const int ni = B.n_inst;
  // row kernels: one warp per grid row, 8 warps per block
  const dim3 gr((unsigned)std::min<long long>((B.max_rows + 7) / 8, 4096), ni);
  // slice: one warp per image row, 8 rows per block
  long long max_h = 1;
  for (int i = 0; B.h_inst && i < ni; ++i) max_h = std::max<long long>(max_h, B.h_inst[i].h);
  if (!B.h_inst) max_h = (B.max_pixels + 31) / 32;
  const dim3 gp((unsigned)std::min<long long>((max_h + 7) / 8, 4096), ni);
  const dim3 gc((B.max_cells + 63) / 64, ni);
  const size_t splat_smem = sizeof(float) * 3 * (size_t)B.max_gl * 64;
  prof_begin(s, DTSGB_K_HFBS_SPLAT);
  if (B.st == Storage::F32) {
    if (splat_smem + sizeof(int) * 256 > 48 * 1024)  // plus the static luma table
      DTSGB_CUDA(cudaFuncSetAttribute(k_splat<float>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)splat_smem));
    k_splat<float><<<gc, 64, splat_smem, s>>>(
        B.d_inst, B.guide, (const float*)B.target, (const float*)B.conf, B.count,
        B.csum, B.b, B.ovf, p);
  } else {
    if (splat_smem + sizeof(int) * 256 > 48 * 1024)  // plus the static luma table
      DTSGB_CUDA(cudaFuncSetAttribute(k_splat<__nv_bfloat16>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)splat_smem));
    k_splat<__nv_bfloat16><<<gc, 64, splat_smem, s>>>(
        B.d_inst, B.guide, (const __nv_bfloat16*)B.target,
        (const __nv_bfloat16*)B.conf, B.count, B.csum, B.b, B.ovf, p);
  }
  DTSGB_CUDA(cudaGetLastError());
  prof_end(s, DTSGB_K_HFBS_SPLAT);
  // bistochastization ping-pong: even iterations read the buffer filled with
  // ones, whose covered pad faces hold 1
  const int gflat = blocks_for(B.total_voxels);
  if (!B.reuse_norm) k_fill_ones<<<gflat, kT, 0, s>>>(B.n0, B.total_voxels);
  // The iterative stages (bistochastization, heavy-ball) touch only their own
  // instance's grid, so they run group by group: all iterations of a group
  // of consecutive instances whose grids fit in L2 before the next group,
  // which then streams from L2 instead of HBM after its first iteration.
  struct Group {
    int first, count;
    long long cols;  // max over the group of gx * gy
  };
  std::vector<Group> groups;
  if (B.h_inst && B.group_voxels > 0 && !B.grad) {
    Group g{0, 0, 0};
    long long vox = 0;
    for (int i = 0; i < ni; ++i) {
      const HInst& H = B.h_inst[i];
      const long long v = (long long)H.gx * H.gy * H.gl;
      if (g.count > 0 && vox + v > B.group_voxels) {
        groups.push_back(g);
        g = Group{i, 0, 0};
        vox = 0;
      }
      ++g.count;
      vox += v;
      g.cols = std::max(g.cols, (long long)H.gx * H.gy);
    }
    groups.push_back(g);
  } else {
    groups.push_back(Group{0, ni, B.max_cells});
  }
  // column kernels (bistochastization): one thread per (x, y)
  auto col_grid = [](const Group& g) {
    return dim3((unsigned)std::min<long long>((g.cols + kT - 1) / kT, 4096), g.count);
  };
  float* src = B.n0;
  float* dst = B.n1;
  for (const Group& g : groups) {
    src = B.n0;
    dst = B.n1;
    if (B.reuse_norm) {
      if (p.bistoch_iter_max % 2) std::swap(src, dst);
      continue;
    }
    long long gvox = 0;  // the group's voxels
    for (int i = 0; B.h_inst && i < g.count; ++i) {
      const HInst& H = B.h_inst[g.first + i];
      gvox += (long long)H.gx * H.gy * H.gl;
    }
    if (hfbs_uses_tb(B) && gvox <= kBistochTBMaxVoxels) {
      // up to kTBK iterations per pass; one pass split in two when the number
      // of passes and of iterations differ in parity, so that the result
      // lands in the buffer the one-step ping-pong leaves it in
      std::vector<int> plan;
      for (int r = p.bistoch_iter_max; r > 0; r -= kTBK) plan.push_back(std::min(kTBK, r));
      if ((int)(plan.size() % 2) != p.bistoch_iter_max % 2) {
        for (int i = (int)plan.size() - 1; i >= 0; --i)
          if (plan[i] >= 2) {
            const int a = plan[i] / 2;
            plan[i] -= a;
            plan.insert(plan.begin() + i + 1, a);
            break;
          }
      }
      long long tiles = 1;
      for (int i = 0; i < g.count; ++i) {
        const HInst& H = B.h_inst[g.first + i];
        tiles = std::max(tiles, (long long)((H.gx + kTBT - 1) / kTBT) * ((H.gy + kTBT - 1) / kTBT));
      }
      DTSGB_CUDA(cudaFuncSetAttribute(k_bistoch_tb, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kTBBistochSmem));
      int it0 = 0;
      for (int steps : plan) {
        const CUtensorMap* ms = grid_map(B, src, s);
        const CUtensorMap* mc = ms ? grid_map(B, B.count, s) : nullptr;
        if (!mc) ms = nullptr;
        prof_begin(s, DTSGB_K_HFBS_BISTOCH);
        DTSGB_CUDA(launch_dependent(k_bistoch_tb, dim3((unsigned)tiles, g.count),
                                    dim3(kTBThreads), kTBBistochSmem, s, B.d_inst + g.first,
                                    src, dst, B.count, it0, steps, ms ? ms + g.first : nullptr,
                                    mc ? mc + g.first : nullptr));
        prof_end(s, DTSGB_K_HFBS_BISTOCH);
        std::swap(src, dst);
        it0 += steps;
      }
    } else {
      for (int it = 0; it < p.bistoch_iter_max; ++it) {
        prof_begin(s, DTSGB_K_HFBS_BISTOCH);
        DTSGB_CUDA(launch_dependent(k_bistoch, col_grid(g), dim3(kT), 0, s, B.d_inst + g.first,
                                    src, dst, B.count, (it % 2 == 0) ? 1.f : 0.f));
        prof_end(s, DTSGB_K_HFBS_BISTOCH);
        std::swap(src, dst);
      }
    }
  }
  float* norm = src;
  float* spare = dst;
  prof_begin(s, DTSGB_K_HFBS_OTHER);
  k_inv_diag<<<gflat, kT, 0, s>>>(B.count, B.csum, norm, B.invA, p.lambda,
                                  B.total_voxels);
  // Laplace blur of (c, b): X -> Y -> Z.
  const dim3 gl_lines(blocks_for(B.max_lines), ni);
  k_laplace_x<<<gr, kT, 0, s>>>(B.d_inst, B.csum, B.t0, B.b, B.t1, p.neg_exp_beta);
  k_laplace<<<gl_lines, kT, 0, s>>>(B.d_inst, 1, B.t0, B.t2, B.t1, spare,
                                    p.neg_exp_beta);
  k_laplace<<<gl_lines, kT, 0, s>>>(B.d_inst, 2, B.t2, B.t0, spare, B.t1,
                                    p.neg_exp_beta);
  // blur_c = t0, blur_b = t1
  k_init_z<<<gflat, kT, 0, s>>>(B.t1, B.t0, B.z0, B.h, B.total_voxels);
  prof_end(s, DTSGB_K_HFBS_OTHER);
  if (B.keep_debug) {
    DTSGB_CUDA(cudaMemcpyAsync(B.dbg_blur_c, B.t0, B.grid_bytes,
                               cudaMemcpyDeviceToDevice, s));
    DTSGB_CUDA(cudaMemcpyAsync(B.dbg_z_init, B.z0, B.grid_bytes,
                               cudaMemcpyDeviceToDevice, s));
    DTSGB_CUDA(cudaMemcpyAsync(B.dbg_norm, norm, B.grid_bytes,
                               cudaMemcpyDeviceToDevice, s));
  }
  float* zs = B.z0;
  float* zd = B.z1;
  if (B.grad) {
    // iterates kept for the adjoint (HfbsGradState)
    const HfbsGradState& G = *B.grad;
    const int K = p.optim_iter_max, S = G.segment;
    const bool tb = hfbs_uses_tb(B);
    const long long tv = B.total_voxels;
    const size_t gbytes = (size_t)tv * sizeof(float);
    if (S == 1) {
      // z_k in hist plane k; h ping-pongs through the free blur temporary t2
      if (K > 0)
        DTSGB_CUDA(cudaMemcpyAsync(G.hist, B.z0, gbytes, cudaMemcpyDeviceToDevice, s));
      float* hs = B.h;
      float* hd = tb ? B.t2 : B.h;
      for (int it = 0; it < K;) {
        const int steps = tb ? std::min(kTBK, K - it) : 1;
        float* zout = it + steps < K ? G.hist + (size_t)(it + steps) * tv : B.z1;
        const int rec_steps = tb ? std::min(steps, K - 1 - it) : 0;
        hfbs_launch_steps(B, p, norm, G.hist + (size_t)it * tv, zout, hs, hd, steps,
                          G.hist + (size_t)(it + 1) * tv, rec_steps, s);
        std::swap(hs, hd);
        it += steps;
      }
      zs = K > 0 ? B.z1 : B.z0;
    } else {
      // z and h at the start of every segment
      float* hs = B.h;
      float* hd = tb ? B.t2 : B.h;
      for (int it = 0; it < K;) {
        if (it % S == 0) {
          DTSGB_CUDA(cudaMemcpyAsync(G.ckz + (size_t)(it / S) * tv, zs, gbytes,
                                     cudaMemcpyDeviceToDevice, s));
          DTSGB_CUDA(cudaMemcpyAsync(G.ckh + (size_t)(it / S) * tv, hs, gbytes,
                                     cudaMemcpyDeviceToDevice, s));
        }
        const int steps = tb ? std::min({kTBK, K - it, S - it % S}) : 1;
        hfbs_launch_steps(B, p, norm, zs, zd, hs, hd, steps, nullptr, 0, s);
        std::swap(zs, zd);
        std::swap(hs, hd);
        it += steps;
      }
    }
  } else if (hfbs_uses_tb(B)) {
    // K heavy-ball steps per pass; h ping-pongs through the free blur
    // temporary t2 (its final value is not needed).  The shared-memory limit
    // is a per-device attribute: set on every call (host-side, cheap).
    DTSGB_CUDA(cudaFuncSetAttribute(k_solve_tb, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kTBSmem));
    DTSGB_CUDA(cudaFuncSetAttribute(k_solve_tbp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kTBPSmem));
    // SMs for the persistent form, 0 when it cannot be resident (then the
    // kernel with one CTA per block runs)
    static const int sms = [] {
      int dev = 0, n = 0, per_sm = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_tbp, kTBThreads,
                                                        kTBPSmem) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
      }
      return per_sm >= 1 ? n : 0;
    }();
    for (const Group& g : groups) {
      zs = B.z0;
      zd = B.z1;
      float* hs = B.h;
      float* hd = B.t2;
      long long tiles = 1;
      for (int i = 0; i < g.count; ++i) {
        const HInst& H = B.h_inst[g.first + i];
        tiles = std::max(tiles, (long long)((H.gx + kTBT - 1) / kTBT) * ((H.gy + kTBT - 1) / kTBT));
      }
      const dim3 gt((unsigned)tiles, g.count);
      // the persistent form with tensor maps, one CTA per SM; else one CTA
      // per block
      const unsigned gp = (unsigned)std::min<long long>(tiles * g.count, sms > 0 ? sms : 1);
      for (int it = 0; it < p.optim_iter_max; it += kTBK) {
        const int steps = std::min(kTBK, p.optim_iter_max - it);
        const TBMaps maps = tb_maps(B, g.first, zs, hs, norm, s);
        prof_begin(s, DTSGB_K_HFBS_SOLVE);
        if (maps.b && sms > 0)
          DTSGB_CUDA(launch_dependent(k_solve_tbp, dim3(gp), dim3(kTBThreads), kTBPSmem, s,
                                      B.d_inst + g.first, g.count, (int)tiles, zd, hs, hd,
                                      p.lambda, p.alpha, p.beta, steps, maps));
        else
          DTSGB_CUDA(launch_dependent(k_solve_tb, gt, dim3(kTBThreads), kTBSmem, s,
                                      B.d_inst + g.first, zs, zd, hs, hd, norm, B.b, B.invA,
                                      p.lambda, p.alpha, p.beta, steps, (float*)nullptr, 0LL,
                                      0, maps));
        prof_end(s, DTSGB_K_HFBS_SOLVE);
        std::swap(zs, zd);
        std::swap(hs, hd);
      }
    }
  } else
  for (const Group& g : groups) {
    zs = B.z0;
    zd = B.z1;
    long long rows = 0;  // one warp per grid row (y, l) of the group's largest grid
    for (int i = 0; i < g.count; ++i)
      rows = B.h_inst ? std::max(rows, (long long)B.h_inst[g.first + i].gy *
                                           B.h_inst[g.first + i].gl)
                      : B.max_rows;
    const dim3 gr_g((unsigned)std::min<long long>((rows + 7) / 8, 4096), g.count);
    for (int it = 0; it < p.optim_iter_max; ++it) {
      prof_begin(s, DTSGB_K_HFBS_SOLVE);
      k_solve<<<gr_g, kT, 0, s>>>(B.d_inst + g.first, zs, zd, B.h, norm, B.b, B.invA,
                                  p.lambda, p.alpha, p.beta);
      prof_end(s, DTSGB_K_HFBS_SOLVE);
      std::swap(zs, zd);
    }
  }
  if (B.keep_debug)
    DTSGB_CUDA(cudaMemcpyAsync(B.dbg_z_final, zs, B.grid_bytes,
                               cudaMemcpyDeviceToDevice, s));
  prof_begin(s, DTSGB_K_HFBS_SLICE);
  long long prows = 1;  // rows of the largest padded slice grid
  for (int i = 0; B.h_inst && i < ni; ++i)
    prows = std::max<long long>(prows, (long long)(B.h_inst[i].gy + 1) * (B.h_inst[i].gl + 2));
  if (!B.h_inst) prows = B.max_lines + 2 * B.max_rows + 260;
  const dim3 gsl((unsigned)std::min<long long>((prows + 7) / 8, 4096), ni);
  k_slice_pack<<<gsl, kT, 0, s>>>(B.d_inst, B.count, B.ovf, zs, B.sgrid);
  k_slice<<<gp, kT, 0, s>>>(B.d_inst, B.guide, B.sgrid, B.out, p);
  prof_end(s, DTSGB_K_HFBS_SLICE);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

}  // namespace dtsgb
