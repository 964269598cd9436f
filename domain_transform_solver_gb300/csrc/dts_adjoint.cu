// Adjoint of the fixed-iteration DTS solve (no reference counterpart: the
// reference has no gradients).  With the windows fixed, one iteration is
//   X: v1 = v - s*(lambda*(v - Bx v) + h(v)),  h = (c/n)(v - t)            (L2)
//                                              h = 0.5 (c/n)(v-t)/sqrt((v-t)^2+e)
//   Y: v2 = v1 - s*lambda*(v1 - By v1)
// so, for an upstream gradient g2 = dL/dv2,
//   g1 = (1 - s*lambda) g2 + s*lambda * By^T g2
//   g  = (1 - s*lambda - s*h'(v)) g1 + s*lambda * Bx^T g1
//   dL/dt += s*h'(v) g1 (and g at v_0 = t),  dL/dc += -s*(dh/dc) g1.
// B^T a at q is the sum of a(p)/n(p) over the pixels p whose window holds q.
// Each p adds its term to the interval of its window: +a at the first pixel
// of the window (clipped to the tile), -a after the last, and a prefix sum
// over the difference array gives B^T.  The terms are fixed-point integers
// (fixed_point.cuh) added with wrapping 32-bit arithmetic, so the
// shared-memory atomics that build the difference array are exact and their
// order does not matter: the result is deterministic.
// One kernel does Y^T for the tile rows over the tile columns plus the X
// halo, then X^T for the tile, mirroring the forward kernel's X-then-Y tile.
//
// The forward iterates the adjoint needs (the X-step inputs v_k) are
// recomputed segment by segment from checkpoints v_0 = t, v_K, v_2K, ...
// saved by the forward, so memory grows with sqrt(N), not N.
#include <algorithm>

#include "../../include/dtsgb.h"
#include "dtsgb_internal.cuh"
#include "fixed_point.cuh"

namespace dtsgb {
namespace {

constexpr int kT = 256;
constexpr int kAdjFirst = 1, kAdjLast = 2;


// Shared-memory layout (byte offsets, 16-byte aligned regions).
template <int TW, int TH, int NT>
struct AdjSmem {
  size_t s2, by, d, seg, rt, mx, total;
  AdjSmem(int hx, int hy) {
    const size_t SR = TH + 2 * hy, SWc = TW + 2 * hx;
    const size_t nseg = std::max<size_t>(1, NT / SWc);
    auto up = [](size_t v) { return (v + 15) / 16 * 16; };
    // The Y bounds (By), the Y segment totals and the X buffers are alive in
    // turn (By until the scatter, the totals in the column prefix, the X
    // buffers in X^T) and share one region; this keeps the 64 x 128 tile of
    // sigma_z = 8 within two CTAs per SM.
    s2 = 0;                                                    // SR x SWc f32
    by = up(s2 + SR * SWc * 4);                                // By | totals | X buffers
    seg = by;                                                  // nseg x SWc u32
    d = up(by + std::max({SR * SWc * 2, (size_t)(NT / 32) * (TW + 1) * 4,
                          nseg * SWc * 4}));
    rt = up(d + (size_t)(TH + 1) * SWc * 4);                   // (TH+1) x SWc u32 at d
    mx = up(rt + (size_t)(2 * std::max(hx, hy) + 2) * 4);
    total = mx + 16;
  }
};

template <typename TS, int MODE, int TW, int TH, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT)
    k_dts_adjoint(const Inst* __restrict__ insts, const Tile* __restrict__ tiles,
                  const float* __restrict__ gin, float* __restrict__ gout,
                  const float* __restrict__ vk, const TS* __restrict__ tgt,
                  const TS* __restrict__ cnf, const uint32_t* __restrict__ bnd,
                  float* __restrict__ grad_t, float* __restrict__ grad_c,
                  float lambda, float step, int hx, int hy, int flags,
                  AdjSmem<TW, TH, NT> L) {
  // flags: kAdjFirst, the first adjoint of a backward (dL/dt and dL/dc start
  // at zero: not read); kAdjLast, the last (its dL/dv_0 goes into dL/dt, as
  // v_0 = t, instead of to gout)
  const bool first = flags & kAdjFirst, last = flags & kAdjLast;
  constexpr int NW = NT / 32;
  extern __shared__ __align__(16) unsigned char smraw[];
  const Tile t = tiles[blockIdx.x];
  const Inst in = insts[t.inst];
  const int W = in.w, H = in.h, P = in.pitch;
  const int SR = TH + 2 * hy, SWc = TW + 2 * hx;
  const int NSEG = max(1, NT / SWc);
  float* S2 = reinterpret_cast<float*>(smraw + L.s2);  // a2 = g2/n_y, then g1
  uint16_t* By = reinterpret_cast<uint16_t*>(smraw + L.by);
  unsigned* Xb = reinterpret_cast<unsigned*>(smraw + L.by);  // X phase, per warp
  unsigned* D = reinterpret_cast<unsigned*>(smraw + L.d);
  unsigned* segtot = reinterpret_cast<unsigned*>(smraw + L.seg);
  float* rtab = reinterpret_cast<float*>(smraw + L.rt);
  unsigned* smax = reinterpret_cast<unsigned*>(smraw + L.mx);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // per-instance bases: every offset below is a 32-bit pixel index
  const float* gin_i = gin + in.off;
  float* gout_i = gout + in.off;
  const float* vk_i = vk + in.off;
  const TS* tgt_i = tgt + in.off;
  const TS* cnf_i = cnf + in.off;
  const uint32_t* bnd_i = bnd + in.off;
  float* gt_i = grad_t + in.off;
  float* gc_i = grad_c + in.off;
  const int nrt = 2 * max(hx, hy) + 2;
  for (int i = tid; i < nrt; i += NT) rtab[i] = i ? __frcp_rn((float)i) : 0.f;
  for (int i = tid; i < (TH + 1) * SWc; i += NT) D[i] = 0u;
  if (tid == 0) *smax = 0u;
  __syncthreads();
  const int gx0 = t.x0 - hx, gy0 = t.y0 - hy;
  const float slam = step * lambda;
  const int lgx = ceil_log2(2 * hx + 1), lgy = ceil_log2(2 * hy + 1);
  // ---- Y^T: a2 = g2 / n_y over the tile + halo --------------------------------
  float m = 0.f;
  // one warp per row, lanes along the row (no index divisions), two rows of
  // loads in flight
  constexpr int NWp = NT / 32;
  for (int r0 = warp; r0 < SR; r0 += 2 * NWp) {
    for (int c0 = lane; c0 < SWc; c0 += 32) {
      uint32_t bb[2];
      float gg[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int r = r0 + u * NWp, x = gx0 + c0, y = gy0 + r;
        const bool ok = r < SR && (unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H;
        const int p = y * P + x;
        bb[u] = ok ? __ldg(bnd_i + p) : 0u;
        gg[u] = ok ? __ldg(gin_i + p) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int r = r0 + u * NWp;
        if (r >= SR) break;
        const uint16_t b16 = (uint16_t)(bb[u] >> 16);
        const int n = min((int)(b16 & 0xff), hy + 1) + min((int)(b16 >> 8), hy);
        const float a = b16 ? gg[u] * rtab[n] : 0.f;
        S2[r * SWc + c0] = a;
        By[r * SWc + c0] = b16;
        m = fmaxf(m, fabsf(a));
      }
    }
  }
  m = warp_max_nonneg(m);
  if (lane == 0) atomicMax(smax, __float_as_uint(m));
  __syncthreads();
  {
    const int F = fx_shift(__uint_as_float(*smax), lgy);
    const float sF = pow2f(F);
    for (int r = warp; r < SR; r += NWp) {
      for (int c = lane; c < SWc; c += 32) {
        const int i = r * SWc + c;
        const uint16_t b16 = By[i];
        if (!b16) continue;  // outside the image (a window always holds its pixel)
        const int dl = min((int)(b16 & 0xff), hy + 1), du = min((int)(b16 >> 8), hy);
        const int lo = max(r - hy - dl + 1, 0), hi = min(r - hy + du, TH - 1);
        if (lo > hi) continue;
        const unsigned A = fx_from(S2[i], sF);
        atomicAdd(D + lo * SWc + c, A);
        atomicAdd(D + (hi + 1) * SWc + c, 0u - A);
      }
    }
    __syncthreads();
    // column prefix over the tile rows, in segments
    const int seg = (TH + NSEG - 1) / NSEG;
    for (int i = tid; i < SWc * NSEG; i += NT) {
      const int c = i % SWc, sg = i / SWc;
      const int k0 = min(sg * seg, TH), k1 = min(k0 + seg, TH);
      unsigned acc = 0;
      for (int k = k0; k < k1; ++k) {
        acc += D[k * SWc + c];
        D[k * SWc + c] = acc;
      }
      segtot[sg * SWc + c] = acc;
    }
    __syncthreads();
    const float isF = pow2f(-F);
    for (int i = tid; i < SWc * NSEG; i += NT) {
      const int c = i % SWc, sg = i / SWc;
      const int k0 = min(sg * seg, TH), k1 = min(k0 + seg, TH);
      unsigned off = 0;
      for (int s2 = 0; s2 < sg; ++s2) off += segtot[s2 * SWc + c];
      const int x = gx0 + c;
      const bool xok = (unsigned)x < (unsigned)W;
      for (int k = k0; k < k1; k += 4) {
        float gv[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int y = t.y0 + k + j;
          gv[j] = (k + j < k1 && xok && y < H) ? __ldg(gin_i + y * P + x) : 0.f;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (k + j >= k1) break;
          const int y = t.y0 + k + j;
          float g1 = 0.f;
          if (xok && y < H) {
            const float bt = fx_window(D[(k + j) * SWc + c] + off, 0u, isF);
            g1 = __fmaf_rn(1.f - slam, gv[j], slam * bt);
          }
          S2[(k + j) * SWc + c] = g1;  // g1, rows of the tile only
        }
      }
    }
  }
  __syncthreads();
  // ---- X^T and the parameter gradients: one warp per tile row ----------------
  // A warp's global loads for its next row are issued before it works on the
  // current one.  Each lane owns CPL adjacent tile columns (vector loads and
  // stores; one warp scan per row).
  constexpr int CPL = TW / 32;  // tile columns per lane, adjacent
  constexpr int BPL = 4;        // prefetched window columns per lane
  static_assert(CPL == 1 || CPL == 2, "tile width 32 or 64");
  struct RowAdj {
    uint32_t bh[BPL];  // packed bounds of window columns lane + 32j
    float v[CPL], tv[CPL], cv[CPL], gt[CPL], gc[CPL];  // tile columns CPL*lane + k
  };
  const int xl = t.x0 + CPL * lane;  // first tile column of this lane
  auto fetch = [&](int rr, RowAdj& R) {
    const int row = (t.y0 + rr) * P;
#pragma unroll
    for (int j = 0; j < BPL; ++j) {
      const int c = lane + 32 * j, x = gx0 + c;
      R.bh[j] = (c < SWc && (unsigned)x < (unsigned)W) ? __ldg(bnd_i + row + x) : 0u;
    }
    const int p = row + xl;
    if (CPL == 2 && xl + 1 < W) {  // both columns inside: 8-byte aligned pairs
      const float2 v = __ldg(reinterpret_cast<const float2*>(vk_i + p));
      const float2 g0 =
          first ? make_float2(0.f, 0.f) : *reinterpret_cast<const float2*>(gt_i + p);
      const float2 g1 =
          first ? make_float2(0.f, 0.f) : *reinterpret_cast<const float2*>(gc_i + p);
      R.v[0] = v.x;
      R.v[CPL - 1] = v.y;
      R.gt[0] = g0.x;
      R.gt[CPL - 1] = g0.y;
      R.gc[0] = g1.x;
      R.gc[CPL - 1] = g1.y;
#pragma unroll
      for (int k = 0; k < CPL; ++k) {
        R.tv[k] = load_f(tgt_i + p + k);
        R.cv[k] = load_f(cnf_i + p + k);
      }
    } else {
#pragma unroll
      for (int k = 0; k < CPL; ++k) {
        const bool ok = xl + k < W;
        R.v[k] = ok ? __ldg(vk_i + p + k) : 0.f;
        R.tv[k] = ok ? load_f(tgt_i + p + k) : 0.f;
        R.cv[k] = ok ? load_f(cnf_i + p + k) : 0.f;
        R.gt[k] = ok && !first ? gt_i[p + k] : 0.f;
        R.gc[k] = ok && !first ? gc_i[p + k] : 0.f;
      }
    }
  };
  const int rows = min(TH, H - t.y0);
  unsigned* xb = Xb + warp * (TW + 1);
  RowAdj cur, nxt;
  if (warp < rows) fetch(warp, cur);
  for (int rr = warp; rr < rows; rr += NW) {
    if (rr + NW < rows) fetch(rr + NW, nxt);
    const int row = (t.y0 + rr) * P;
    const float* g1r = S2 + rr * SWc;
    // visit(b, c) for the window columns c of this lane: the first BPL from
    // the prefetched registers, any further ones (halos above 32) reloaded
    auto for_columns = [&](auto&& visit) {
#pragma unroll
      for (int j = 0; j < BPL; ++j) {
        const int c = lane + 32 * j;
        if (c < SWc && cur.bh[j]) visit(cur.bh[j], c);
      }
      for (int c = lane + 32 * BPL; c < SWc; c += 32) {
        const int x = gx0 + c;
        if ((unsigned)x < (unsigned)W) visit(__ldg(bnd_i + row + x), c);
      }
    };
    for (int k = lane; k <= TW; k += 32) xb[k] = 0u;
    float mx = 0.f;
    for_columns([&](uint32_t b, int c) {
      const int n = min((int)(b & 0xff), hx + 1) + min((int)((b >> 8) & 0xff), hx);
      mx = fmaxf(mx, fabsf(g1r[c] * rtab[n]));
    });
    mx = warp_max_nonneg(mx);
    const int F = fx_shift(mx, lgx);
    const float sF = pow2f(F), isF = pow2f(-F);
    __syncwarp();
    for_columns([&](uint32_t b, int c) {
      const int dl = min((int)(b & 0xff), hx + 1), du = min((int)((b >> 8) & 0xff), hx);
      const int lo = max(c - hx - dl + 1, 0), hi = min(c - hx + du, TW - 1);
      if (lo > hi) return;
      const unsigned A = fx_from(g1r[c] * rtab[dl + du], sF);
      atomicAdd(xb + lo, A);
      atomicAdd(xb + hi + 1, 0u - A);
    });
    __syncwarp();
    // inclusive prefix of the difference array over this lane's columns
    unsigned incl[CPL];
    incl[0] = xb[CPL * lane];
#pragma unroll
    for (int k = 1; k < CPL; ++k) incl[k] = incl[k - 1] + xb[CPL * lane + k];
    const unsigned off = warp_incl_scan(incl[CPL - 1], lane) - incl[CPL - 1];
    float go[CPL], gtn[CPL], gcn[CPL];
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
      const int x = xl + k;
      go[k] = gtn[k] = gcn[k] = 0.f;
      if (x >= W) continue;
      const float bt = fx_window(incl[k] + off, 0u, isF);
      const float g1 = g1r[hx + CPL * lane + k];
      const uint32_t b = __ldg(bnd_i + row + x);
      const float rn = rtab[min((int)(b & 0xff), hx + 1) + min((int)((b >> 8) & 0xff), hx)];
      const float v = cur.v[k], tv = cur.tv[k], cv = cur.cv[k];
      const float d = v - tv;
      float dh_dv, dh_dc;
      if (MODE == 0) {
        dh_dv = cv * rn;
        dh_dc = d * rn;
      } else {
        const float rt = __fsqrt_rn(__fmaf_rn(d, d, 1e-6f));
        dh_dv = __fdiv_rn(0.5f * (cv * rn) * 1e-6f, rt * rt * rt);
        dh_dc = __fdiv_rn(0.5f * d * rn, rt);
      }
      go[k] = __fmaf_rn(1.f - slam - step * dh_dv, g1, slam * bt);
      gtn[k] = cur.gt[k] + step * dh_dv * g1;
      gcn[k] = cur.gc[k] - step * dh_dc * g1;
      if (last) gtn[k] += go[k];
    }
    const int p = row + xl;
    if (CPL == 2 && xl + 1 < W) {
      if (!last) *reinterpret_cast<float2*>(gout_i + p) = make_float2(go[0], go[CPL - 1]);
      *reinterpret_cast<float2*>(gt_i + p) = make_float2(gtn[0], gtn[CPL - 1]);
      *reinterpret_cast<float2*>(gc_i + p) = make_float2(gcn[0], gcn[CPL - 1]);
    } else {
#pragma unroll
      for (int k = 0; k < CPL; ++k)
        if (xl + k < W) {
          if (!last) gout_i[p + k] = go[k];
          gt_i[p + k] = gtn[k];
          gc_i[p + k] = gcn[k];
        }
    }
    __syncwarp();  // the warp's buffer is cleared for its next row
    cur = nxt;
  }
}

__global__ void k_axpy_planes(const Inst* __restrict__ insts, const float* __restrict__ a,
                              float* __restrict__ y) {
  const Inst in = insts[blockIdx.y];
  const long long n = (long long)in.pitch * in.h;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[in.off + i] += a[in.off + i];
}

template <typename TS, int MODE, int TW, int TH>
int launch_adj_shape(const DtsLaunch& L, const float* gin, float* gout, const float* vk,
                     const void* t, const void* c, const uint32_t* bounds, float* gt,
                     float* gc, float lambda, float step, int hx, int hy, int flags,
                     cudaStream_t s) {
  constexpr int NT = TW >= 64 ? 512 : 256;
  const AdjSmem<TW, TH, NT> lay(hx, hy);
  if (lay.total > 227 * 1024)
    return fail(DTSGB_ERR_UNSUPPORTED, "sigma_z too large for the adjoint");
  if (lay.total > 48 * 1024)
    DTSGB_CUDA(cudaFuncSetAttribute(k_dts_adjoint<TS, MODE, TW, TH, NT>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)lay.total));
  k_dts_adjoint<TS, MODE, TW, TH, NT><<<L.n_tiles, NT, lay.total, s>>>(
      L.d_inst, L.d_tiles, gin, gout, vk, (const TS*)t, (const TS*)c, bounds, gt, gc,
      lambda, step, hx, hy, flags, lay);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

template <typename TS, int MODE>
int launch_adj_t(const DtsLaunch& L, const float* gin, float* gout, const float* vk,
                 const void* t, const void* c, const uint32_t* bounds, float* gt, float* gc,
                 float lambda, float step, int hx, int hy, int flags, cudaStream_t s) {
  if (L.small)
    return launch_adj_shape<TS, MODE, kIterSmallTW, kIterSmallTH>(
        L, gin, gout, vk, t, c, bounds, gt, gc, lambda, step, hx, hy, flags, s);
  if (L.d_tiles_small && AdjSmem<kIterTW, kIterTH, 512>(hx, hy).total > 227 * 1024)
    return launch_adj_shape<TS, MODE, kIterSmallTW, kIterSmallTH>(
        L.as_small(), gin, gout, vk, t, c, bounds, gt, gc, lambda, step, hx, hy, flags, s);
  return launch_adj_shape<TS, MODE, kIterTW, kIterTH>(L, gin, gout, vk, t, c, bounds, gt,
                                                      gc, lambda, step, hx, hy, flags, s);
}

int launch_adjoint(const DtsLaunch& L, Storage st, IterMode mode, const float* gin,
                   float* gout, const float* vk, const void* t, const void* c,
                   const uint32_t* bounds, float* gt, float* gc, float lambda,
                   float step, int hx, int hy, int flags, cudaStream_t s) {
  ProfScope ps(s, DTSGB_K_DTS_ADJOINT);
  if (st == Storage::F32) {
    if (mode == IterMode::L2)
      return launch_adj_t<float, 0>(L, gin, gout, vk, t, c, bounds, gt, gc, lambda, step,
                                    hx, hy, flags, s);
    return launch_adj_t<float, 1>(L, gin, gout, vk, t, c, bounds, gt, gc, lambda, step, hx,
                                  hy, flags, s);
  }
  if (mode == IterMode::L2)
    return launch_adj_t<__nv_bfloat16, 0>(L, gin, gout, vk, t, c, bounds, gt, gc, lambda,
                                          step, hx, hy, flags, s);
  return launch_adj_t<__nv_bfloat16, 1>(L, gin, gout, vk, t, c, bounds, gt, gc, lambda,
                                        step, hx, hy, flags, s);
}

}  // namespace

int dts_checkpoint_segment(int num_iterations) {
  // fewest planes held (ceil(N/K) - 1 + K), and among those the fewest
  // recomputed iterations (N - ceil(N/K)): the smallest such K
  const int n = std::max(num_iterations, 1);
  int best = 1;
  long long best_planes = -1;
  for (int k = 1; k <= n; ++k) {
    const long long planes = (n + k - 1) / k - 1 + k;
    if (best_planes < 0 || planes < best_planes) {
      best_planes = planes;
      best = k;
    }
  }
  return best;
}

// Destination of the iterate v_next of an N-iteration forward from v_cur:
// -1 = checkpoint plane, else ping-pong plane 0 / 1 (never the one read).
static int forward_dst(int cur, int next, int n, int seg) {
  if (next < n && next % seg == 0) return -1;
  return cur == 0 ? 1 : 0;
}

int dts_checkpointed_result_index(int num_iterations, int seg) {
  int cur = 0;
  for (int it = 0; it < num_iterations; ++it) cur = forward_dst(cur, it + 1, num_iterations, seg);
  return cur;
}

int dts_forward_checkpointed(const DtsLaunch& L, Storage st, IterMode mode,
                             const DtsGrad& G, const void* target, const void* conf,
                             const uint32_t* bounds, float lambda, float step, int halo,
                             int num_iterations, float* v0, float* v1, int* result_idx,
                             cudaStream_t s) {
  int st_ = launch_init_var(L, st, target, v0, s);
  if (st_) return st_;
  float* buf[2] = {v0, v1};
  const float* cur = v0;
  int ci = 0;
  for (int it = 0; it < num_iterations; ++it) {
    const int next = it + 1;
    const int di = forward_dst(ci, next, num_iterations, G.seg);
    float* dst = di < 0 ? G.cp[next / G.seg - 1] : buf[di];
    st_ = launch_dts_iter(L, st, mode, cur, dst, target, conf, bounds, lambda, step, -1.f,
                          halo, halo, s);
    if (st_) return st_;
    cur = dst;
    ci = di;
  }
  // the last iteration never writes a checkpoint
  *result_idx = ci;
  return DTSGB_OK;
}

int dts_backward(const DtsLaunch& L, const Inst* d_inst, int n_inst, long long plane,
                 Storage st, IterMode mode, const DtsGrad& G, const void* target,
                 const void* conf, const uint32_t* bounds, float lambda, float step,
                 int halo, int num_iterations, float* grad_t, float* grad_c,
                 cudaStream_t s) {
  if (num_iterations <= 0) {  // v = t: dL/dt = dL/dv, dL/dc = 0
    DTSGB_CUDA(cudaMemsetAsync(grad_t, 0, plane * sizeof(float), s));
    DTSGB_CUDA(cudaMemsetAsync(grad_c, 0, plane * sizeof(float), s));
    k_axpy_planes<<<dim3(64, n_inst), kT, 0, s>>>(d_inst, G.g[0], grad_t);
    DTSGB_CUDA(cudaGetLastError());
    return DTSGB_OK;
  }
  // the first adjoint writes dL/dt and dL/dc (no zeroing pass), the last
  // adds dL/dv_0 to dL/dt (no final pass)
  float* g = G.g[0];  // holds dL/dv_N on entry
  float* gn = G.g[1];
  const int nseg = (num_iterations + G.seg - 1) / G.seg;
  for (int j = nseg - 1; j >= 0; --j) {
    const int start = j * G.seg;
    const int len = std::min(G.seg, num_iterations - start);
    // X-step inputs v_start .. v_start+len-1 of this segment: the first is
    // t (segment 0) or a checkpoint, the others are recomputed into segbuf
    const float* x0 = j == 0 ? G.segbuf[0] : G.cp[j - 1];
    if (j == 0) {
      int st_ = launch_init_var(L, st, target, G.segbuf[0], s);
      if (st_) return st_;
    }
    for (int k = 1; k < len; ++k) {
      int st_ = launch_dts_iter(L, st, mode, k == 1 ? x0 : G.segbuf[k - 1], G.segbuf[k],
                                target, conf, bounds, lambda, step, -1.f, halo, halo, s);
      if (st_) return st_;
    }
    for (int k = len - 1; k >= 0; --k) {
      const int flags = (j == nseg - 1 && k == len - 1 ? kAdjFirst : 0) |
                        (j == 0 && k == 0 ? kAdjLast : 0);
      int st_ = launch_adjoint(L, st, mode, g, gn, k == 0 ? x0 : G.segbuf[k], target, conf,
                               bounds, grad_t, grad_c, lambda, step, halo, halo, flags, s);
      if (st_) return st_;
      std::swap(g, gn);
    }
  }
  return DTSGB_OK;
}

}  // namespace dtsgb
