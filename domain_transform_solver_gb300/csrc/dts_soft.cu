// Soft-window DTS: the fixed-iteration DTS solve with windows whose ends are
// fractional, so that the result is a differentiable function of the edge
// weights dH, dV (no reference counterpart: the reference's windows are
// integer, src/domain_transform_filter.cuh:7-28, so its result is piecewise
// constant in the edge weights and their gradient is zero almost
// everywhere).
//
// Along a line (a row for the X half-step with e = dH, a column for Y with
// e = dV), the transformed distance between pixels p and q is
// D_pq = sum of e(j) over min(p,q) < j <= max(p,q) (a difference of the
// reference's integrated ct), and the integer window {q : D_pq <= sigma}
// becomes the weights
//   w_pq = ramp((sigma - D_pq) / tau),  ramp(x) = clamp(x + 1/2, 0, 1),
// a linear ramp of width tau (transformed-domain units) centred on the
// reference's threshold; tau -> 0 gives back the integer windows clipped at
// the line ends.  The box mean is B(p) = sum_q w_pq v(q) / n(p), n(p) =
// sum_q w_pq, and the half-steps keep the reference's form
// (src/domain_transform_solver.cuh:12-116) with this B and n:
//   X: v' = v - s * (lambda * (v - Bx) + h),  h = (c/n)(v - t)            L2
//                                              h = 0.5 (c/n)(v-t)/sqrt((v-t)^2+1e-6)
//   Y: v'' = v' - s * lambda * (v' - By)
// The mode differs from the reference's windows in two documented ways:
// windows are clipped at the line ends (the reference's one-sided collapse
// there is a jump in the edge weights), and the Y window runs to the image
// height (no width limit).
//
// Adjoint, for a = dL/d(half-step output), with coef(p) = a(p) * s / n(p):
//   dL/dv(q) = a(q) * (1 - s*lambda - s*h'(q)) + lambda * sum_p coef(p) w_pq
//   dL/dw_pq = coef(p) * (lambda * (v(q) - B(p)) + h(p))        =: G_pq
//   dL/de(j) = -(1/tau) * sum over pairs a < j <= b on the ramp
//              (|D_ab - sigma| < tau/2) of (G_ab + G_ba)
//   dL/dt, dL/dc from h as in the integer-window adjoint.
// Weights are symmetric (w_pq = w_qp), so every kernel walks outwards from
// its own pixel, summing e as it goes (D grows since e > 0; a walk stops
// where D reaches sigma + tau/2 or at the line end).  Distances are summed
// in 32-bit fixed point (Ramp), exactly, so that a pair has one distance
// whichever end it is summed from.
//
// Layout of the work: the forward keeps every iterate, the X half-step's
// result and each half-step's n and B, so the adjoint of a half-step is a
// pointwise pass (coef, alpha, beta, a * diag) and one window walk per pixel
// (k_soft_adjoint*), which also collects the ramp-band pair terms of its
// own pixel (diff, summed over the iterations); dL/de is then one prefix of
// diff along each line (k_soft_edge_scan, compensated).  The edge weights
// are fixed through a solve, so each pixel's window is planned once
// (k_soft_plan*) and the half-steps and adjoints sum planned windows over
// shared-memory tiles of the lines (rows of 256 or 1024 pixels, or 32
// columns x 64 rows, staged once with their halo).  Windows a plan cannot
// hold are walked: from tiles when the smallest edge weight bounds them
// within 40 pixels, otherwise by a thread per pixel over global memory.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/dtsgb.h"
#include "color.cuh"
#include "dtsgb_internal.cuh"

using namespace dtsgb;

namespace {

constexpr int kST = 256;

// Every launch of this file's kernels is timed by the library's profiler
// when it is on: the planned half-steps (DTSGB_K_SOFT_HALF_X, _Y) and
// adjoints (DTSGB_K_SOFT_ADJ_X, _Y) by kind, everything else as DTSGB_K_SOFT.
#define SOFT_LAUNCH(kernel, grid, stream, ...)            \
  do {                                                    \
    ProfScope ps_((stream), DTSGB_K_SOFT);                \
    kernel<<<(grid), kST, 0, (stream)>>>(__VA_ARGS__);    \
  } while (0)

struct SInst {
  int w, h;
  long long off;  // element offset of pixel (0,0); rows dense (pitch = w)
};

// planes of the arena (total floats each), then the iterates v_0 .. v_N
// and, per iteration k, the X half-step's result u_k and the window
// weights n and means B of both half-steps (kept for the adjoint)
enum {
  P_EH = 0, P_EV, P_FH, P_FV, P_T, P_C, P_U, P_COEF, P_ALPHA, P_BETA, P_ADIAG, P_DIFF,
  P_DIFFY,
  P_G0, P_G1, P_GT, P_GC, P_GEH, P_GEV,
  // window plans (k_soft_plan): n, counts, and two planes of float2 weights per axis
  P_PNX, P_PCX, P_PWX, P_PNY = P_PWX + 2, P_PCY, P_PWY, P_ITER = P_PWY + 2
};

__device__ __forceinline__ float ramp(float x) { return fminf(fmaxf(x + 0.5f, 0.f), 1.f); }

// A pixel's line: index i along it, length L, element stride st, pointer to
// element 0 of the line (plane base + instance offset).
struct Line {
  int i, L;
  long long st, base;
};

__device__ __forceinline__ bool pixel_line(const SInst& I, long long k, int axis, Line& ln) {
  int y, x;
  if (k < 0x7fffffffLL) {  // 32-bit division for every realistic image
    y = (int)((unsigned)k / (unsigned)I.w);
    x = (int)k - y * I.w;
  } else {
    y = (int)(k / I.w);
    x = (int)(k - (long long)y * I.w);
  }
  if (axis == 0) {
    ln = Line{x, I.w, 1, I.off + (long long)y * I.w};
  } else {
    ln = Line{y, I.h, I.w, I.off + x};
  }
  return true;
}

// Values along one line at line index q, from global memory (through L1) or
// from a shared-memory tile of the line (rows of `stride` entries, `off` the
// column of this line, `base` the line index of tile row 0).  E: edge
// weight in fixed point (the 32-bit words of a plane of ints), V: the value
// the window averages; A, Bt, X: the adjoint's pair coefficients alpha,
// beta and the half-step input.
struct GlobalLine {
  const float *e, *v, *al, *be, *x;
  long long st;
  int L;
  __device__ __forceinline__ int E(int q) const { return __float_as_int(e[q * st]); }
  __device__ __forceinline__ float V(int q) const { return v[q * st]; }
  __device__ __forceinline__ float A(int q) const { return al[q * st]; }
  __device__ __forceinline__ float Bt(int q) const { return be[q * st]; }
  __device__ __forceinline__ float X(int q) const { return x[q * st]; }
};
struct TileLine {
  const float *e, *v, *al, *be, *x;
  int base, stride, off, L;
  __device__ __forceinline__ int at(int q) const { return (q - base) * stride + off; }
  __device__ __forceinline__ int E(int q) const { return __float_as_int(e[at(q)]); }
  __device__ __forceinline__ float V(int q) const { return v[at(q)]; }
  __device__ __forceinline__ float A(int q) const { return al[at(q)]; }
  __device__ __forceinline__ float Bt(int q) const { return be[at(q)]; }
  __device__ __forceinline__ float X(int q) const { return x[at(q)]; }
};

// Distances in fixed point: an edge weight e becomes round(min(e, cap) 2^F),
// cap = sigma + tau/2 + 1 (a window holding a larger weight ends before it
// either way) and F the largest with 2 cap 2^F < 2^31, so every distance sum
// is exact: the same pair gets the same distance whichever end it is
// summed from, which the edge-weight gradient's prefix relies on.  A walk
// stops at D >= hiF (sigma + tau/2), a pixel is on the ramp band when
// D > loF (sigma - tau/2), and its weight is ramp((sigma - D 2^-F) / tau)
// there and 1 before it.
struct Ramp {
  int hiF, loF;
  float sig, scl, itau, wc;  // sigma, 2^-F, 1/tau, ramp(sigma/tau)
  __device__ __forceinline__ float w(int D) const {
    return D <= loF ? 1.f : ramp(__fmaf_rn(-(float)D, scl, sig) * itau);
  }
};

// n(p) and sum_q w_pq V(q) over the soft window of line index i (the ramp's
// argument (sigma - D) / tau as a product with 1/tau: within an ulp of the
// quotient).  Each side is walked four pixels at a time, the next four's
// loads issued together; the sums accumulate in the serial order and stop
// at the same pixel as a one-by-one walk.
template <class LN>
__device__ __forceinline__ void soft_window(const LN& ln, int i, const Ramp& R, float* n_out,
                                            float* s_out) {
  constexpr int U = 4;
  float n = R.wc, S = R.wc * ln.V(i);
  int D = 0;
  for (int q = i + 1; q < ln.L; q += U) {  // right side: e(q), V(q)
    int ev[U];
    float vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool in = q + u < ln.L;
      ev[u] = in ? ln.E(q + u) : R.hiF;
      vv[u] = in ? ln.V(q + u) : 0.f;
    }
    bool done = false;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (done) break;
      D += ev[u];
      if (D >= R.hiF) {
        done = true;
        break;
      }
      const float w = R.w(D);
      n += w;
      S = __fmaf_rn(w, vv[u], S);
    }
    if (done) break;
  }
  D = 0;
  for (int q = i - 1; q >= 0; q -= U) {  // left side: e(q + 1), V(q)
    int ev[U];
    float vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool in = q - u >= 0;
      ev[u] = in ? ln.E(q - u + 1) : R.hiF;
      vv[u] = in ? ln.V(q - u) : 0.f;
    }
    bool done = false;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (done) break;
      D += ev[u];
      if (D >= R.hiF) {
        done = true;
        break;
      }
      const float w = R.w(D);
      n += w;
      S = __fmaf_rn(w, vv[u], S);
    }
    if (done) break;
  }
  *n_out = n;
  *s_out = S;
}

// Data term h and its derivatives with respect to the residual d = v - t
// (dh/dd), and to c (dh/dc), for confidence c and rn = 1/n (the window
// weight's reciprocal, one division per pixel).
__device__ __forceinline__ void data_term(int mode, float v, float t, float c, float rn,
                                          float* h, float* hd, float* hc) {
  const float d = v - t, cn = c * rn;
  if (mode == 0) {  // L2: (c/n) d
    *h = cn * d;
    *hd = cn;
    *hc = d * rn;
  } else {  // Charbonnier: 0.5 (c/n) d / sqrt(d^2 + 1e-6)
    const float q = d * d + 1e-6f, r = rsqrtf(q);
    *h = 0.5f * cn * d * r;
    *hd = 0.5f * cn * 1e-6f * r / q;
    *hc = 0.5f * d * r * rn;
  }
}

// The adjoint's walk of pixel i's soft window over V = coef (n and S as in
// soft_window) that also collects the pair terms of dL/de:
//   dL/de(j) = -(1/tau) * sum over pairs a < j <= b with lo < D_ab < hi of
//              T_ab,  T_ab = G_ab + G_ba = alpha(a) x(b) + beta(a)
//                                        + alpha(b) x(a) + beta(b)
// (G_ab = coef(a) (lambda (x(b) - B(a)) + h(a)), alpha = lambda coef, beta =
// coef (h - lambda B)).  A pair's far end is among the pixels the window
// walk of its near end visits last (lo < D < hi), so the walk returns
// diff(i) = sum of T over i's right-side band minus the sum over its
// left-side band, and dL/de(j) = -(1/tau) * sum_{i<j} diff(i) (pairs that
// start before j count in the first sum, those that end before j cancel in
// the second): a prefix along the line (k_soft_edge_scan).
template <class LN>
__device__ __forceinline__ void soft_window_adj(const LN& ln, int i, const Ramp& R,
                                                float* n_out, float* s_out, float* diff_out) {
  constexpr int U = 4;
  const float ai = ln.A(i), bi = ln.Bt(i), xi = ln.X(i);
  float n = R.wc, S = R.wc * ln.V(i), diff = 0.f;
  int D = 0;
  for (int q = i + 1; q < ln.L; q += U) {  // right side: e(q), V(q)
    int ev[U];
    float vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool in = q + u < ln.L;
      ev[u] = in ? ln.E(q + u) : R.hiF;
      vv[u] = in ? ln.V(q + u) : 0.f;
    }
    bool done = false;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (done) break;
      D += ev[u];
      if (D >= R.hiF) {
        done = true;
        break;
      }
      const float w = R.w(D);
      n += w;
      S = __fmaf_rn(w, vv[u], S);
      if (D > R.loF) {
        const int b = q + u;
        diff += __fmaf_rn(ai, ln.X(b), bi) + __fmaf_rn(ln.A(b), xi, ln.Bt(b));
      }
    }
    if (done) break;
  }
  D = 0;
  for (int q = i - 1; q >= 0; q -= U) {  // left side: e(q + 1), V(q)
    int ev[U];
    float vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool in = q - u >= 0;
      ev[u] = in ? ln.E(q - u + 1) : R.hiF;
      vv[u] = in ? ln.V(q - u) : 0.f;
    }
    bool done = false;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (done) break;
      D += ev[u];
      if (D >= R.hiF) {
        done = true;
        break;
      }
      const float w = R.w(D);
      n += w;
      S = __fmaf_rn(w, vv[u], S);
      if (D > R.loF) {
        const int a = q - u;
        diff -= __fmaf_rn(ln.A(a), xi, ln.Bt(a)) + __fmaf_rn(ai, ln.X(a), bi);
      }
    }
    if (done) break;
  }
  *n_out = n;
  *s_out = S;
  *diff_out = diff;
}

// ---- the half-step ----------------------------------------------------------
// vout = half-step(vin) along `axis`; data term on X.  nout / Bout (nullable)
// keep each pixel's window weight n and mean B for the adjoint.
// tv, cv: t[p] and c[p] (read only when data)
__device__ __forceinline__ void half_update_v(long long p, float v, float n, float S, float tv,
                                              float cv, float* __restrict__ vout,
                                              float* __restrict__ nout,
                                              float* __restrict__ Bout, int data, int mode,
                                              float lambda, float step) {
  const float rn = 1.f / n;
  const float B = S * rn;
  float h = 0.f, hd, hc;
  if (data) data_term(mode, v, tv, cv, rn, &h, &hd, &hc);
  vout[p] = v - step * (lambda * (v - B) + h);
  if (nout) nout[p] = n;
  if (Bout) Bout[p] = B;
}

__device__ __forceinline__ void half_update(long long p, float v, float n, float S,
                                            const float* __restrict__ t,
                                            const float* __restrict__ c,
                                            float* __restrict__ vout, float* __restrict__ nout,
                                            float* __restrict__ Bout, int data, int mode,
                                            float lambda, float step) {
  half_update_v(p, v, n, S, data ? t[p] : 0.f, data ? c[p] : 0.f, vout, nout, Bout, data,
                mode, lambda, step);
}

// Global-memory form: any edge weights.
__global__ void k_soft_half(const SInst* __restrict__ insts, const float* __restrict__ vin,
                            float* __restrict__ vout, const float* __restrict__ e,
                            const float* __restrict__ t, const float* __restrict__ c,
                            float* __restrict__ nout, float* __restrict__ Bout,
                            int axis, int data, int mode, Ramp R, float lambda, float step) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    Line l;
    pixel_line(I, k, axis, l);
    const GlobalLine ln{e + l.base, vin + l.base, nullptr, nullptr, nullptr, l.st, l.L};
    float n, S;
    soft_window(ln, l.i, R, &n, &S);
    const long long p = I.off + k;
    half_update(p, vin[p], n, S, t, c, vout, nout, Bout, data, mode, lambda, step);
  }
}

// Shared-memory tiles of the lines, when every window ends within `halo`
// pixels (edge weights >= e_min > 0): X tiles are kTX pixels of one row,
// Y tiles kTYC columns x kTYR rows; the tile and its halo are staged once
// (coalesced rows) and every walk reads shared memory.  Same arithmetic in
// the same order as the global form, so the results are identical.
constexpr int kTX = 256, kTYC = 32, kTYR = 64, kTYT = 8;  // Y: kTYC x kTYT threads

template <int AXIS>
struct TileGeom {
  int n0, n1;  // tiles along the line and across lines of an instance
  __device__ TileGeom(const SInst& I, int len = AXIS == 0 ? kTX : kTYR) {
    if (AXIS == 0) {
      n0 = (I.w + len - 1) / len;
      n1 = I.h;
    } else {
      n0 = (I.h + kTYR - 1) / kTYR;
      n1 = (I.w + kTYC - 1) / kTYC;
    }
  }
};

// Stages NF planes of one tile (line positions [l0 - halo, l0 + len +
// halo) of the lines of the tile) into shared memory, zero outside the image.
// A thread loads U entries of every plane into registers before it stores
// any: the stores go through generic pointers that the compiler cannot tell
// apart from the planes' addresses, so a store between two loads would
// serialise them (one memory latency per entry and plane).
template <int AXIS, int NF>
__device__ __forceinline__ void stage_tile(const SInst& I, int l0, int cross,
                                           const float* const* src, float* const* dst,
                                           int halo, int len) {
  constexpr int U = 4;  // line positions per batch
  const int TL = len + 2 * halo;
  if (AXIS == 0) {  // one row `cross`
    const long long row = I.off + (long long)cross * I.w;
    for (int i0 = threadIdx.x; i0 < TL; i0 += U * kTX) {
      float v[U][NF];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int x = l0 - halo + i0 + u * kTX;
        const bool in = i0 + u * kTX < TL && x >= 0 && x < I.w;
#pragma unroll
        for (int f = 0; f < NF; ++f) v[u][f] = in ? src[f][row + x] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * kTX;
        if (i < TL) {
#pragma unroll
          for (int f = 0; f < NF; ++f) dst[f][i] = v[u][f];
        }
      }
    }
  } else {  // columns cross .. cross + kTYC - 1
    const int x = cross + threadIdx.x;
    for (int i0 = threadIdx.y; i0 < TL; i0 += U * kTYT) {
      float v[U][NF];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int y = l0 - halo + i0 + u * kTYT;
        const bool in = i0 + u * kTYT < TL && x < I.w && y >= 0 && y < I.h;
        const long long p = I.off + (long long)y * I.w + x;
#pragma unroll
        for (int f = 0; f < NF; ++f) v[u][f] = in ? src[f][p] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * kTYT;
        if (i < TL) {
#pragma unroll
          for (int f = 0; f < NF; ++f) dst[f][i * kTYC + threadIdx.x] = v[u][f];
        }
      }
    }
  }
}

template <int AXIS>
__global__ void __launch_bounds__(256)
    k_soft_half_tile(const SInst* __restrict__ insts, const float* __restrict__ vin,
                     float* __restrict__ vout, const float* __restrict__ e,
                     const float* __restrict__ t, const float* __restrict__ c,
                     float* __restrict__ nout, float* __restrict__ Bout, int data, int mode,
                     Ramp R, float lambda, float step, int halo) {
  extern __shared__ float smf[];
  const SInst I = insts[blockIdx.y];
  const TileGeom<AXIS> G(I);
  const int len = AXIS == 0 ? kTX : kTYR;
  const int TL = len + 2 * halo, TS = AXIS == 0 ? TL : TL * kTYC;
  float* se = smf;
  float* sv = smf + TS;
  const float* srcs[2] = {e, vin};
  float* dsts[2] = {se, sv};
  for (int tile = blockIdx.x; tile < G.n0 * G.n1; tile += gridDim.x) {
    const int t1 = tile / G.n0, t0 = tile - t1 * G.n0;
    const int l0 = t0 * len, cross = AXIS == 0 ? t1 : t1 * kTYC;
    __syncthreads();  // the previous tile's walks are done
    stage_tile<AXIS, 2>(I, l0, cross, srcs, dsts, halo, len);
    __syncthreads();
    if (AXIS == 0) {
      const int x = l0 + threadIdx.x;
      if (x < I.w) {
        const TileLine ln{se, sv, nullptr, nullptr, nullptr, l0 - halo, 1, 0, I.w};
        float n, S;
        soft_window(ln, x, R, &n, &S);
        const long long p = I.off + (long long)cross * I.w + x;
        half_update(p, ln.V(x), n, S, t, c, vout, nout, Bout, data, mode, lambda, step);
      }
    } else {
      const int x = cross + threadIdx.x;
      const TileLine ln{se, sv, nullptr, nullptr, nullptr, l0 - halo, kTYC, (int)threadIdx.x,
                        I.h};
      for (int y = l0 + threadIdx.y; y < min(l0 + kTYR, I.h); y += kTYT) {
        if (x >= I.w) break;
        float n, S;
        soft_window(ln, y, R, &n, &S);
        const long long p = I.off + (long long)y * I.w + x;
        half_update(p, ln.V(y), n, S, t, c, vout, nout, Bout, data, mode, lambda, step);
      }
    }
  }
}

// ---- the adjoint ----------------------------------------------------------------
// First pass of a half-step's adjoint (pointwise, from the window weight n
// and mean B the forward kept), for a = dL/d(half-step output): coef(p) =
// a(p) s / n(p), alpha = lambda coef, beta = coef (h - lambda B) and a(p)
// times the diagonal factor 1 - s*lambda - s*h'(p); on X also the local
// dL/dt, dL/dc terms.
__global__ void k_soft_pre(const SInst* __restrict__ insts, const float* __restrict__ val,
                           const float* __restrict__ a, const float* __restrict__ nk,
                           const float* __restrict__ Bk, const float* __restrict__ t,
                           const float* __restrict__ c, float* __restrict__ coef,
                           float* __restrict__ alpha, float* __restrict__ beta,
                           float* __restrict__ adiag, float* __restrict__ gt,
                           float* __restrict__ gc, int data, int mode, float lambda,
                           float step) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    const long long p = I.off + k;
    const float ap = a[p], n = nk[p];
    float h = 0.f, hd = 0.f, hc = 0.f;
    if (data) {
      data_term(mode, val[p], t[p], c[p], 1.f / n, &h, &hd, &hc);
      gt[p] += ap * step * hd;  // dh/dt = -dh/dd, and v' has -s*h
      gc[p] -= ap * step * hc;
    }
    const float cf = ap * step * (1.f / n);
    coef[p] = cf;
    alpha[p] = lambda * cf;
    beta[p] = cf * (h - lambda * Bk[p]);
    adiag[p] = ap * (1.f - step * lambda - step * hd);
  }
}

// Second pass, per pixel q of the half-step's line:
//   dL/d(input)(q) = a(q) diag(q) + lambda * sum_p coef(p) w_pq (the weights
//   are symmetric, so q walks its own window), and diff(q) of
//   soft_window_adj for the edge-weight gradient.
__global__ void k_soft_adjoint(const SInst* __restrict__ insts, const float* __restrict__ adiag,
                               const float* __restrict__ coef, const float* __restrict__ alpha,
                               const float* __restrict__ beta, const float* __restrict__ val,
                               const float* __restrict__ e, float* __restrict__ aout,
                               float* __restrict__ diff, int axis, Ramp R, float lambda) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    Line l;
    pixel_line(I, k, axis, l);
    const GlobalLine ln{e + l.base, coef + l.base, alpha + l.base, beta + l.base,
                        val + l.base, l.st, l.L};
    float n, S, d;
    soft_window_adj(ln, l.i, R, &n, &S, &d);
    const long long p = I.off + k;
    aout[p] = __fmaf_rn(lambda, S, adiag[p]);
    diff[p] += d;
  }
}

template <int AXIS>
__global__ void __launch_bounds__(256)
    k_soft_adjoint_tile(const SInst* __restrict__ insts, const float* __restrict__ adiag,
                        const float* __restrict__ coef, const float* __restrict__ alpha,
                        const float* __restrict__ beta, const float* __restrict__ val,
                        const float* __restrict__ e, float* __restrict__ aout,
                        float* __restrict__ diff, Ramp R, float lambda, int halo) {
  extern __shared__ float smf[];
  const SInst I = insts[blockIdx.y];
  const TileGeom<AXIS> G(I);
  const int len = AXIS == 0 ? kTX : kTYR;
  const int TL = len + 2 * halo, TS = AXIS == 0 ? TL : TL * kTYC;
  float* sm[5] = {smf, smf + TS, smf + 2 * TS, smf + 3 * TS, smf + 4 * TS};
  const float* srcs[5] = {e, coef, alpha, beta, val};
  for (int tile = blockIdx.x; tile < G.n0 * G.n1; tile += gridDim.x) {
    const int t1 = tile / G.n0, t0 = tile - t1 * G.n0;
    const int l0 = t0 * len, cross = AXIS == 0 ? t1 : t1 * kTYC;
    __syncthreads();
    stage_tile<AXIS, 5>(I, l0, cross, srcs, sm, halo, len);
    __syncthreads();
    const TileLine ln{sm[0], sm[1], sm[2], sm[3], sm[4], l0 - halo,
                      AXIS == 0 ? 1 : kTYC, AXIS == 0 ? 0 : (int)threadIdx.x,
                      AXIS == 0 ? I.w : I.h};
    auto one = [&](int i, long long p) {
      float n, S, d;
      soft_window_adj(ln, i, R, &n, &S, &d);
      aout[p] = __fmaf_rn(lambda, S, adiag[p]);
      diff[p] += d;
    };
    if (AXIS == 0) {
      const int x = l0 + threadIdx.x;
      if (x < I.w) one(x, I.off + (long long)cross * I.w + x);
    } else {
      const int x = cross + threadIdx.x;
      for (int y = l0 + threadIdx.y; y < min(l0 + kTYR, I.h); y += kTYT) {
        if (x >= I.w) break;
        one(y, I.off + (long long)y * I.w + x);
      }
    }
  }
}

// dL/de(j) -= (1/tau) * sum_{i<j} diff(i) along every line.  The prefix is
// the gradient itself, summed over the whole line, so only short runs are
// summed in plain FP32 and everything longer compensated.  Rows: a warp
// per row, FP32 scans of 32-pixel chunks and a Kahan carry; columns: 32
// columns x 32 row segments per block, Kahan sums along each segment, the
// segments' totals in FP64.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

constexpr int kScanChunks = 16;  // 32-pixel chunks a warp holds in registers

__global__ void k_soft_edge_scan_x(const SInst* __restrict__ insts,
                                   const float* __restrict__ diff, float* __restrict__ ge,
                                   float tau) {
  // a warp per row: 512 pixels of diff and of the gradient loaded at once
  // (coalesced, lane k of chunk j holds pixel 32 j + k), FP32 warp scans per
  // chunk, the carry across chunks a Kahan pair
  const SInst I = insts[blockIdx.y];
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int y = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; y < I.h; y += warps) {
    const float* d = diff + I.off + (long long)y * I.w;
    float* g = ge + I.off + (long long)y * I.w;
    float cs = 0.f, cc = 0.f;  // the carry is cs - cc
    for (int x0 = 0; x0 < I.w; x0 += 32 * kScanChunks) {
      float v[kScanChunks], gv[kScanChunks];
#pragma unroll
      for (int j = 0; j < kScanChunks; ++j) {
        const int x = x0 + 32 * j + lane;
        v[j] = x < I.w ? d[x] : 0.f;
        gv[j] = x < I.w ? g[x] : 0.f;
      }
#pragma unroll
      for (int j = 0; j < kScanChunks; ++j) {
        float incl = v[j];
        for (int o = 1; o < 32; o <<= 1) {
          const float t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        gv[j] -= ((cs - cc) + (incl - v[j])) / tau;
        kahan_add(cs, cc, __shfl_sync(0xffffffffu, incl, 31));
      }
#pragma unroll
      for (int j = 0; j < kScanChunks; ++j) {
        const int x = x0 + 32 * j + lane;
        if (x < I.w) g[x] = gv[j];
      }
    }
  }
}

__global__ void __launch_bounds__(1024)
    k_soft_edge_scan_y(const SInst* __restrict__ insts, const float* __restrict__ diff,
                       float* __restrict__ ge, float tau) {
  __shared__ double seg_sum[32][33];
  const SInst I = insts[blockIdx.y];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int seg = (I.h + 31) / 32;
  const int y0 = min(I.h, ty * seg), y1 = min(I.h, y0 + seg);
  for (int xb = blockIdx.x * 32; xb < I.w; xb += gridDim.x * 32) {
    const int x = xb + tx;
    float s = 0.f, c = 0.f;
    if (x < I.w)
      for (int y = y0; y < y1; ++y) kahan_add(s, c, diff[I.off + (long long)y * I.w + x]);
    __syncthreads();  // the previous column group's sums are read
    seg_sum[ty][tx] = (double)s - (double)c;
    __syncthreads();
    double excl = 0.0;
    for (int k = 0; k < ty; ++k) excl += seg_sum[k][tx];
    float cs = (float)excl, cc = (float)((double)cs - excl);
    if (x < I.w)
      for (int y = y0; y < y1; ++y) {
        const long long p = I.off + (long long)y * I.w + x;
        ge[p] -= (cs - cc) / tau;
        kahan_add(cs, cc, diff[p]);
      }
  }
}

// ---- window plans ------------------------------------------------------------
// The edge weights stay fixed through a solve and its adjoint, and so do the
// soft windows: a plan of one axis records, per pixel, the full-weight
// pixels on each side (dl, du), the ramp pixel beyond them (nrl, nru: 0 or
// 1 a side) with its weight, and n.  One ramp pixel a side is all a window
// can hold when tau does not exceed the smallest edge weight (the ramp band
// is tau wide and consecutive distances differ by an edge weight; the
// guide's are at least 1 and tau is 1 by default); other windows keep the
// walking kernels.  Sums over a planned window add the same terms in the
// same order as a walk, so a planned half-step or adjoint gives bitwise the
// walk's results while skipping its distance arithmetic.  counts = dl |
// du << 8 | nrl << 16 | nru << 24, weights = (left ramp, right ramp).
constexpr int kPlanRamp = 1;

__global__ void k_soft_plan(const SInst* __restrict__ insts, const float* __restrict__ e,
                            int axis, Ramp R, float* __restrict__ nout,
                            unsigned* __restrict__ counts, float2* __restrict__ wts,
                            int* __restrict__ stat) {
  __shared__ int bext, bovf;
  if (threadIdx.x == 0) bext = bovf = 0;
  __syncthreads();
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  int ext = 0, ovf = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    Line l;
    pixel_line(I, k, axis, l);
    const GlobalLine ln{e + l.base, nullptr, nullptr, nullptr, nullptr, l.st, l.L};
    float n = R.wc;
    int full[2] = {0, 0}, nr[2] = {0, 0};
    float wr[2] = {0.f, 0.f};
#pragma unroll
    for (int side = 0; side < 2; ++side) {  // right, then left: the walks' order
      int D = 0;
      for (int m = 1;; ++m) {
        const int q = side == 0 ? l.i + m : l.i - m;
        if (side == 0 ? q >= l.L : q < 0) break;
        D += side == 0 ? ln.E(q) : ln.E(q + 1);
        if (D >= R.hiF) break;
        const float w = R.w(D);
        n += w;
        if (D <= R.loF) {
          ++full[side];
        } else {
          if (nr[side] == 0) wr[side] = w;
          ++nr[side];
        }
      }
    }
    if (nr[0] > kPlanRamp || nr[1] > kPlanRamp || full[0] > 255 || full[1] > 255) ovf = 1;
    ext = max(ext, max(full[0] + nr[0], full[1] + nr[1]));
    const long long p = I.off + k;
    nout[p] = n;
    counts[p] = (unsigned)min(full[1], 255) | (unsigned)min(full[0], 255) << 8 |
                (unsigned)min(nr[1], 3) << 16 | (unsigned)min(nr[0], 3) << 24;
    wts[p] = make_float2(wr[1], wr[0]);
  }
  atomicMax(&bext, ext);
  if (ovf) atomicOr(&bovf, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicMax(&stat[0], bext);
    if (bovf) atomicOr(&stat[1], 1);
  }
}

// The plan from shared-memory tiles of the edge weights, converted to fixed
// point as they are staged (the conversion of k_soft_fix, so the plan is the
// global kernel's): a window side that would reach past the tile's halo
// flags the plan as overflowing (stat[1]) and the solve falls back to the
// global-memory plan.
constexpr int kPlanHalo = 24;

template <int AXIS>
__global__ void __launch_bounds__(256)
    k_soft_plan_tile(const SInst* __restrict__ insts, const float* __restrict__ e, Ramp R,
                     float cap, float scale, float* __restrict__ nout,
                     unsigned* __restrict__ counts, float2* __restrict__ wts,
                     int* __restrict__ stat) {
  extern __shared__ float smf[];
  __shared__ int bext, bovf;
  if (threadIdx.x == 0 && threadIdx.y == 0) bext = bovf = 0;
  const SInst I = insts[blockIdx.y];
  const TileGeom<AXIS> G(I);
  const int len = AXIS == 0 ? kTX : kTYR, halo = kPlanHalo;
  int ext = 0, ovf = 0;
  for (int tile = blockIdx.x; tile < G.n0 * G.n1; tile += gridDim.x) {
    const int t1 = tile / G.n0, t0 = tile - t1 * G.n0;
    const int l0 = t0 * len, cross = AXIS == 0 ? t1 : t1 * kTYC;
    __syncthreads();
    {  // stage the fixed-point weights (zero outside the image)
      const int TL = len + 2 * halo;
      if (AXIS == 0) {
        const long long row = I.off + (long long)cross * I.w;
        for (int i = threadIdx.x; i < TL; i += kTX) {
          const int x = l0 - halo + i;
          smf[i] = __int_as_float(
              x >= 0 && x < I.w
                  ? (int)rintf(fmaxf(fminf(e[row + x], cap), 0.f) * scale)
                  : 0);
        }
      } else {
        const int x = cross + threadIdx.x;
        for (int i = threadIdx.y; i < TL; i += kTYT) {
          const int y = l0 - halo + i;
          const bool in = x < I.w && y >= 0 && y < I.h;
          smf[i * kTYC + threadIdx.x] = __int_as_float(
              in ? (int)rintf(fmaxf(fminf(e[I.off + (long long)y * I.w + x], cap), 0.f) *
                              scale)
                 : 0);
        }
      }
    }
    __syncthreads();
    const TileLine ln{smf, nullptr, nullptr, nullptr, nullptr, l0 - halo,
                      AXIS == 0 ? 1 : kTYC, AXIS == 0 ? 0 : (int)threadIdx.x,
                      AXIS == 0 ? I.w : I.h};
    auto one = [&](int i, long long p) {
      float n = R.wc;
      int full[2] = {0, 0}, nr[2] = {0, 0};
      float wr[2] = {0.f, 0.f};
#pragma unroll
      for (int side = 0; side < 2; ++side) {  // right, then left: the walks' order
        int D = 0;
        for (int m = 1;; ++m) {
          const int q = side == 0 ? i + m : i - m;
          if (side == 0 ? q >= ln.L : q < 0) break;
          if (m > halo - 1) {  // past the staged halo
            ovf = 1;
            break;
          }
          D += side == 0 ? ln.E(q) : ln.E(q + 1);
          if (D >= R.hiF) break;
          const float w = R.w(D);
          n += w;
          if (D <= R.loF) {
            ++full[side];
          } else {
            if (nr[side] == 0) wr[side] = w;
            ++nr[side];
          }
        }
      }
      if (nr[0] > kPlanRamp || nr[1] > kPlanRamp) ovf = 1;
      ext = max(ext, max(full[0] + nr[0], full[1] + nr[1]));
      nout[p] = n;
      counts[p] = (unsigned)min(full[1], 255) | (unsigned)min(full[0], 255) << 8 |
                  (unsigned)min(nr[1], 3) << 16 | (unsigned)min(nr[0], 3) << 24;
      wts[p] = make_float2(wr[1], wr[0]);
    };
    if (AXIS == 0) {
      const int x = l0 + threadIdx.x;
      if (x < I.w) one(x, I.off + (long long)cross * I.w + x);
    } else {
      const int x = cross + threadIdx.x;
      for (int y = l0 + threadIdx.y; y < min(l0 + kTYR, I.h); y += kTYT) {
        if (x >= I.w) break;
        one(y, I.off + (long long)y * I.w + x);
      }
    }
  }
  __syncthreads();
  atomicMax(&bext, ext);
  if (ovf) atomicOr(&bovf, 1);
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    atomicMax(&stat[0], bext);
    if (bovf) atomicOr(&stat[1], 1);
  }
}

// sum_q w_pq V(q) over pixel i's planned window, and its weight n, in the
// walks' order.
template <class LN>
__device__ __forceinline__ float plan_sum(const LN& ln, int i, unsigned cnt, float2 w2,
                                          float wc, float* n_out = nullptr) {
  const int dl = cnt & 255, du = (cnt >> 8) & 255, nrl = (cnt >> 16) & 255, nru = cnt >> 24;
  float S = wc * ln.V(i), n = wc;
  for (int m = 1; m <= du; ++m) {
    S += ln.V(i + m);
    n += 1.f;
  }
  if (nru) {
    S = __fmaf_rn(w2.y, ln.V(i + du + 1), S);
    n += w2.y;
  }
  for (int m = 1; m <= dl; ++m) {
    S += ln.V(i - m);
    n += 1.f;
  }
  if (nrl) {
    S = __fmaf_rn(w2.x, ln.V(i - dl - 1), S);
    n += w2.x;
  }
  if (n_out) *n_out = n;
  return S;
}

// X tiles of PX x 256 pixels (a thread takes pixels t, t + 256, ...): more
// loads in flight per thread on wide images.
template <int AXIS, int PX = 1>
__global__ void __launch_bounds__(256)
    k_soft_half_plan(const SInst* __restrict__ insts, const float* __restrict__ vin,
                     float* __restrict__ vout, const unsigned* __restrict__ counts,
                     const float2* __restrict__ wts,
                     const float* __restrict__ t, const float* __restrict__ c,
                     float* __restrict__ Bout, int data, int mode, float wc, float lambda,
                     float step, int halo) {
  extern __shared__ float smf[];
  const SInst I = insts[blockIdx.y];
  const int len = AXIS == 0 ? kTX * PX : kTYR;
  const TileGeom<AXIS> G(I, len);
  const float* srcs[1] = {vin};
  float* dsts[1] = {smf};
  constexpr int OWN = AXIS == 0 ? PX : kTYR / kTYT;  // pixels per thread
  for (int tile = blockIdx.x; tile < G.n0 * G.n1; tile += gridDim.x) {
    const int t1 = tile / G.n0, t0 = tile - t1 * G.n0;
    const int l0 = t0 * len, cross = AXIS == 0 ? t1 : t1 * kTYC;
    // own pixel k: line index and global index (< 0: outside the image)
    auto own_i = [&](int k) -> int {
      return AXIS == 0 ? l0 + (int)threadIdx.x + kTX * k : l0 + (int)threadIdx.y + kTYT * k;
    };
    auto own_p = [&](int k) -> long long {
      if (AXIS == 0) {
        const int x = l0 + threadIdx.x + kTX * k;
        return x < I.w ? I.off + (long long)cross * I.w + x : -1;
      }
      const int x = cross + threadIdx.x, y = l0 + threadIdx.y + kTYT * k;
      return (x < I.w && y < I.h) ? I.off + (long long)y * I.w + x : -1;
    };
    // X: the own pixels' plan, t and c, loaded before the tile is staged, so
    // that these loads are in flight with the staging's (Y's eight pixels a
    // thread load after the staging)
    constexpr int OP = AXIS == 0 ? OWN : 1;
    unsigned cn[OP];
    float2 w2[OP];
    float tv[OP], cv[OP];
    if (AXIS == 0) {
#pragma unroll
      for (int k = 0; k < OP; ++k) {
        const long long p = own_p(k);
        cn[k] = p >= 0 ? counts[p] : 0u;
        w2[k] = p >= 0 ? wts[p] : make_float2(0.f, 0.f);
        tv[k] = p >= 0 && data ? t[p] : 0.f;
        cv[k] = p >= 0 && data ? c[p] : 0.f;
      }
    }
    __syncthreads();
    stage_tile<AXIS, 1>(I, l0, cross, srcs, dsts, halo, len);
    __syncthreads();
    const TileLine ln{nullptr, smf, nullptr, nullptr, nullptr, l0 - halo,
                      AXIS == 0 ? 1 : kTYC, AXIS == 0 ? 0 : (int)threadIdx.x,
                      AXIS == 0 ? I.w : I.h};
    if (AXIS == 0) {
#pragma unroll
      for (int k = 0; k < OP; ++k) {
        const long long p = own_p(k);
        if (p < 0) continue;
        const int i = own_i(k);
        float n;
        const float S = plan_sum(ln, i, cn[k], w2[k], wc, &n);
        half_update_v(p, ln.V(i), n, S, tv[k], cv[k], vout, nullptr, Bout, data, mode, lambda,
                      step);
      }
    } else {
      const int x = cross + threadIdx.x;
      for (int y = l0 + threadIdx.y; y < min(l0 + kTYR, I.h); y += kTYT) {
        if (x >= I.w) break;
        const long long p = I.off + (long long)y * I.w + x;
        float n;
        const float S = plan_sum(ln, y, counts[p], wts[p], wc, &n);
        half_update(p, ln.V(y), n, S, t, c, vout, nullptr, Bout, data, mode, lambda, step);
      }
    }
  }
}

// The planned adjoint with its pointwise first pass fused in: the tile
// stages a = dL/d(output), n, B, the input x (and t, c on X), every staged
// entry becomes (coef, alpha, beta) in place (its owner taking a * diag and
// dL/dt, dL/dc on the way), and the window sums (over
// coef, plan_sum) and the ramp band's pair terms (diff) follow, in
// soft_window_adj's order.  The same expressions as k_soft_pre +
// k_soft_adjoint_tile, without their four intermediate planes.
template <int AXIS, int PX = 1>
__global__ void __launch_bounds__(256)
    k_soft_adjoint_fused(const SInst* __restrict__ insts, const float* __restrict__ a,
                         const float* __restrict__ nplan, const float* __restrict__ Bk,
                         const float* __restrict__ val, const float* __restrict__ t,
                         const float* __restrict__ c, const unsigned* __restrict__ counts,
                         const float2* __restrict__ wts, float* __restrict__ aout,
                         float* __restrict__ diff, float* __restrict__ gt,
                         float* __restrict__ gc, int data, int mode, float lambda, float step,
                         float wc, int halo) {
  extern __shared__ float smf[];
  constexpr int OWN = AXIS == 0 ? PX : kTYR / kTYT;  // pixels per thread
  const SInst I = insts[blockIdx.y];
  const int len = AXIS == 0 ? kTX * PX : kTYR;
  const TileGeom<AXIS> G(I, len);
  const int TL = len + 2 * halo, TS = AXIS == 0 ? TL : TL * kTYC;
  const int nf = data ? 6 : 4;
  float* F[6] = {smf, smf + TS, smf + 2 * TS, smf + 3 * TS, smf + 4 * TS, smf + 5 * TS};
  const float* srcs[6] = {a, nplan, Bk, val, t, c};
  for (int tile = blockIdx.x; tile < G.n0 * G.n1; tile += gridDim.x) {
    const int t1 = tile / G.n0, t0 = tile - t1 * G.n0;
    const int l0 = t0 * len, cross = AXIS == 0 ? t1 : t1 * kTYC;
    // own pixel k: line index and global index (< 0: outside the image)
    auto own_i = [&](int k) -> int {
      return AXIS == 0 ? l0 + (int)threadIdx.x + kTX * k : l0 + (int)threadIdx.y + kTYT * k;
    };
    auto own_p = [&](int k) -> long long {
      if (AXIS == 0) {
        const int x = l0 + threadIdx.x + kTX * k;
        return x < I.w ? I.off + (long long)cross * I.w + x : -1;
      }
      const int x = cross + threadIdx.x, y = l0 + threadIdx.y + kTYT * k;
      return (x < I.w && y < I.h) ? I.off + (long long)y * I.w + x : -1;
    };
    // The own pixels' plan and pair sums (and on X their dL/dt, dL/dc) are
    // loaded ahead of their use: on X all four before the tile is staged,
    // so that these loads are in flight with the staging's; on Y (eight
    // pixels a thread: registers) a ring of RING pixels, the first ones
    // before the staging and each later one when its slot frees up.
    constexpr int RING = AXIS == 0 ? OWN : 2, OG = AXIS == 0 ? OWN : 1;
    unsigned cn[RING];
    float2 w2[RING];
    float dv[RING], gtv[OG], gcv[OG];
    auto load_own = [&](int k, int slot) {
      const long long p = own_p(k);
      cn[slot] = p >= 0 ? counts[p] : 0u;
      w2[slot] = p >= 0 ? wts[p] : make_float2(0.f, 0.f);
      dv[slot] = p >= 0 ? diff[p] : 0.f;
      if (AXIS == 0) {
        gtv[slot % OG] = p >= 0 && data ? gt[p] : 0.f;
        gcv[slot % OG] = p >= 0 && data ? gc[p] : 0.f;
      }
    };
#pragma unroll
    for (int k = 0; k < RING; ++k) load_own(k, k);
    __syncthreads();
    if (data)
      stage_tile<AXIS, 6>(I, l0, cross, srcs, F, halo, len);
    else
      stage_tile<AXIS, 4>(I, l0, cross, srcs, F, halo, len);
    __syncthreads();
    const TileLine ln{nullptr, F[0], F[1], F[2], F[3], l0 - halo,
                      AXIS == 0 ? 1 : kTYC, AXIS == 0 ? 0 : (int)threadIdx.x,
                      AXIS == 0 ? I.w : I.h};
    // Every staged entry becomes (coef, alpha, beta) in place; a thread
    // transforms its own pixels' entries (taking their a * diag and dL/dt,
    // dL/dc on the way, X only) and a share of the halo's.
    // returns a * diag of own pixel k (p >= 0)
    auto transform = [&](int e, long long p, int k) -> float {
      const float ap = F[0][e], n = F[1][e];
      float h = 0.f, hd = 0.f, hc = 0.f;
      const float rn = 1.f / n;
      if (data) data_term(mode, F[3][e], F[4][e], F[5][e], rn, &h, &hd, &hc);
      float adg = 0.f;
      if (AXIS == 0 && p >= 0) {
        if (data) {
          gt[p] = gtv[k % OG] + ap * step * hd;  // dh/dt = -dh/dd, and v' has -s*h
          gc[p] = gcv[k % OG] - ap * step * hc;
        }
        adg = ap * (1.f - step * lambda - step * hd);
      }
      const float cf = ap * step * rn;
      F[0][e] = cf;
      F[1][e] = lambda * cf;
      F[2][e] = cf * (h - lambda * F[2][e]);
      return adg;
    };
    float adg[OWN];
    if (AXIS == 0) {
      // own pixels transformed with their a * diag, the halo shared out
      // over the first 2 halo threads
#pragma unroll
      for (int k = 0; k < OWN; ++k) adg[k] = transform(ln.at(own_i(k)), own_p(k), k);
      const int t = threadIdx.x;
      if (t < 2 * halo) (void)transform(t < halo ? t : len + t, -1, 0);
    } else {
      // eight own pixels a thread: their a * diag (and dL/dt, dL/dc) first,
      // then the whole tile transformed, entries spread over the threads
#pragma unroll
      for (int k = 0; k < OWN; ++k) {
        const long long p = own_p(k);
        adg[k] = 0.f;
        if (p < 0) continue;
        const int e = ln.at(own_i(k));
        const float ap = F[0][e];
        float hd = 0.f;
        if (data) {
          float h, hc;
          data_term(mode, F[3][e], F[4][e], F[5][e], 1.f / F[1][e], &h, &hd, &hc);
          gt[p] += ap * step * hd;
          gc[p] -= ap * step * hc;
        }
        adg[k] = ap * (1.f - step * lambda - step * hd);
      }
      __syncthreads();
      const int tid = threadIdx.x + kTYC * threadIdx.y;
      for (int e = tid; e < TS; e += kTYC * kTYT) (void)transform(e, -1, 0);
    }
    __syncthreads();
    // window sum and band pair terms of own pixel k (p >= 0) from its ring slot
    auto finish = [&](int k, long long p, int slot) {
      const int i = own_i(k);
      const unsigned cnt = cn[slot];
      const float S = plan_sum(ln, i, cnt, w2[slot], wc);
      aout[p] = __fmaf_rn(lambda, S, adg[k]);
      const int dl = cnt & 255, du = (cnt >> 8) & 255, nrl = (cnt >> 16) & 255,
                nru = cnt >> 24;
      const float ai = ln.A(i), bi = ln.Bt(i), xi = ln.X(i);
      float d = 0.f;
      if (nru) {
        const int b = i + du + 1;
        d += __fmaf_rn(ai, ln.X(b), bi) + __fmaf_rn(ln.A(b), xi, ln.Bt(b));
      }
      if (nrl) {
        const int aa = i - dl - 1;
        d -= __fmaf_rn(ln.A(aa), xi, ln.Bt(aa)) + __fmaf_rn(ai, ln.X(aa), bi);
      }
      diff[p] = dv[slot] + d;
    };
    if (AXIS == 0) {
#pragma unroll
      for (int k = 0; k < OWN; ++k) {
        const long long p = own_p(k);
        if (p >= 0) finish(k, p, k);
      }
    } else {
#pragma unroll
      for (int k = 0; k < OWN; ++k) {
        const long long p = own_p(k);
        if (p >= 0) finish(k, p, k % RING);
        if (k + RING < OWN) load_own(k + RING, k % RING);
      }
    }
  }
}

// The smallest edge weight of the instances' pixels in a plane pair (the
// tiles' halo bound); a weight that is not finite and positive counts as 0,
// which keeps the global-memory kernels.  One atomic per block.
__global__ void k_soft_emin(const SInst* __restrict__ insts, const float* __restrict__ a,
                            const float* __restrict__ b, unsigned* __restrict__ out) {
  __shared__ float wmin[kST / 32];
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  float m = INFINITY;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    const float x = a[I.off + k], y = b[I.off + k];
    m = fminf(m, (x > 0.f && x < INFINITY) ? x : 0.f);
    m = fminf(m, (y > 0.f && y < INFINITY) ? y : 0.f);
  }
  for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kST / 32; ++w) m = fminf(m, wmin[w]);
    atomicMin(out, __float_as_uint(m));  // m >= 0: its bits order like the values
  }
}

// Edge weights to the walks' fixed point (Ramp): round(min(e, cap) 2^F);
// a weight that is not positive counts as 0, a NaN as the cap.
__global__ void k_soft_fix(const SInst* __restrict__ insts, const float* __restrict__ e,
                           int* __restrict__ out, float cap, float scale) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x)
    out[I.off + k] = (int)rintf(fmaxf(fminf(e[I.off + k], cap), 0.f) * scale);
}

__global__ void k_soft_axpy(const SInst* __restrict__ insts, const float* __restrict__ x,
                            float* __restrict__ y) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x)
    y[I.off + k] += x[I.off + k];
}

__global__ void k_soft_edges(const SInst* __restrict__ insts, const uchar4* __restrict__ g,
                             float rx, float ry, float* __restrict__ eh,
                             float* __restrict__ ev) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  const uchar4 zero = make_uchar4(0, 0, 0, 0);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(k / I.w), x = (int)(k - (long long)y * I.w);
    const long long p = I.off + k;
    const uchar4 cur = g[p];
    eh[p] = edge_weight(cur, x > 0 ? g[p - 1] : zero, rx);
    ev[p] = edge_weight(cur, y > 0 ? g[p - I.w] : zero, ry);
  }
}

__global__ void k_soft_fill(float* __restrict__ p, long long n, float v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

}  // namespace

struct dtsgb_soft_s {
  int n = 0;
  std::vector<SInst> inst;
  long long total = 0, max_px = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  SInst* d_inst = nullptr;
  float* arena = nullptr;
  int planes = 0;
  int n_iter = -1;  // iterations of the last solve (-1: none to differentiate)
  dtsgb_optimize_params opt{};
  float tau = 1.f;
  float* plane(int k) const { return arena + (size_t)k * total; }
  unsigned* d_emin = nullptr;  // smallest edge weight (float bits)
  int* d_stat = nullptr;       // window plans: [0] widest window side, [1] overflow
  bool use_plan = false;       // the last solve's windows are planned
  int plan_halo = 0;
  Ramp ramp{};                 // fixed-point distances of the last solve
  int halo = 1 << 30;          // tile halo of the last solve; above kMaxHalo: global kernels
  // per-iteration planes after v_0 .. v_N: u_k, nX_k, BX_k, nY_k, BY_k
  float* kept(int which, int k) const { return plane(P_ITER + n_kept + 1 + which * n_kept + k); }
  int n_kept = 0;  // iterations the kept planes are laid out for
};

namespace {

dim3 soft_grid(const dtsgb_soft_s* s) {
  long long b = (s->max_px + kST - 1) / kST;
  return dim3((unsigned)std::max<long long>(1, std::min<long long>(b, 152 * 8)), s->n);
}

int ensure_planes(dtsgb_soft_t s, int planes) {
  if (planes <= s->planes) return DTSGB_OK;
  DTSGB_CUDA(cudaStreamSynchronize(s->stream));
  dfree(s->arena);
  s->planes = 0;
  if (int st = dalloc(&s->arena, (size_t)planes * s->total)) return st;
  s->planes = planes;
  return DTSGB_OK;
}

// Largest tile halo of the shared-memory kernels (the Y adjoint tile then
// holds 5 x 32 x (64 + 80) floats, 92 KB).
constexpr int kMaxHalo = 40;

long long max_tiles(const dtsgb_soft_s* s, int axis, int px = 1) {
  long long m = 1;
  const int lx = kTX * px;
  for (const SInst& I : s->inst)
    m = std::max(m, axis == 0 ? (long long)((I.w + lx - 1) / lx) * I.h
                              : (long long)((I.h + kTYR - 1) / kTYR) * ((I.w + kTYC - 1) / kTYC));
  return m;
}

// Pixels per thread of the planned X kernels: 4 when the widest image spans
// 1024 pixels.
int plan_px(const dtsgb_soft_s* s) {
  int w = 0;
  for (const SInst& I : s->inst) w = std::max(w, I.w);
  return w >= 4 * kTX ? 4 : 1;
}

// The tiles' halo for this solve's edge weights and sigma, tau: every walk
// (window, pair band) stops once its distance reaches sigma + tau/2, after
// at most ceil((sigma + tau/2) / e_min) pixels; the chunked walks load up to
// three more, and one more covers the rounding of the distance sums.
int soft_halo(dtsgb_soft_t s, float sigma, float tau, int* halo) {
  const unsigned inf_bits = 0x7f800000u;
  DTSGB_CUDA(cudaMemcpyAsync(s->d_emin, &inf_bits, 4, cudaMemcpyHostToDevice, s->stream));
  {
    ProfScope ps(s->stream, DTSGB_K_SOFT);
    k_soft_emin<<<soft_grid(s), kST, 0, s->stream>>>(s->d_inst, s->plane(P_EH), s->plane(P_EV),
                                                     s->d_emin);
  }
  DTSGB_CUDA(cudaGetLastError());
  unsigned bits = 0;
  DTSGB_CUDA(cudaMemcpyAsync(&bits, s->d_emin, 4, cudaMemcpyDeviceToHost, s->stream));
  DTSGB_CUDA(cudaStreamSynchronize(s->stream));
  float emin;
  std::memcpy(&emin, &bits, 4);
  const double reach = (double)sigma + 0.5 * (double)tau;
  *halo = emin > 0.f ? (int)std::min(1e9, std::ceil(reach / emin)) + 5 : (1 << 30);
  return DTSGB_OK;
}

// The fixed-point distances for sigma, tau (Ramp).
Ramp make_ramp(float sigma, float tau) {
  const double hi = (double)sigma + 0.5 * (double)tau, lo = (double)sigma - 0.5 * (double)tau;
  const double cap = hi + 1.0;
  const int F = (int)std::floor(30.0 - std::log2(cap));
  const double sc = std::ldexp(1.0, F);
  Ramp R;
  R.hiF = (int)std::ceil(hi * sc);
  R.loF = (int)std::floor(std::max(lo, 0.0) * sc);
  R.sig = sigma;
  R.scl = (float)std::ldexp(1.0, -F);
  R.itau = 1.f / tau;
  R.wc = std::min(std::max(sigma * R.itau + 0.5f, 0.f), 1.f);
  return R;
}

int fix_edges(dtsgb_soft_t s, float sigma, float tau) {
  s->ramp = make_ramp(sigma, tau);
  const float cap = (float)((double)sigma + 0.5 * (double)tau + 1.0);
  const float scale = 1.f / s->ramp.scl;
  for (int axis = 0; axis < 2; ++axis) {
    ProfScope ps(s->stream, DTSGB_K_SOFT);
    k_soft_fix<<<soft_grid(s), kST, 0, s->stream>>>(
        s->d_inst, s->plane(axis == 0 ? P_EH : P_EV),
        reinterpret_cast<int*>(s->plane(axis == 0 ? P_FH : P_FV)), cap, scale);
  }
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

// Plans both axes' windows from shared-memory tiles of the float edge
// weights (no fixed-point planes, no e_min); true when no window overflows.
int plan_windows_tiled(dtsgb_soft_t s, float sigma, float tau, bool* ok) {
  s->ramp = make_ramp(sigma, tau);
  const float cap = (float)((double)sigma + 0.5 * (double)tau + 1.0);
  const float scale = 1.f / s->ramp.scl;
  DTSGB_CUDA(cudaMemsetAsync(s->d_stat, 0, 2 * sizeof(int), s->stream));
  for (int axis = 0; axis < 2; ++axis) {
    const int base = axis == 0 ? P_PNX : P_PNY;
    const dim3 g((unsigned)std::min<long long>(max_tiles(s, axis), 152 * 16), s->n);
    float* e = s->plane(axis == 0 ? P_EH : P_EV);
    unsigned* cnt = reinterpret_cast<unsigned*>(s->plane(base + 1));
    float2* wts = reinterpret_cast<float2*>(s->plane(base + 2));
    ProfScope ps(s->stream, DTSGB_K_SOFT);
    if (axis == 0)
      k_soft_plan_tile<0><<<g, kTX, sizeof(float) * (kTX + 2 * kPlanHalo), s->stream>>>(
          s->d_inst, e, s->ramp, cap, scale, s->plane(base), cnt, wts, s->d_stat);
    else
      k_soft_plan_tile<1><<<g, dim3(kTYC, kTYT),
                            sizeof(float) * (kTYR + 2 * kPlanHalo) * kTYC, s->stream>>>(
          s->d_inst, e, s->ramp, cap, scale, s->plane(base), cnt, wts, s->d_stat);
  }
  DTSGB_CUDA(cudaGetLastError());
  int st[2] = {0, 0};
  DTSGB_CUDA(cudaMemcpyAsync(st, s->d_stat, sizeof st, cudaMemcpyDeviceToHost, s->stream));
  DTSGB_CUDA(cudaStreamSynchronize(s->stream));
  *ok = st[1] == 0;
  s->plan_halo = st[0];
  s->use_plan = *ok;
  return DTSGB_OK;
}

// Plans both axes' windows; they are used when no side of any window has
// more than kPlanRamp ramp pixels and every window fits the tiles' halo.
int plan_windows(dtsgb_soft_t s) {
  DTSGB_CUDA(cudaMemsetAsync(s->d_stat, 0, 2 * sizeof(int), s->stream));
  for (int axis = 0; axis < 2; ++axis) {
    const int base = axis == 0 ? P_PNX : P_PNY;
    ProfScope ps(s->stream, DTSGB_K_SOFT);
    k_soft_plan<<<soft_grid(s), kST, 0, s->stream>>>(
        s->d_inst, s->plane(axis == 0 ? P_FH : P_FV), axis, s->ramp, s->plane(base),
        reinterpret_cast<unsigned*>(s->plane(base + 1)),
        reinterpret_cast<float2*>(s->plane(base + 2)), s->d_stat);
  }
  DTSGB_CUDA(cudaGetLastError());
  int st[2] = {0, 0};
  DTSGB_CUDA(cudaMemcpyAsync(st, s->d_stat, sizeof st, cudaMemcpyDeviceToHost, s->stream));
  DTSGB_CUDA(cudaStreamSynchronize(s->stream));
  s->plan_halo = st[0];
  s->use_plan = st[1] == 0 && st[0] <= kMaxHalo;
  return DTSGB_OK;
}

int launch_half(dtsgb_soft_t s, const float* vin, float* vout, const float* e, const float* t,
                const float* c, float* nout, float* Bout, int axis, int data, int mode,
                float lambda, float step) {
  ProfScope ps(s->stream, !s->use_plan ? DTSGB_K_SOFT
                          : axis == 0 ? DTSGB_K_SOFT_HALF_X
                                      : DTSGB_K_SOFT_HALF_Y);
  const int H = s->halo;
  const Ramp R = s->ramp;
  if (s->use_plan) {
    const int PH = s->plan_halo, base = axis == 0 ? P_PNX : P_PNY;
    const unsigned* cnt = reinterpret_cast<const unsigned*>(s->plane(base + 1));
    const float2* wts = reinterpret_cast<const float2*>(s->plane(base + 2));
    const int px = axis == 0 ? plan_px(s) : 1;
    const dim3 g((unsigned)std::min<long long>(max_tiles(s, axis, px), 152 * 16), s->n);
    if (axis == 0 && px == 4)
      k_soft_half_plan<0, 4><<<g, kTX, sizeof(float) * (4 * kTX + 2 * PH), s->stream>>>(
          s->d_inst, vin, vout, cnt, wts, t, c, Bout, data, mode, R.wc, lambda, step, PH);
    else if (axis == 0)
      k_soft_half_plan<0><<<g, kTX, sizeof(float) * (kTX + 2 * PH), s->stream>>>(
          s->d_inst, vin, vout, cnt, wts, t, c, Bout, data, mode, R.wc, lambda, step, PH);
    else
      k_soft_half_plan<1><<<g, dim3(kTYC, kTYT), sizeof(float) * (kTYR + 2 * PH) * kTYC,
                            s->stream>>>(s->d_inst, vin, vout, cnt, wts, t, c, Bout, data, mode,
                                         R.wc, lambda, step, PH);
  } else if (H > kMaxHalo) {
    k_soft_half<<<soft_grid(s), kST, 0, s->stream>>>(s->d_inst, vin, vout, e, t, c, nout, Bout,
                                                     axis, data, mode, R, lambda, step);
  } else {
    const long long tiles = max_tiles(s, axis);
    const dim3 g((unsigned)std::min<long long>(tiles, 152 * 16), s->n);
    if (axis == 0) {
      const size_t sm = sizeof(float) * 2 * (kTX + 2 * H);
      k_soft_half_tile<0><<<g, kTX, sm, s->stream>>>(s->d_inst, vin, vout, e, t, c, nout, Bout,
                                                     data, mode, R, lambda, step, H);
    } else {
      const size_t sm = sizeof(float) * 2 * (kTYR + 2 * H) * kTYC;
      k_soft_half_tile<1><<<g, dim3(kTYC, kTYT), sm, s->stream>>>(
          s->d_inst, vin, vout, e, t, c, nout, Bout, data, mode, R, lambda, step, H);
    }
  }
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

int launch_adjoint(dtsgb_soft_t s, const float* adiag, const float* coef, const float* alpha,
                   const float* beta, const float* val, const float* e, float* aout, int axis,
                   float lambda) {
  ProfScope ps(s->stream, DTSGB_K_SOFT);
  float* diff = s->plane(axis == 0 ? P_DIFF : P_DIFFY);
  const int H = s->halo;
  const Ramp R = s->ramp;
  if (H > kMaxHalo) {
    k_soft_adjoint<<<soft_grid(s), kST, 0, s->stream>>>(s->d_inst, adiag, coef, alpha, beta,
                                                        val, e, aout, diff, axis, R, lambda);
  } else {
    const long long tiles = max_tiles(s, axis);
    const dim3 g((unsigned)std::min<long long>(tiles, 152 * 16), s->n);
    if (axis == 0) {
      const size_t sm = sizeof(float) * 5 * (kTX + 2 * H);
      k_soft_adjoint_tile<0><<<g, kTX, sm, s->stream>>>(s->d_inst, adiag, coef, alpha, beta,
                                                        val, e, aout, diff, R, lambda, H);
    } else {
      const size_t sm = sizeof(float) * 5 * (kTYR + 2 * H) * kTYC;
      DTSGB_CUDA(cudaFuncSetAttribute(k_soft_adjoint_tile<1>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      k_soft_adjoint_tile<1><<<g, dim3(kTYC, kTYT), sm, s->stream>>>(
          s->d_inst, adiag, coef, alpha, beta, val, e, aout, diff, R, lambda, H);
    }
  }
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

// The planned adjoint of one half-step with its pointwise pass fused in
// (k_soft_adjoint_fused); its band pair terms add into the axis's diff plane.
int launch_adjoint_fused(dtsgb_soft_t s, const float* a, const float* Bk, const float* val,
                         const float* t, const float* c, float* aout, float* gt, float* gc,
                         int axis, int data, int mode, float lambda, float step) {
  ProfScope ps(s->stream, axis == 0 ? DTSGB_K_SOFT_ADJ_X : DTSGB_K_SOFT_ADJ_Y);
  float* diff = s->plane(axis == 0 ? P_DIFF : P_DIFFY);
  const int PH = s->plan_halo, base = axis == 0 ? P_PNX : P_PNY;
  const unsigned* cnt = reinterpret_cast<const unsigned*>(s->plane(base + 1));
  const float2* wts = reinterpret_cast<const float2*>(s->plane(base + 2));
  const float* nplan = s->plane(base);
  const float wc = s->ramp.wc;
  const int nf = data ? 6 : 4;
  const int px = axis == 0 ? plan_px(s) : 1;
  const dim3 g((unsigned)std::min<long long>(max_tiles(s, axis, px), 152 * 16), s->n);
  if (axis == 0 && px == 4) {
    k_soft_adjoint_fused<0, 4><<<g, kTX, sizeof(float) * nf * (4 * kTX + 2 * PH), s->stream>>>(
        s->d_inst, a, nplan, Bk, val, t, c, cnt, wts, aout, diff, gt, gc, data, mode, lambda,
        step, wc, PH);
  } else if (axis == 0) {
    k_soft_adjoint_fused<0><<<g, kTX, sizeof(float) * nf * (kTX + 2 * PH), s->stream>>>(
        s->d_inst, a, nplan, Bk, val, t, c, cnt, wts, aout, diff, gt, gc, data, mode, lambda,
        step, wc, PH);
  } else {
    const size_t sm = sizeof(float) * nf * (kTYR + 2 * PH) * kTYC;
    DTSGB_CUDA(cudaFuncSetAttribute(k_soft_adjoint_fused<1>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_soft_adjoint_fused<1><<<g, dim3(kTYC, kTYT), sm, s->stream>>>(
        s->d_inst, a, nplan, Bk, val, t, c, cnt, wts, aout, diff, gt, gc, data, mode, lambda,
        step, wc, PH);
  }
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

// The edge-weight gradients from the band pair terms summed over all the
// iterations (the prefix is linear, so one per axis serves them all).
int launch_edge_scans(dtsgb_soft_t s, float tau) {
  int max_w = 1, max_h = 1;
  for (const SInst& I : s->inst) {
    max_w = std::max(max_w, I.w);
    max_h = std::max(max_h, I.h);
  }
  {
    ProfScope ps(s->stream, DTSGB_K_SOFT);
    k_soft_edge_scan_x<<<dim3((unsigned)std::min(1024, (max_h + 7) / 8), s->n), kST, 0,
                         s->stream>>>(s->d_inst, s->plane(P_DIFF), s->plane(P_GEH), tau);
  }
  {
    ProfScope ps(s->stream, DTSGB_K_SOFT);
    k_soft_edge_scan_y<<<dim3((unsigned)std::min(1024, (max_w + 31) / 32), s->n),
                         dim3(32, 32), 0, s->stream>>>(s->d_inst, s->plane(P_DIFFY),
                                                       s->plane(P_GEV), tau);
  }
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

// n device pointers (dense W*H floats) <-> plane k of the arena
int copy_planes(dtsgb_soft_t s, const float* const* src, int k, bool in) {
  for (int i = 0; i < s->n; ++i) {
    if (!src[i]) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null device pointer");
    const size_t bytes = (size_t)s->inst[i].w * s->inst[i].h * sizeof(float);
    float* a = s->plane(k) + s->inst[i].off;
    if (in)
      DTSGB_CUDA(cudaMemcpyAsync(a, src[i], bytes, cudaMemcpyDeviceToDevice, s->stream));
    else
      DTSGB_CUDA(cudaMemcpyAsync(const_cast<float*>(src[i]), a, bytes,
                                 cudaMemcpyDeviceToDevice, s->stream));
  }
  return DTSGB_OK;
}

}  // namespace

extern "C" {

DTSGB_API int dtsgb_soft_create(int n, const int* widths, const int* heights,
                                dtsgb_soft_t* out) {
  if (!out || !widths || !heights || n <= 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "bad arguments");
  *out = nullptr;
  auto* s = new dtsgb_soft_s();
  s->n = n;
  long long off = 0;
  for (int i = 0; i < n; ++i) {
    if (widths[i] <= 0 || heights[i] <= 0) {
      delete s;
      return fail(DTSGB_ERR_INVALID_DIMS, "image dims must be positive");
    }
    const long long px = (long long)widths[i] * heights[i];
    s->inst.push_back(SInst{widths[i], heights[i], off});
    off += round_up_ll(px, 32);
    s->max_px = std::max(s->max_px, px);
  }
  s->total = off;
  int st = dalloc(&s->d_inst, (size_t)n);
  if (!st) st = dalloc(&s->d_emin, 1);
  if (!st) st = dalloc(&s->d_stat, 2);
  if (!st && cudaMemcpy(s->d_inst, s->inst.data(), n * sizeof(SInst),
                        cudaMemcpyHostToDevice) != cudaSuccess)
    st = fail(DTSGB_ERR_CUDA, "instance table upload");
  if (!st && cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
    st = fail(DTSGB_ERR_CUDA, "stream creation");
  if (st) {
    dfree(s->d_inst);
    dfree(s->d_emin);
    dfree(s->d_stat);
    delete s;
    return st;
  }
  s->own_stream = true;
  if ((st = ensure_planes(s, P_ITER + 2))) {
    dtsgb_soft_destroy(s);
    return st;
  }
  *out = s;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_soft_destroy(dtsgb_soft_t s) {
  if (!s) return DTSGB_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  dfree(s->arena);
  dfree(s->d_inst);
  dfree(s->d_emin);
  dfree(s->d_stat);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_soft_set_stream(dtsgb_soft_t s, void* stream) {
  if (!s) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  DTSGB_CUDA(cudaStreamSynchronize(s->stream));
  if (s->own_stream) cudaStreamDestroy(s->stream);
  s->own_stream = stream == nullptr;
  if (s->own_stream) {
    DTSGB_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  } else {
    s->stream = (cudaStream_t)stream;
  }
  return DTSGB_OK;
}

DTSGB_API int dtsgb_soft_edge_weights(dtsgb_soft_t s, int color_space,
                                      const void* const* rgba,
                                      const dtsgb_filter_params* f, float* const* dH,
                                      float* const* dV) {
  if (!s || !rgba || !f || !dH || !dV) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (color_space < DTSGB_RGB || color_space > DTSGB_YYY)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid color space");
  if (!finite_pos(f->sigma_x) || !finite_pos(f->sigma_y) || !finite_pos(f->sigma_r))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "filter sigmas must be finite, positive");
  // the guide goes through plane P_U (4 bytes per pixel), converted in place
  uchar4* g = reinterpret_cast<uchar4*>(s->plane(P_U));
  for (int i = 0; i < s->n; ++i) {
    if (!rgba[i] || !dH[i] || !dV[i])
      return fail(DTSGB_ERR_INVALID_ARGUMENT, "null device pointer");
    DTSGB_CUDA(cudaMemcpyAsync(g + s->inst[i].off, rgba[i],
                               (size_t)s->inst[i].w * s->inst[i].h * 4,
                               cudaMemcpyDeviceToDevice, s->stream));
  }
  if (int st = launch_color_convert_flat(g, s->total, color_space, s->stream)) return st;
  const float rx = f->sigma_x / f->sigma_r, ry = f->sigma_y / f->sigma_r;
  {
    ProfScope ps(s->stream, DTSGB_K_SOFT);
    k_soft_edges<<<soft_grid(s), kST, 0, s->stream>>>(s->d_inst, g, rx, ry, s->plane(P_EH),
                                                      s->plane(P_EV));
  }
  DTSGB_CUDA(cudaGetLastError());
  if (int st = copy_planes(s, dH, P_EH, false)) return st;
  if (int st = copy_planes(s, dV, P_EV, false)) return st;
  DTSGB_CUDA(cudaStreamSynchronize(s->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_soft_solve(dtsgb_soft_t s, const float* const* dH, const float* const* dV,
                               const float* const* target, const float* const* confidence,
                               const dtsgb_optimize_params* p, float tau, float* const* out) {
  if (!s || !dH || !dV || !target || !p || !out)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (p->loss < DTSGB_L1 || p->loss > DTSGB_CHARBONNIER)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid loss");
  if (p->num_iterations < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "num_iterations < 0");
  if (!finite_pos(p->sigma_z) || p->sigma_z >= 254.f)
    return fail(DTSGB_ERR_UNSUPPORTED, "sigma_z must be in (0, 254)");
  if (!finite_pos(tau) || tau > 2.f * p->sigma_z)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "tau must be in (0, 2 sigma_z]");
  if (!std::isfinite(p->lambda) || !std::isfinite(p->step_size))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "lambda / step_size not finite");
  s->n_iter = -1;
  const int N = p->loss == DTSGB_L1 ? 0 : p->num_iterations;
  if (int st = ensure_planes(s, P_ITER + 6 * N + 1)) return st;
  s->n_kept = N;
  if (int st = copy_planes(s, dH, P_EH, true)) return st;
  if (int st = copy_planes(s, dV, P_EV, true)) return st;
  if (int st = copy_planes(s, target, P_T, true)) return st;
  if (confidence) {
    if (int st = copy_planes(s, confidence, P_C, true)) return st;
  } else {
    ProfScope ps(s->stream, DTSGB_K_SOFT);
    k_soft_fill<<<152 * 8, kST, 0, s->stream>>>(s->plane(P_C), s->total, 1.f);
  }
  DTSGB_CUDA(cudaMemcpyAsync(s->plane(P_ITER), s->plane(P_T), (size_t)s->total * 4,
                             cudaMemcpyDeviceToDevice, s->stream));
  const dim3 g = soft_grid(s);
  const int mode = p->loss == DTSGB_L2 ? 0 : 1;
  if (N > 0) {
    bool planned = false;
    if (int st = plan_windows_tiled(s, p->sigma_z, tau, &planned)) return st;
    if (!planned) {  // the walking kernels' fixed-point planes and halo, and a global plan
      if (int st = soft_halo(s, p->sigma_z, tau, &s->halo)) return st;
      if (int st = fix_edges(s, p->sigma_z, tau)) return st;
      if (int st = plan_windows(s)) return st;
    }
  }
  for (int k = 0; k < N; ++k) {
    if (int st = launch_half(s, s->plane(P_ITER + k), s->kept(0, k), s->plane(P_FH),
                             s->plane(P_T), s->plane(P_C), s->kept(1, k), s->kept(2, k), 0, 1,
                             mode, p->lambda, p->step_size))
      return st;
    if (int st = launch_half(s, s->kept(0, k), s->plane(P_ITER + k + 1), s->plane(P_FV),
                             nullptr, nullptr, s->kept(3, k), s->kept(4, k), 1, 0, mode,
                             p->lambda, p->step_size))
      return st;
  }
  DTSGB_CUDA(cudaGetLastError());
  if (int st = copy_planes(s, out, P_ITER + N, false)) return st;
  s->n_iter = N;
  s->opt = *p;
  s->tau = tau;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_soft_backward(dtsgb_soft_t s, const float* const* grad_out,
                                  float* const* grad_target, float* const* grad_confidence,
                                  float* const* grad_dH, float* const* grad_dV) {
  if (!s || !grad_out) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (s->n_iter < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "no soft solve to differentiate");
  const dtsgb_optimize_params& p = s->opt;
  const int N = s->n_iter, mode = p.loss == DTSGB_L2 ? 0 : 1;
  const float tau = s->tau, lam = p.lambda, step = p.step_size;
  if (int st = copy_planes(s, grad_out, P_G0, true)) return st;
  for (int k : {P_GT, P_GC, P_GEH, P_GEV, P_DIFF, P_DIFFY})
    DTSGB_CUDA(cudaMemsetAsync(s->plane(k), 0, (size_t)s->total * 4, s->stream));
  const dim3 g = soft_grid(s);
  float* a = s->plane(P_G0);
  float* b = s->plane(P_G1);
  for (int k = N - 1; k >= 0; --k) {
    float* vk = s->plane(P_ITER + k);
    float* uk = s->kept(0, k);  // the X half-step's result, the Y half-step's input
    if (s->use_plan) {
      // Y^T: a = dL/dv_{k+1} -> b = dL/du, and dL/ddV; X^T: b -> a = dL/dv_k,
      // dL/dt, dL/dc and dL/ddH
      if (int st = launch_adjoint_fused(s, a, s->kept(4, k), uk, nullptr, nullptr, b, nullptr,
                                        nullptr, 1, 0, mode, lam, step))
        return st;
      if (int st = launch_adjoint_fused(s, b, s->kept(2, k), vk, s->plane(P_T), s->plane(P_C),
                                        a, s->plane(P_GT), s->plane(P_GC), 0, 1, mode, lam,
                                        step))
        return st;
      continue;
    }
    // Y^T: a = dL/dv_{k+1} -> b = dL/du, and dL/ddV
    SOFT_LAUNCH(k_soft_pre, g, s->stream, s->d_inst, uk, a, s->kept(3, k), s->kept(4, k),
                nullptr, nullptr, s->plane(P_COEF), s->plane(P_ALPHA), s->plane(P_BETA),
                s->plane(P_ADIAG), nullptr, nullptr, 0, mode, lam, step);
    if (int st = launch_adjoint(s, s->plane(P_ADIAG), s->plane(P_COEF), s->plane(P_ALPHA),
                                s->plane(P_BETA), uk, s->plane(P_FV), b, 1, lam))
      return st;
    // X^T: b = dL/du -> a = dL/dv_k, dL/dt, dL/dc and dL/ddH
    SOFT_LAUNCH(k_soft_pre, g, s->stream, s->d_inst, vk, b, s->kept(1, k), s->kept(2, k),
                s->plane(P_T), s->plane(P_C), s->plane(P_COEF), s->plane(P_ALPHA),
                s->plane(P_BETA), s->plane(P_ADIAG), s->plane(P_GT), s->plane(P_GC), 1, mode,
                lam, step);
    if (int st = launch_adjoint(s, s->plane(P_ADIAG), s->plane(P_COEF), s->plane(P_ALPHA),
                                s->plane(P_BETA), vk, s->plane(P_FH), a, 0, lam))
      return st;
  }
  if (int st = launch_edge_scans(s, tau)) return st;
  // v_0 = t
  SOFT_LAUNCH(k_soft_axpy, g, s->stream, s->d_inst, a, s->plane(P_GT));
  DTSGB_CUDA(cudaGetLastError());
  const struct {
    float* const* dst;
    int plane;
  } outs[4] = {{grad_target, P_GT}, {grad_confidence, P_GC}, {grad_dH, P_GEH},
               {grad_dV, P_GEV}};
  for (const auto& o : outs)
    if (o.dst)
      if (int st = copy_planes(s, o.dst, o.plane, false)) return st;
  DTSGB_CUDA(cudaStreamSynchronize(s->stream));
  return DTSGB_OK;
}

}  // extern "C"
