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
// where D reaches sigma + tau/2 or at the line end).  One thread per pixel,
// global memory through L1: this mode exists for gradients with respect to
// the edge weights and for their finite-difference checks, not for speed.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/dtsgb.h"
#include "color.cuh"
#include "dtsgb_internal.cuh"

using namespace dtsgb;

namespace {

constexpr int kST = 256;

// Launches of this file's kernels, timed by the library's profiler as one
// kind (DTSGB_K_SOFT) when it is on.
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
enum {
  P_EH = 0, P_EV, P_T, P_C, P_U, P_COEF, P_B, P_HV, P_DIAG, P_G0, P_G1, P_GT, P_GC,
  P_GEH, P_GEV, P_ITER
};

__device__ __forceinline__ float ramp(float x) { return fminf(fmaxf(x + 0.5f, 0.f), 1.f); }

// A pixel's line: index i along it, length L, element stride st, pointer to
// element 0 of the line (plane base + instance offset).
struct Line {
  int i, L;
  long long st, base;
};

__device__ __forceinline__ bool pixel_line(const SInst& I, long long k, int axis, Line& ln) {
  const int y = (int)(k / I.w), x = (int)(k - (long long)y * I.w);
  if (axis == 0) {
    ln = Line{x, I.w, 1, I.off + (long long)y * I.w};
  } else {
    ln = Line{y, I.h, I.w, I.off + x};
  }
  return true;
}

// n(p) and sum_q w_pq val(q) over p's soft window.
__device__ __forceinline__ void soft_window(const float* __restrict__ e,
                                            const float* __restrict__ val, const Line& ln,
                                            float sigma, float tau, float* n_out,
                                            float* s_out) {
  const float wc = ramp(sigma / tau), stop = sigma + 0.5f * tau;
  float n = wc, S = wc * val[ln.base + ln.i * ln.st];
  float D = 0.f;
  for (int q = ln.i + 1; q < ln.L; ++q) {
    D += e[ln.base + q * ln.st];
    if (!(D < stop)) break;
    const float w = ramp((sigma - D) / tau);
    n += w;
    S = __fmaf_rn(w, val[ln.base + q * ln.st], S);
  }
  D = 0.f;
  for (int q = ln.i - 1; q >= 0; --q) {
    D += e[ln.base + (q + 1) * ln.st];
    if (!(D < stop)) break;
    const float w = ramp((sigma - D) / tau);
    n += w;
    S = __fmaf_rn(w, val[ln.base + q * ln.st], S);
  }
  *n_out = n;
  *s_out = S;
}

// Data term h and its derivatives with respect to the residual d = v - t
// (dh/dd), and to c (dh/dc), for confidence c and window weight n.
__device__ __forceinline__ void data_term(int mode, float v, float t, float c, float n,
                                          float* h, float* hd, float* hc) {
  const float d = v - t, cn = c / n;
  if (mode == 0) {  // L2: (c/n) d
    *h = cn * d;
    *hd = cn;
    *hc = d / n;
  } else {  // Charbonnier: 0.5 (c/n) d / sqrt(d^2 + 1e-6)
    const float q = d * d + 1e-6f, r = rsqrtf(q);
    *h = 0.5f * cn * d * r;
    *hd = 0.5f * cn * 1e-6f * r / q;
    *hc = 0.5f * d * r / n;
  }
}

// One soft half-step: vout = half-step(vin) along `axis`; data term on X.
__global__ void k_soft_half(const SInst* __restrict__ insts, const float* __restrict__ vin,
                            float* __restrict__ vout, const float* __restrict__ e,
                            const float* __restrict__ t, const float* __restrict__ c,
                            int axis, int data, int mode, float sigma, float tau,
                            float lambda, float step) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    Line ln;
    pixel_line(I, k, axis, ln);
    float n, S;
    soft_window(e, vin, ln, sigma, tau, &n, &S);
    const long long p = I.off + k;
    const float v = vin[p], B = S / n;
    float h = 0.f, hd, hc;
    if (data) data_term(mode, v, t[p], c[p], n, &h, &hd, &hc);
    vout[p] = v - step * (lambda * (v - B) + h);
  }
}

// Adjoint, first pass of a half-step: per pixel p the window weight n(p),
// mean B(p), data term h(p), coef(p) = a(p) s / n(p) and the diagonal factor
// 1 - s*lambda - s*h'(p); on X also the local dL/dt, dL/dc terms.
__global__ void k_soft_pre(const SInst* __restrict__ insts, const float* __restrict__ val,
                           const float* __restrict__ a, const float* __restrict__ e,
                           const float* __restrict__ t, const float* __restrict__ c,
                           float* __restrict__ coef, float* __restrict__ Bo,
                           float* __restrict__ ho, float* __restrict__ diag,
                           float* __restrict__ gt, float* __restrict__ gc, int axis, int data,
                           int mode, float sigma, float tau, float lambda, float step) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    Line ln;
    pixel_line(I, k, axis, ln);
    float n, S;
    soft_window(e, val, ln, sigma, tau, &n, &S);
    const long long p = I.off + k;
    const float ap = a[p];
    float h = 0.f, hd = 0.f, hc = 0.f;
    if (data) {
      data_term(mode, val[p], t[p], c[p], n, &h, &hd, &hc);
      gt[p] += ap * step * hd;  // dh/dt = -dh/dd, and v' has -s*h
      gc[p] -= ap * step * hc;
    }
    coef[p] = ap * step / n;
    Bo[p] = S / n;
    ho[p] = h;
    diag[p] = 1.f - step * lambda - step * hd;
  }
}

// Adjoint, second pass: dL/d(half-step input) = a * diag + lambda * sum_p
// coef(p) w_pq (the weights are symmetric, so q walks its own window).
__global__ void k_soft_scatter(const SInst* __restrict__ insts, const float* __restrict__ a,
                               const float* __restrict__ coef, const float* __restrict__ diag,
                               const float* __restrict__ e, float* __restrict__ aout,
                               int axis, float sigma, float tau, float lambda) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    Line ln;
    pixel_line(I, k, axis, ln);
    float n, S;
    soft_window(e, coef, ln, sigma, tau, &n, &S);
    const long long p = I.off + k;
    aout[p] = __fmaf_rn(lambda, S, a[p] * diag[p]);
  }
}

// Adjoint, third pass: dL/de(j) for the edge weight between j-1 and j on the
// line, from every pair a < j <= b whose distance is on the ramp.
__global__ void k_soft_edge(const SInst* __restrict__ insts, const float* __restrict__ val,
                            const float* __restrict__ coef, const float* __restrict__ Bv,
                            const float* __restrict__ hv, const float* __restrict__ e,
                            float* __restrict__ ge, int axis, float sigma, float tau,
                            float lambda) {
  const SInst I = insts[blockIdx.y];
  const long long npx = (long long)I.w * I.h;
  const float lo = sigma - 0.5f * tau, hi = sigma + 0.5f * tau;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx;
       k += (long long)gridDim.x * blockDim.x) {
    Line ln;
    pixel_line(I, k, axis, ln);
    const int j = ln.i;
    if (j == 0) continue;  // e(0) enters no distance
    const float ej = e[ln.base + j * ln.st];
    float acc = 0.f, D0 = 0.f;  // D0 = sum of e over a < i < j
    for (int ia = j - 1; ia >= 0; --ia) {
      if (ia < j - 1) D0 += e[ln.base + (ia + 1) * ln.st];
      if (!(D0 + ej < hi)) break;
      const long long pa = ln.base + ia * ln.st;
      const float ca = coef[pa], Ba = Bv[pa], ha = hv[pa], va = val[pa];
      float D = D0;
      for (int ib = j; ib < ln.L; ++ib) {
        D += e[ln.base + ib * ln.st];
        if (!(D < hi)) break;
        if (D > lo) {
          const long long pb = ln.base + ib * ln.st;
          // G_ab (b in a's window) + G_ba (a in b's window)
          acc += ca * (lambda * (val[pb] - Ba) + ha) +
                 coef[pb] * (lambda * (va - Bv[pb]) + hv[pb]);
        }
      }
    }
    ge[I.off + k] -= acc / tau;
  }
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
  if (!st && cudaMemcpy(s->d_inst, s->inst.data(), n * sizeof(SInst),
                        cudaMemcpyHostToDevice) != cudaSuccess)
    st = fail(DTSGB_ERR_CUDA, "instance table upload");
  if (!st && cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
    st = fail(DTSGB_ERR_CUDA, "stream creation");
  if (st) {
    dfree(s->d_inst);
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
  k_soft_edges<<<soft_grid(s), kST, 0, s->stream>>>(s->d_inst, g, rx, ry, s->plane(P_EH),
                                                    s->plane(P_EV));
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
  if (int st = ensure_planes(s, P_ITER + N + 1)) return st;
  if (int st = copy_planes(s, dH, P_EH, true)) return st;
  if (int st = copy_planes(s, dV, P_EV, true)) return st;
  if (int st = copy_planes(s, target, P_T, true)) return st;
  if (confidence) {
    if (int st = copy_planes(s, confidence, P_C, true)) return st;
  } else {
    k_soft_fill<<<152 * 8, kST, 0, s->stream>>>(s->plane(P_C), s->total, 1.f);
  }
  DTSGB_CUDA(cudaMemcpyAsync(s->plane(P_ITER), s->plane(P_T), (size_t)s->total * 4,
                             cudaMemcpyDeviceToDevice, s->stream));
  const dim3 g = soft_grid(s);
  const int mode = p->loss == DTSGB_L2 ? 0 : 1;
  for (int k = 0; k < N; ++k) {
    SOFT_LAUNCH(k_soft_half, g, s->stream, s->d_inst, s->plane(P_ITER + k), s->plane(P_U),
                                          s->plane(P_EH), s->plane(P_T), s->plane(P_C), 0,
                                          1, mode, p->sigma_z, tau, p->lambda, p->step_size);
    SOFT_LAUNCH(k_soft_half, g, s->stream, s->d_inst, s->plane(P_U), s->plane(P_ITER + k + 1),
                                          s->plane(P_EV), nullptr, nullptr, 1, 0, mode,
                                          p->sigma_z, tau, p->lambda, p->step_size);
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
  const float tau = s->tau, sg = p.sigma_z, lam = p.lambda, step = p.step_size;
  if (int st = copy_planes(s, grad_out, P_G0, true)) return st;
  for (int k : {P_GT, P_GC, P_GEH, P_GEV})
    DTSGB_CUDA(cudaMemsetAsync(s->plane(k), 0, (size_t)s->total * 4, s->stream));
  const dim3 g = soft_grid(s);
  float* a = s->plane(P_G0);
  float* b = s->plane(P_G1);
  for (int k = N - 1; k >= 0; --k) {
    float* vk = s->plane(P_ITER + k);
    // u = X half-step of v_k (the Y half-step's input)
    SOFT_LAUNCH(k_soft_half, g, s->stream, s->d_inst, vk, s->plane(P_U), s->plane(P_EH),
                                          s->plane(P_T), s->plane(P_C), 0, 1, mode, sg, tau,
                                          lam, step);
    // Y^T: a = dL/dv_{k+1} -> b = dL/du, and dL/ddV
    SOFT_LAUNCH(k_soft_pre, g, s->stream, s->d_inst, s->plane(P_U), a, s->plane(P_EV),
                                         nullptr, nullptr, s->plane(P_COEF), s->plane(P_B),
                                         s->plane(P_HV), s->plane(P_DIAG), nullptr, nullptr,
                                         1, 0, mode, sg, tau, lam, step);
    SOFT_LAUNCH(k_soft_scatter, g, s->stream, s->d_inst, a, s->plane(P_COEF),
                                             s->plane(P_DIAG), s->plane(P_EV), b, 1, sg, tau,
                                             lam);
    SOFT_LAUNCH(k_soft_edge, g, s->stream, s->d_inst, s->plane(P_U), s->plane(P_COEF),
                                          s->plane(P_B), s->plane(P_HV), s->plane(P_EV),
                                          s->plane(P_GEV), 1, sg, tau, lam);
    // X^T: b = dL/du -> a = dL/dv_k, dL/dt, dL/dc and dL/ddH
    SOFT_LAUNCH(k_soft_pre, g, s->stream, s->d_inst, vk, b, s->plane(P_EH), s->plane(P_T),
                                         s->plane(P_C), s->plane(P_COEF), s->plane(P_B),
                                         s->plane(P_HV), s->plane(P_DIAG), s->plane(P_GT),
                                         s->plane(P_GC), 0, 1, mode, sg, tau, lam, step);
    SOFT_LAUNCH(k_soft_scatter, g, s->stream, s->d_inst, b, s->plane(P_COEF),
                                             s->plane(P_DIAG), s->plane(P_EH), a, 0, sg, tau,
                                             lam);
    SOFT_LAUNCH(k_soft_edge, g, s->stream, s->d_inst, vk, s->plane(P_COEF), s->plane(P_B),
                                          s->plane(P_HV), s->plane(P_EH), s->plane(P_GEH), 0,
                                          sg, tau, lam);
  }
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
