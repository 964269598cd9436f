/*
 * CPU oracle for the DTS / HFBS hot path -- TEST INFRASTRUCTURE ONLY.
 * See oracle.h for what it is, how it is built and why parity is unpinned.
 * Every function cites the reference file:line it restates.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define EXPORT __attribute__((visibility("default")))

#if defined(ORA_REAL_IS_FLOAT)
#define R_SQRT sqrtf
#define R_FMA fmaf
#define R_EXP expf
#else
#define R_SQRT sqrt
#define R_FMA fma
#define R_EXP exp
#endif

EXPORT int ora_real_bytes(void) { return (int)sizeof(REAL); }

/* Worker threads of the OpenMP loops (timing of the CPU baseline at one
 * thread and at all host threads); 0 restores the default. */
#ifdef _OPENMP
#include <omp.h>
EXPORT void ora_set_threads(int n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }
EXPORT int ora_get_threads(void) { return omp_get_max_threads(); }
#else
EXPORT void ora_set_threads(int n) { (void)n; }
EXPORT int ora_get_threads(void) { return 1; }
#endif

/* ======================================================================
 * a1. Colour conversion -- src/color_space.cuh:11-40.
 * The reference evaluates double expressions and converts to unsigned char
 * (truncation toward zero; every value lies in [0, 255.5]).
 *   Y  = R*0.299 + 0.587*G + 0.114*B              (color_space.cuh:19,36)
 *   Cb = 128 - R*0.168736 - 0.331264*G + 0.5*B     (color_space.cuh:20)
 *   Cr = 128 + R*0.5 - 0.418688*G - 0.081312*B     (color_space.cuh:21)
 * contract selects the evaluation order:
 *   0: every multiply and add rounded on its own;
 *   1: nvcc's default contraction with the first product of Y fused,
 *      Y = fma(0.114,B, fma(R,0.299, 0.587*G));
 *   2: the same but the second product of Y fused,
 *      Y = fma(0.114,B, fma(0.587,G, R*0.299)).
 * Cb and Cr have one contraction order only:
 *      Cb = fma(0.5,B, fma(-0.331264,G, fma(-R,0.168736,128)))
 *      Cr = fma(-0.081312,B, fma(-0.418688,G, fma(R,0.5,128)))
 * ====================================================================== */
static double ora_y_expr(int r, int g, int b, int contract) {
  const double R = r, G = g, B = b;
  if (contract == 0) {
    volatile double t1 = R * 0.299, t2 = 0.587 * G, t3 = 0.114 * B;
    volatile double s = t1 + t2;
    return s + t3;
  }
  if (contract == 1) return fma(0.114, B, fma(R, 0.299, 0.587 * G));
  return fma(0.114, B, fma(0.587, G, R * 0.299));
}
static double ora_cb_expr(int r, int g, int b, int contract) {
  const double R = r, G = g, B = b;
  if (contract == 0) {
    volatile double t1 = R * 0.168736, t2 = 0.331264 * G, t3 = 0.5 * B;
    volatile double s = 128.0 - t1;
    s = s - t2;
    return s + t3;
  }
  return fma(0.5, B, fma(-0.331264, G, fma(-R, 0.168736, 128.0)));
}
static double ora_cr_expr(int r, int g, int b, int contract) {
  const double R = r, G = g, B = b;
  if (contract == 0) {
    volatile double t1 = R * 0.5, t2 = 0.418688 * G, t3 = 0.081312 * B;
    volatile double s = 128.0 + t1;
    s = s - t2;
    return s - t3;
  }
  return fma(-0.081312, B, fma(-0.418688, G, fma(R, 0.5, 128.0)));
}
static uint8_t ora_to_u8(double v) { return (uint8_t)(int)v; }

EXPORT void ora_color_convert(int color_space, int contract, const uint8_t* in,
                              uint8_t* out, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const int r = in[4 * i], g = in[4 * i + 1], b = in[4 * i + 2];
    const uint8_t a = in[4 * i + 3];
    uint8_t o0 = (uint8_t)r, o1 = (uint8_t)g, o2 = (uint8_t)b;
    if (color_space == ORA_YCBCR) {
      o0 = ora_to_u8(ora_y_expr(r, g, b, contract));
      o1 = ora_to_u8(ora_cb_expr(r, g, b, contract));
      o2 = ora_to_u8(ora_cr_expr(r, g, b, contract));
    } else if (color_space == ORA_YYY) {
      o0 = o1 = o2 = ora_to_u8(ora_y_expr(r, g, b, contract));
    }
    out[4 * i] = o0;
    out[4 * i + 1] = o1;
    out[4 * i + 2] = o2;
    out[4 * i + 3] = a;
  }
}

/* ======================================================================
 * DTS state: the buffers of DomainTransformFilterStruct
 * (src/domain_transform_filter_struct.cuh:10-63) and
 * DomainTransformSolverStruct (src/domain_transform_solver_struct.cuh:10-29),
 * stored densely (row pitch = current width) and in natural orientation
 * (the reference stores ct_V and the Y sums transposed; only the layout
 * differs).
 * ====================================================================== */
#define ORA_MAX_OVR 16
struct ora_dts {
  int max_w, max_h, w, h;
  int ref_y_limit, contract;
  uint8_t* color;
  REAL *dH, *dV, *ctH, *ctV, *var, *target, *conf;
  /* the solver's own filter params (filter_params_, set only by its public
   * ComputeColorSpaceDifferential, src/domain_transform_solver.cu:89-93) */
  float fp_sx, fp_sy, fp_sr;
  /* DomainTransformStereo: right image, its dHdx, centre offset */
  uint8_t* right_color;
  REAL* right_dH;
  float center_offset;
  int n_ovr;
  int ovr_axis[ORA_MAX_OVR];
  float ovr_sigma[ORA_MAX_OVR];
  int32_t *ovr_l[ORA_MAX_OVR], *ovr_u[ORA_MAX_OVR];
};

static REAL* ora_alloc_real(size_t n) { return (REAL*)calloc(n, sizeof(REAL)); }

EXPORT ora_dts* ora_dts_create(int max_w, int max_h) {
  ora_dts* s = (ora_dts*)calloc(1, sizeof(ora_dts));
  const size_t n = (size_t)max_w * max_h;
  s->max_w = s->w = max_w;
  s->max_h = s->h = max_h;
  s->ref_y_limit = 1;
  s->contract = ORA_CONTRACT_NVCC;
  s->color = (uint8_t*)calloc(n * 4, 1);
  s->dH = ora_alloc_real(n);
  s->dV = ora_alloc_real(n);
  s->ctH = ora_alloc_real(n);
  s->ctV = ora_alloc_real(n);
  s->var = ora_alloc_real(n);
  s->target = ora_alloc_real(n);
  s->conf = ora_alloc_real(n);
  s->right_color = (uint8_t*)calloc(n * 4, 1);
  s->right_dH = ora_alloc_real(n);
  return s;
}

EXPORT void ora_dts_clear_bounds_override(ora_dts* s) {
  for (int i = 0; i < s->n_ovr; ++i) {
    free(s->ovr_l[i]);
    free(s->ovr_u[i]);
  }
  s->n_ovr = 0;
}

EXPORT void ora_dts_destroy(ora_dts* s) {
  if (!s) return;
  ora_dts_clear_bounds_override(s);
  free(s->color);
  free(s->dH);
  free(s->dV);
  free(s->ctH);
  free(s->ctV);
  free(s->var);
  free(s->target);
  free(s->conf);
  free(s->right_color);
  free(s->right_dH);
  free(s);
}

EXPORT void ora_dts_set_compat(ora_dts* s, int ref_y_limit, int contract) {
  s->ref_y_limit = ref_y_limit;
  s->contract = contract;
}

/* DomainTransformFilter::SetImageDim -- src/domain_transform_filter.cu:114-122
 * (invalid dims are reported and ignored). */
EXPORT int ora_dts_set_image_dim(ora_dts* s, int w, int h) {
  if (w > 0 && w <= s->max_w && h > 0 && h <= s->max_h) {
    s->w = w;
    s->h = h;
    return 0;
  }
  return -1;
}

/* ClearAll -- src/domain_transform_filter.cu:202-216,
 * src/domain_transform_solver.cu:248-255. */
EXPORT void ora_dts_clear_all(ora_dts* s) {
  const size_t n = (size_t)s->max_w * s->max_h;
  memset(s->color, 0, n * 4);
  memset(s->dH, 0, n * sizeof(REAL));
  memset(s->dV, 0, n * sizeof(REAL));
  memset(s->ctH, 0, n * sizeof(REAL));
  memset(s->ctV, 0, n * sizeof(REAL));
  memset(s->var, 0, n * sizeof(REAL));
  memset(s->target, 0, n * sizeof(REAL));
  memset(s->conf, 0, n * sizeof(REAL));
}

/* InitFrame -- src/domain_transform_filter.cu:18-49 and
 * src/domain_transform_solver.cu:46-61 (confidence NULL -> all ones). */
EXPORT void ora_dts_init_frame(ora_dts* s, int color_space, const uint8_t* rgba,
                               const float* target, const float* confidence) {
  const int64_t n = (int64_t)s->w * s->h;
  ora_color_convert(color_space, s->contract, rgba, s->color, n);
  if (target)
    for (int64_t i = 0; i < n; ++i) s->target[i] = (REAL)target[i];
  if (confidence) {
    for (int64_t i = 0; i < n; ++i) s->conf[i] = (REAL)confidence[i];
  } else {
    const size_t nmax = (size_t)s->max_w * s->max_h;
    for (size_t i = 0; i < nmax; ++i) s->conf[i] = 1;
  }
}

/* Target and confidence at the oracle's own precision (NULL keeps a plane);
 * used by finite-difference checks, whose perturbations a float would round
 * away. */
EXPORT void ora_dts_set_target_conf(ora_dts* s, const REAL* target,
                                    const REAL* confidence) {
  const int64_t n = (int64_t)s->w * s->h;
  if (target) memcpy(s->target, target, (size_t)n * sizeof(REAL));
  if (confidence) memcpy(s->conf, confidence, (size_t)n * sizeof(REAL));
}

/* a2. dHdx / dVdy -- src/domain_transform_common_kernels.cuh:71-116 and
 * ComputeColorSpaceDifferential, src/domain_transform_filter.cu:92-110.
 * The backward neighbour of column 0 / row 0 is read through a surface with
 * zero boundary mode, i.e. (0,0,0,0). */
static const float kInv255Sq = (float)0.0000153787; /* common_kernels.cuh:10 */

static REAL ora_edge(const uint8_t* a, const uint8_t* b, float ratio) {
  int ssd = 0;
  for (int k = 0; k < 4; ++k) {
    const int d = (int)a[k] - (int)b[k];
    ssd += d * d;
  }
  REAL t = (REAL)ssd * (REAL)kInv255Sq;
  t = t * (REAL)ratio;
  return R_SQRT(R_FMA(t, (REAL)ratio, (REAL)1));
}

static void ora_edges(const uint8_t* color, int W, int H, float rx, float ry,
                      REAL* dH, REAL* dV) {
  static const uint8_t zero4[4] = {0, 0, 0, 0};
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      const uint8_t* cur = color + 4 * ((size_t)y * W + x);
      const uint8_t* left = x > 0 ? cur - 4 : zero4;
      const uint8_t* up = y > 0 ? cur - 4 * (size_t)W : zero4;
      dH[(size_t)y * W + x] = ora_edge(cur, left, rx);
      dV[(size_t)y * W + x] = ora_edge(cur, up, ry);
    }
  }
}

/* DomainTransformFilter::ComputeColorSpaceDifferential: the DT of the
 * current guide for these sigmas (Filter calls this base version, which does
 * not touch the solver's filter_params_). */
static void dts_diff(ora_dts* s, float sigma_x, float sigma_y, float sigma_r) {
  ora_edges(s->color, s->w, s->h, sigma_x / sigma_r, sigma_y / sigma_r, s->dH,
            s->dV);
}

/* DomainTransformSolver::ComputeColorSpaceDifferential
 * (src/domain_transform_solver.cu:89-93): records filter_params_ too. */
EXPORT void ora_dts_differential(ora_dts* s, float sigma_x, float sigma_y,
                                 float sigma_r) {
  s->fp_sx = sigma_x;
  s->fp_sy = sigma_y;
  s->fp_sr = sigma_r;
  dts_diff(s, sigma_x, sigma_y, sigma_r);
}

/* DomainTransformStereo::InitRightFrame / ProcessRightFrame
 * (src/domain_transform_stereo.cu:17-27): the right image in the same colour
 * space, and its dHdx for the solver's filter_params_. */
EXPORT void ora_dts_init_right_frame(ora_dts* s, float center_offset,
                                     int color_space, const uint8_t* rgba) {
  s->center_offset = center_offset;
  ora_color_convert(color_space, s->contract, rgba, s->right_color,
                    (int64_t)s->w * s->h);
}

EXPORT void ora_dts_process_right_frame(ora_dts* s) {
  const size_t n = (size_t)s->w * s->h;
  REAL* dv = ora_alloc_real(n);
  ora_edges(s->right_color, s->w, s->h, s->fp_sx / s->fp_sr, s->fp_sy / s->fp_sr,
            s->right_dH, dv);
  free(dv);
}

/* a3. IntegrateColorDifferentials -- src/domain_transform_filter.cu:85-90,
 * src/domain_transform_common_functions.h:44-99: inclusive prefix sums of dH
 * along rows (ct_H) and of dV along columns (ct_V).  The reference sums with
 * a CUB block scan; the oracle sums sequentially. */
static void ora_row_prefix(const REAL* in, REAL* out, int W, int H) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y) {
    REAL acc = 0;
    for (int x = 0; x < W; ++x) {
      acc += in[(size_t)y * W + x];
      out[(size_t)y * W + x] = acc;
    }
  }
}
static void ora_col_prefix(const REAL* in, REAL* out, int W, int H) {
#pragma omp parallel for schedule(static)
  for (int x = 0; x < W; ++x) {
    REAL acc = 0;
    for (int y = 0; y < H; ++y) {
      acc += in[(size_t)y * W + x];
      out[(size_t)y * W + x] = acc;
    }
  }
}

EXPORT void ora_dts_integrate(ora_dts* s) {
  ora_row_prefix(s->dH, s->ctH, s->w, s->h);
  ora_col_prefix(s->dV, s->ctV, s->w, s->h);
}

/* a4. LinearSearchLowerAndUpperBound2DX -- src/domain_transform_filter.cuh:7-28.
 *   lower = first i <= p (descending) with ct(p) - sigma > ct(i), else p-1;
 *   upper = (first i >= p, i < limit, with ct(p) + sigma < ct(i)) - 1, else p.
 * ct(i) is ct[i*stride]; n is the number of valid entries along the axis.
 * limit may exceed n (the Y-pass quirk); entries past n read as zero in the
 * reference's zero-filled allocation and never satisfy the upper test, so
 * the effective limit is min(limit, n). */
static void ora_search(const REAL* ct, size_t stride, int p, int n, int limit,
                       REAL sigma, int32_t* lo, int32_t* up, REAL* margin) {
  const REAL val = ct[(size_t)p * stride];
  const REAL lthr = val - sigma, uthr = val + sigma;
  int l = p - 1, u = p;
  REAL m = INFINITY, d;
  int found = 0;
  for (int i = p; i >= 0; --i) {
    if (lthr > ct[(size_t)i * stride]) {
      l = i;
      found = 1;
      break;
    }
  }
  if (found) {
    d = lthr - ct[(size_t)l * stride];
    if (d < m) m = d;
    d = ct[(size_t)(l + 1) * stride] - lthr;
    if (d < m) m = d;
  } else {
    d = ct[0] - lthr;
    if (d < m) m = d;
  }
  const int lim = limit < n ? limit : n;
  found = 0;
  int i;
  for (i = p; i < lim; ++i) {
    if (uthr < ct[(size_t)i * stride]) {
      u = i - 1;
      found = 1;
      break;
    }
  }
  if (found) {
    d = ct[(size_t)i * stride] - uthr;
    if (d < m) m = d;
    d = uthr - ct[(size_t)(i - 1) * stride];
    if (d < m) m = d;
  } else if (p < lim) {
    d = uthr - ct[(size_t)(lim - 1) * stride];
    if (d < m) m = d;
  }
  *lo = l;
  *up = u;
  if (margin) *margin = m;
}

static int ora_y_limit(const ora_dts* s) {
  return s->ref_y_limit ? s->w : s->h;
}

EXPORT void ora_dts_bounds(const ora_dts* s, int axis, float sigma, int32_t* l,
                           int32_t* u, REAL* margin) {
  const int W = s->w, H = s->h;
  if (axis == 0) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const size_t k = (size_t)y * W + x;
        ora_search(s->ctH + (size_t)y * W, 1, x, W, W, (REAL)sigma, l + k,
                   u + k, margin ? margin + k : NULL);
      }
  } else {
    const int lim = ora_y_limit(s);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < W; ++x)
      for (int y = 0; y < H; ++y) {
        const size_t k = (size_t)y * W + x;
        ora_search(s->ctV + x, (size_t)W, y, H, lim, (REAL)sigma, l + k, u + k,
                   margin ? margin + k : NULL);
      }
  }
}

EXPORT void ora_dts_add_bounds_override(ora_dts* s, int axis, float sigma,
                                        const int32_t* l, const int32_t* u) {
  if (s->n_ovr >= ORA_MAX_OVR) return;
  const size_t n = (size_t)s->w * s->h;
  const int k = s->n_ovr++;
  s->ovr_axis[k] = axis;
  s->ovr_sigma[k] = sigma;
  s->ovr_l[k] = (int32_t*)malloc(n * sizeof(int32_t));
  s->ovr_u[k] = (int32_t*)malloc(n * sizeof(int32_t));
  memcpy(s->ovr_l[k], l, n * sizeof(int32_t));
  memcpy(s->ovr_u[k], u, n * sizeof(int32_t));
}

/* Bounds for one pass: the override for (axis, sigma) if present, else the
 * reference search.  Caller frees. */
static void ora_pass_bounds(const ora_dts* s, int axis, float sigma,
                            int32_t** l, int32_t** u) {
  const size_t n = (size_t)s->w * s->h;
  *l = (int32_t*)malloc(n * sizeof(int32_t));
  *u = (int32_t*)malloc(n * sizeof(int32_t));
  for (int k = 0; k < s->n_ovr; ++k) {
    if (s->ovr_axis[k] == axis && s->ovr_sigma[k] == sigma) {
      memcpy(*l, s->ovr_l[k], n * sizeof(int32_t));
      memcpy(*u, s->ovr_u[k], n * sizeof(int32_t));
      return;
    }
  }
  ora_dts_bounds(s, axis, sigma, *l, *u, NULL);
}

/* Window mean (S(u) - S(l)) / (u - l) over a prefix sum S along one axis;
 * S(-1) reads the slot before the row in the reference (pitch padding); the
 * oracle defines it as 0. */
static REAL ora_window_mean(const REAL* S, size_t stride, int l, int u) {
  const REAL su = S[(size_t)u * stride];
  const REAL sl = l >= 0 ? S[(size_t)l * stride] : (REAL)0;
  return (su - sl) / (REAL)(u - l);
}

/* a5. FilterX / FilterY -- src/domain_transform_filter.cuh:30-71. */
static void ora_box_pass(const ora_dts* s, int axis, const REAL* in, REAL* out,
                         const int32_t* l, const int32_t* u) {
  const int W = s->w, H = s->h;
  const size_t n = (size_t)W * H;
  REAL* S = ora_alloc_real(n);
  if (axis == 0) {
    ora_row_prefix(in, S, W, H);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const size_t k = (size_t)y * W + x;
        out[k] = ora_window_mean(S + (size_t)y * W, 1, l[k], u[k]);
      }
  } else {
    ora_col_prefix(in, S, W, H);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const size_t k = (size_t)y * W + x;
        out[k] = ora_window_mean(S + x, (size_t)W, l[k], u[k]);
      }
  }
  free(S);
}

/* DomainTransformFilter::Filter -- src/domain_transform_filter.cu:124-188:
 * recompute the DT for these sigmas, then num_iter x {X box, Y box} with the
 * sigma schedule: iteration 0 unscaled, iteration i>=1 scaled by
 * 3*2^(N-i-1)/sqrt(4^N-1) (computed in double, stored as float). */
static void ora_filter_buffers(ora_dts* s, float sx, float sy, float sr,
                               const REAL* in, REAL* out, int num_iter) {
  dts_diff(s, sx, sy, sr);
  ora_dts_integrate(s);
  const size_t n = (size_t)s->w * s->h;
  REAL* a = ora_alloc_real(n);
  REAL* b = ora_alloc_real(n);
  memcpy(a, in, n * sizeof(REAL));
  for (int it = 0; it < num_iter; ++it) {
    float sig_x = sx, sig_y = sy;
    if (it != 0) {
      const float mult = (float)(3 * pow(2.0, (double)(num_iter - (it + 1))) /
                                 sqrt(pow(4.0, (double)num_iter) - 1));
      sig_x *= mult;
      sig_y *= mult;
    }
    int32_t *l, *u;
    ora_pass_bounds(s, 0, sig_x, &l, &u);
    ora_box_pass(s, 0, a, b, l, u);
    free(l);
    free(u);
    ora_pass_bounds(s, 1, sig_y, &l, &u);
    ora_box_pass(s, 1, b, a, l, u);
    free(l);
    free(u);
  }
  memcpy(s->var, a, n * sizeof(REAL));
  memcpy(out, a, n * sizeof(REAL));
  free(a);
  free(b);
}

EXPORT void ora_dts_filter(ora_dts* s, float sx, float sy, float sr,
                           const float* in, REAL* out, int num_iter) {
  const size_t n = (size_t)s->w * s->h;
  REAL* tmp = ora_alloc_real(n);
  for (size_t i = 0; i < n; ++i) tmp[i] = (REAL)in[i];
  ora_filter_buffers(s, sx, sy, sr, tmp, out, num_iter);
  free(tmp);
}

/* a8. ComputeConfidence -- src/domain_transform_solver.cu:206-246 and
 * ComputeConfidenceKernel :21-44.  conf = exp(-(DT(t^2)-DT(t)^2)*0.5/s0^2)
 * for x > left_clear (so column 0 is always cleared), 0 when the variance is
 * negative or not finite.  The two Filter calls leave the DT of the
 * confidence sigmas in place for any later Optimize. */
EXPORT void ora_dts_compute_confidence(ora_dts* s, float sx, float sy, float sr,
                                       float sigma0, int left_clear) {
  const int W = s->w, H = s->h;
  const size_t n = (size_t)W * H;
  REAL* dtz = ora_alloc_real(n);
  REAL* sq = ora_alloc_real(n);
  REAL* dtz2 = ora_alloc_real(n);
  ora_filter_buffers(s, sx, sy, sr, s->target, dtz, 3);
  for (size_t i = 0; i < n; ++i) sq[i] = s->target[i] * s->target[i];
  ora_filter_buffers(s, sx, sy, sr, sq, dtz2, 3);
  const float scale = 0.5f / (sigma0 * sigma0);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t k = (size_t)y * W + x;
      REAL c = 0;
      if (x > left_clear) {
        const REAL var = dtz2[k] - dtz[k] * dtz[k];
        c = (var < 0 || !isfinite(var)) ? (REAL)0 : R_EXP(-var * (REAL)scale);
      }
      s->conf[k] = c;
    }
  free(dtz);
  free(sq);
  free(dtz2);
}

/* a6/a7. DomainTransformSolver::Optimize -- src/domain_transform_solver.cu:
 * 100-202 with OptimizeX / OptimizeY, src/domain_transform_solver.cuh:12-116.
 *   X: v' = v - s*(lambda*(v - B_x) + 0.5*g),
 *      g = 2*(c/n)*(v-t)                  (L2)
 *      g = (c/n)*(v-t)/sqrt((v-t)^2+1e-6) (Charbonnier)
 *   Y: v' = v - s*lambda*(v - B_y)
 * sigma is sigma_z in every iteration (kDMIter = 1).  RobustLoss::L1 has no
 * kernel in either switch, so the result stays the target.  With
 * overwrite in (0,1) the target is copied over v where c > overwrite before
 * each half-step (CopyVariableFlagGreaterThanThresh, common_kernels.cuh:36-50).
 */
static void dts_optimize(ora_dts* s, int num_iterations, int loss,
                         float lambda, float sigma_z, float step,
                         float overwrite, int stereo, float photo_lambda);

EXPORT void ora_dts_optimize(ora_dts* s, int num_iterations, int loss,
                             float lambda, float sigma_z, float step,
                             float overwrite) {
  dts_optimize(s, num_iterations, loss, lambda, sigma_z, step, overwrite, 0, 0.f);
}

/* DomainTransformStereo::Optimize (src/domain_transform_stereo.cu:44-158):
 * Optimize with PhotometricL2LossTerm (src/domain_transform_loss_term.cuh:
 * 20-39) added to the data gradient of the X half-step:
 *   xr = center_offset + x - v;  if 0 <= xr < W:
 *   g += lambda_p * 2 * SAD4(left(x,y), right((int)xr, y)) / 255
 *        * ((dH_right((int)xr, y)^2 - 1) * (sigma_r / sigma_x)^2)
 * with the solver's filter_params_ sigmas. */
EXPORT void ora_dts_optimize_stereo(ora_dts* s, int num_iterations, int loss,
                                    float lambda, float sigma_z, float step,
                                    float photo_lambda, float overwrite) {
  dts_optimize(s, num_iterations, loss, lambda, sigma_z, step, overwrite, 1,
               photo_lambda);
}

static const float kInv255 = (float)0.00392156863; /* common_kernels.cuh:9 */

static REAL photometric(const ora_dts* s, int x, int y, REAL d, REAL alpha,
                        REAL lam_p) {
  const int W = s->w;
  const REAL xr = (REAL)s->center_offset + (REAL)x - d;
  if (!(xr >= 0 && xr < (REAL)W)) return 0;
  const int xi = (int)xr;
  const uint8_t* a = s->color + 4 * ((size_t)y * W + x);
  const uint8_t* b = s->right_color + 4 * ((size_t)y * W + xi);
  int sad = 0;
  for (int k = 0; k < 4; ++k) sad += abs((int)a[k] - (int)b[k]);
  const REAL gr = s->right_dH[(size_t)y * W + xi];
  return lam_p * 2 * ((REAL)sad * (REAL)kInv255) * ((gr * gr - 1) * alpha);
}

static void dts_optimize(ora_dts* s, int num_iterations, int loss,
                         float lambda, float sigma_z, float step,
                         float overwrite, int stereo, float photo_lambda) {
  const int W = s->w, H = s->h;
  const float sxr = s->fp_sr / s->fp_sx;  /* "sigma_x_div_sigma_r", stereo.cu:80 */
  const REAL alpha = (REAL)(sxr * sxr);
  const size_t n = (size_t)W * H;
  REAL* v = ora_alloc_real(n);
  REAL* S = ora_alloc_real(n);
  memcpy(v, s->target, n * sizeof(REAL));
  const int do_over = overwrite > 0 && overwrite < 1;
  if (loss != ORA_L2 && loss != ORA_CHARBONNIER) {
    memcpy(s->var, v, n * sizeof(REAL));
    free(v);
    free(S);
    return;
  }
  int32_t *lx, *ux, *ly, *uy;
  ora_pass_bounds(s, 0, sigma_z, &lx, &ux);
  ora_pass_bounds(s, 1, sigma_z, &ly, &uy);
  const REAL lam = lambda, st = step;
  for (int it = 0; it < num_iterations; ++it) {
    if (do_over)
      for (size_t k = 0; k < n; ++k)
        if (s->conf[k] > (REAL)overwrite) v[k] = s->target[k];
    ora_row_prefix(v, S, W, H);
    REAL* vx = ora_alloc_real(n);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
      for (int x = 0; x < W; ++x) {
        const size_t k = (size_t)y * W + x;
        const int l = lx[k], u = ux[k];
        const REAL B = ora_window_mean(S + (size_t)y * W, 1, l, u);
        const REAL cn = s->conf[k] / (REAL)(u - l);
        const REAL d = v[k] - s->target[k];
        REAL g;
        if (loss == ORA_L2)
          g = 2 * cn * d;
        else
          g = cn * d / R_SQRT(d * d + (REAL)0.000001);
        if (stereo) g += photometric(s, x, y, v[k], alpha, (REAL)photo_lambda);
        const REAL stepv = -(lam * (v[k] - B) + (REAL)0.5 * g);
        vx[k] = v[k] + st * stepv;
      }
    }
    memcpy(v, vx, n * sizeof(REAL));
    free(vx);
    if (do_over)
      for (size_t k = 0; k < n; ++k)
        if (s->conf[k] > (REAL)overwrite) v[k] = s->target[k];
    ora_col_prefix(v, S, W, H);
    REAL* vy = ora_alloc_real(n);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const size_t k = (size_t)y * W + x;
        const REAL B = ora_window_mean(S + x, (size_t)W, ly[k], uy[k]);
        vy[k] = v[k] + st * (-(lam * (v[k] - B)));
      }
    memcpy(v, vy, n * sizeof(REAL));
    free(vy);
  }
  memcpy(s->var, v, n * sizeof(REAL));
  free(lx);
  free(ux);
  free(ly);
  free(uy);
  free(v);
  free(S);
}

/* Adjoint of Optimize (no reference counterpart: the reference has no
 * gradients).  With the windows fixed, one iteration is
 *   X: v1 = v - s*(lambda*(v - Bx v) + 0.5*g(v)),  0.5*g = (c/n)(v-t)  (L2)
 *                                            or 0.5*(c/n)(v-t)/sqrt((v-t)^2+e)
 *   Y: v2 = v1 - s*lambda*(v1 - By v1)
 * where B averages over the pixel's window.  Given dL/dv_N (gout), this
 * accumulates dL/dt and dL/dc over all iterations (v_0 = t).  The forward
 * iterates are recomputed and kept (test-size images only). */
static void box_transpose(const ora_dts* s, int axis, const REAL* gin,
                          const int32_t* l, const int32_t* u, REAL* gout) {
  /* gout(q) = sum over p with q in (l_p, u_p] of gin(p) / (u_p - l_p) */
  const int W = s->w, H = s->h;
  const size_t n = (size_t)W * H;
  for (size_t k = 0; k < n; ++k) gout[k] = 0;
  /* windows stay inside their row (axis 0) or column (axis 1): one thread
   * per row / column, each scattering in a fixed order */
  const int lines = axis == 0 ? H : W, len = axis == 0 ? W : H;
#pragma omp parallel for schedule(static)
  for (int li = 0; li < lines; ++li)
    for (int j = 0; j < len; ++j) {
      const size_t p = axis == 0 ? (size_t)li * W + j : (size_t)j * W + li;
      const REAL a = gin[p] / (REAL)(u[p] - l[p]);
      for (int q = l[p] + 1; q <= u[p]; ++q) {
        const size_t k = axis == 0 ? (size_t)li * W + q : (size_t)q * W + li;
        gout[k] += a;
      }
    }
}

EXPORT int ora_dts_backward(ora_dts* s, int num_iterations, int loss,
                            float lambda, float sigma_z, float step,
                            const REAL* grad_out, REAL* grad_t, REAL* grad_c) {
  if (loss != ORA_L2 && loss != ORA_CHARBONNIER) return -1;
  const int W = s->w, H = s->h;
  const size_t n = (size_t)W * H;
  int32_t *lx, *ux, *ly, *uy;
  ora_pass_bounds(s, 0, sigma_z, &lx, &ux);
  ora_pass_bounds(s, 1, sigma_z, &ly, &uy);
  const REAL lam = lambda, st = step, eps = (REAL)0.000001;
  /* forward, keeping the X-step input of every iteration */
  REAL* vs = ora_alloc_real(n * (size_t)(num_iterations + 1));
  REAL* S = ora_alloc_real(n);
  REAL* tmp = ora_alloc_real(n);
  memcpy(vs, s->target, n * sizeof(REAL));
  for (int it = 0; it < num_iterations; ++it) {
    const REAL* v = vs + n * it;
    REAL* vn = vs + n * (it + 1);
    ora_row_prefix(v, S, W, H);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const size_t k = (size_t)y * W + x;
        const REAL B = ora_window_mean(S + (size_t)y * W, 1, lx[k], ux[k]);
        const REAL cn = s->conf[k] / (REAL)(ux[k] - lx[k]);
        const REAL d = v[k] - s->target[k];
        const REAL hg = loss == ORA_L2 ? cn * d : (REAL)0.5 * cn * d / R_SQRT(d * d + eps);
        tmp[k] = v[k] - st * (lam * (v[k] - B) + hg);
      }
    ora_col_prefix(tmp, S, W, H);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const size_t k = (size_t)y * W + x;
        const REAL B = ora_window_mean(S + x, (size_t)W, ly[k], uy[k]);
        vn[k] = tmp[k] - st * lam * (tmp[k] - B);
      }
  }
  REAL* g = ora_alloc_real(n);
  REAL* g1 = ora_alloc_real(n);
  memcpy(g, grad_out, n * sizeof(REAL));
  for (size_t k = 0; k < n; ++k) grad_t[k] = grad_c[k] = 0;
  for (int it = num_iterations - 1; it >= 0; --it) {
    const REAL* v = vs + n * it;
    /* Y^T */
    box_transpose(s, 1, g, ly, uy, tmp);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) g1[k] = (1 - st * lam) * g[k] + st * lam * tmp[k];
    /* X^T */
    box_transpose(s, 0, g1, lx, ux, tmp);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) {
      const REAL nk = (REAL)(ux[k] - lx[k]);
      const REAL d = v[k] - s->target[k];
      REAL dh_dv, dh_dc;  /* derivatives of 0.5*g */
      if (loss == ORA_L2) {
        dh_dv = s->conf[k] / nk;
        dh_dc = d / nk;
      } else {
        const REAL r = R_SQRT(d * d + eps);
        dh_dv = (REAL)0.5 * (s->conf[k] / nk) * eps / (r * r * r);
        dh_dc = (REAL)0.5 * d / (nk * r);
      }
      grad_t[k] += st * dh_dv * g1[k];
      grad_c[k] += -st * dh_dc * g1[k];
      g[k] = (1 - st * lam - st * dh_dv) * g1[k] + st * lam * tmp[k];
    }
  }
  for (size_t k = 0; k < n; ++k) grad_t[k] += g[k];
  free(vs);
  free(S);
  free(tmp);
  free(g);
  free(g1);
  free(lx);
  free(ux);
  free(ly);
  free(uy);
  return 0;
}

/* Download -- src/domain_transform_filter.cu:51-74 and
 * src/domain_transform_solver.cu:63-87. */
EXPORT void ora_dts_download(const ora_dts* s, int type, void* dst) {
  const size_t n = (size_t)s->w * s->h;
  switch (type) {
    case ORA_COLOR_IMAGE:
      memcpy(dst, s->color, n * 4);
      break;
    case ORA_DIFFERENTIAL:
      memcpy(dst, s->dH, n * sizeof(REAL));
      break;
    case ORA_INTEGRAL:
      memcpy(dst, s->ctH, n * sizeof(REAL));
      break;
    case ORA_TARGET:
      memcpy(dst, s->target, n * sizeof(REAL));
      break;
    case ORA_CONFIDENCE:
      memcpy(dst, s->conf, n * sizeof(REAL));
      break;
    case ORA_OPTIMIZED_QUANTITY:
      memcpy(dst, s->var, n * sizeof(REAL));
      break;
    default:
      break;
  }
}

/* ======================================================================
 * HFBS -- src/hfbs.h:18-150, src/hfbs.cu:17-759.
 * Grids are dense gx*gy*gl (x fastest).  Reads outside the interior follow
 * the reference's buffers:
 *  - index -1 on any axis: surface read with zero boundary mode -> 0;
 *  - index g on an axis (the pad plane): FillGrid (hfbs.cu:33-61) writes
 *    pad planes only where its 8^3-block launch reaches them, i.e. when
 *    g % 8 != 0 and the plane lies inside the max-size allocation; such a
 *    "covered" face holds the last fill value of that buffer.  In the
 *    bistochastization ping-pong (hfbs.cu:644-662) the source is `scratch`
 *    (filled with 1) on even iterations and `splat_norm` (filled with 0) on
 *    odd ones, so covered faces read 1 on even iterations, 0 otherwise.
 *    Every other pad read in the solve and slice is 0;
 *  - bins with luma bin == gl (sigma_l dividing 255) land in the z = gl pad
 *    plane of the splat buffers (if inside the allocation) and are read back
 *    only by the slice.
 * ====================================================================== */
struct ora_hfbs {
  int max_w, max_h, max_gx, max_gy, max_gl, w, h;
  int contract;
  ora_hfbs_params p;
  uint8_t* color;
  REAL *target, *conf, *optim;
  int gx, gy, gl;
  REAL* grids[ORA_G_COUNT];
  REAL* overflow_count; /* gx*gy, the z = gl plane of splat_sum */
};

EXPORT ora_hfbs* ora_hfbs_create(int max_w, int max_h, int max_gx, int max_gy,
                                 int max_gl) {
  ora_hfbs* s = (ora_hfbs*)calloc(1, sizeof(ora_hfbs));
  const size_t n = (size_t)max_w * max_h;
  s->max_w = s->w = max_w;
  s->max_h = s->h = max_h;
  s->max_gx = max_gx;
  s->max_gy = max_gy;
  s->max_gl = max_gl;
  s->contract = ORA_CONTRACT_NVCC;
  /* HFBSGridParams defaults, src/hfbs.h:18-60. */
  s->p.sigma_x = 8.0f;
  s->p.sigma_y = 8.0f;
  s->p.sigma_l = 4.0f;
  s->p.lambda = 8.0f;
  s->p.alpha = 1.0f;
  s->p.beta = 0.9f;
  s->p.bistoch_iter_max = 20;
  s->p.optim_iter_max = 140;
  s->p.neg_exp_beta = 0.9f;
  s->p.grid_x = s->p.grid_y = s->p.grid_l = 1;
  s->color = (uint8_t*)calloc(n * 4, 1);
  s->target = ora_alloc_real(n);
  s->conf = ora_alloc_real(n);
  s->optim = ora_alloc_real(n);
  return s;
}

static void ora_hfbs_free_grids(ora_hfbs* s) {
  for (int i = 0; i < ORA_G_COUNT; ++i) {
    free(s->grids[i]);
    s->grids[i] = NULL;
  }
  free(s->overflow_count);
  s->overflow_count = NULL;
}

EXPORT void ora_hfbs_destroy(ora_hfbs* s) {
  if (!s) return;
  ora_hfbs_free_grids(s);
  free(s->color);
  free(s->target);
  free(s->conf);
  free(s->optim);
  free(s);
}

EXPORT void ora_hfbs_set_compat(ora_hfbs* s, int contract) {
  s->contract = contract;
}

/* HFBS::SetImageDim -- src/hfbs.cu:527-538. */
EXPORT int ora_hfbs_set_image_dim(ora_hfbs* s, int w, int h) {
  if (h > s->max_h || w > s->max_w) return -1;
  s->w = w;
  s->h = h;
  return 0;
}

EXPORT void ora_hfbs_set_params(ora_hfbs* s, const ora_hfbs_params* p) {
  s->p = *p;
}

/* HFBS::ClearAll -- src/hfbs.cu:745-759. */
EXPORT void ora_hfbs_clear_all(ora_hfbs* s) {
  const size_t n = (size_t)s->max_w * s->max_h;
  memset(s->color, 0, n * 4);
  memset(s->target, 0, n * sizeof(REAL));
  memset(s->conf, 0, n * sizeof(REAL));
  memset(s->optim, 0, n * sizeof(REAL));
}

/* HFBS::InitFrame -- src/hfbs.cu:498-525, 540-553. */
EXPORT void ora_hfbs_init_frame(ora_hfbs* s, int color_space,
                                const uint8_t* rgba, const float* target,
                                const float* confidence) {
  const int64_t n = (int64_t)s->w * s->h;
  ora_color_convert(color_space, s->contract, rgba, s->color, n);
  if (target)
    for (int64_t i = 0; i < n; ++i) s->target[i] = (REAL)target[i];
  if (confidence) {
    for (int64_t i = 0; i < n; ++i) s->conf[i] = (REAL)confidence[i];
  } else {
    const size_t nmax = (size_t)s->max_w * s->max_h;
    for (size_t i = 0; i < nmax; ++i) s->conf[i] = 1;
  }
}

/* target / confidence at REAL precision (finite-difference checks); NULL
 * keeps a plane. */
EXPORT void ora_hfbs_set_target_conf(ora_hfbs* s, const REAL* target,
                                     const REAL* confidence) {
  const size_t n = (size_t)s->w * s->h;
  if (target) memcpy(s->target, target, n * sizeof(REAL));
  if (confidence) memcpy(s->conf, confidence, n * sizeof(REAL));
}

#define GI(x, y, z) (((size_t)(z) * gy + (y)) * gx + (x))

/* Laplace sweeps -- src/hfbs.cu:355-427: along one axis,
 *   forward  r = s(0); d(0) = r; r = s(i) + beta*r; d(i) = r
 *   backward r = s(g-1); r = beta*r; d(i) += r; r += s(i)  (i = g-2 .. 0)
 * i.e. d(i) = sum_j beta^|i-j| s(j). */
static void ora_laplace(const REAL* src, REAL* dst, int gx, int gy, int gl,
                        int axis, REAL beta) {
  const int len = axis == 0 ? gx : (axis == 1 ? gy : gl);
  const size_t stride = axis == 0 ? 1 : (axis == 1 ? (size_t)gx : (size_t)gx * gy);
  const int na = axis == 0 ? gy : gx, nb = axis == 2 ? gy : gl;
#pragma omp parallel for schedule(static)
  for (int bidx = 0; bidx < nb; ++bidx)
    for (int aidx = 0; aidx < na; ++aidx) {
      size_t base;
      if (axis == 0) base = GI(0, aidx, bidx);
      else if (axis == 1) base = GI(aidx, 0, bidx);
      else base = GI(aidx, bidx, 0);
      REAL r = src[base];
      dst[base] = r;
      for (int i = 1; i < len; ++i) {
        r = R_FMA(beta, r, src[base + i * stride]);
        dst[base + i * stride] = r;
      }
      r = src[base + (size_t)(len - 1) * stride];
      for (int i = len - 2; i >= 0; --i) {
        r = beta * r;
        dst[base + i * stride] = dst[base + i * stride] + r;
        r = r + src[base + i * stride];
      }
    }
}

/* One SolveHFBS heavy-ball step, src/hfbs.cu:201-239: zd = zs - alpha*h'
 * with h' = beta*h + Huber(zs - q), q = (b + lambda*norm*N(norm*zs))*invA and
 * N the six-neighbour sum.  Neighbours outside the interior read 0. */
static void ora_hfbs_step(const REAL* zs, REAL* zd, REAL* h, const REAL* norm,
                          const REAL* b, const REAL* invA, int gx, int gy, int gl,
                          const ora_hfbs_params* p) {
  const REAL lam = p->lambda, beta = p->beta, alpha = p->alpha;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < gl; ++z)
    for (int y = 0; y < gy; ++y)
      for (int x = 0; x < gx; ++x) {
        REAL d = 0;
        if (x > 0) d += zs[GI(x - 1, y, z)] * norm[GI(x - 1, y, z)];
        if (x + 1 < gx) d += zs[GI(x + 1, y, z)] * norm[GI(x + 1, y, z)];
        if (y > 0) d += zs[GI(x, y - 1, z)] * norm[GI(x, y - 1, z)];
        if (y + 1 < gy) d += zs[GI(x, y + 1, z)] * norm[GI(x, y + 1, z)];
        if (z > 0) d += zs[GI(x, y, z - 1)] * norm[GI(x, y, z - 1)];
        if (z + 1 < gl) d += zs[GI(x, y, z + 1)] * norm[GI(x, y, z + 1)];
        const size_t g = GI(x, y, z);
        const REAL q = (b[g] + lam * norm[g] * d) * invA[g];
        const REAL zc = zs[g];
        const REAL grad = zc - q;
        const REAL gc = fabs((double)grad) > 1.345 ? (grad > 0 ? (REAL)1 : (REAL)-1)
                                                   : grad;
        const REAL hn = beta * h[g] + gc;
        h[g] = hn;
        zd[g] = zc - alpha * hn;
      }
}

/* HFBS::Optimize -- src/hfbs.cu:586-743. */
EXPORT int ora_hfbs_optimize(ora_hfbs* s) {
  const int W = s->w, H = s->h;
  ora_hfbs_params* p = &s->p;
  /* grid sizes, hfbs.cu:589-591 (float division for x/y, double for l) */
  p->grid_x = (int)ceilf((float)W / p->sigma_x);
  p->grid_y = (int)ceilf((float)H / p->sigma_y);
  p->grid_l = (int)ceil(255.0 / (double)p->sigma_l);
  const int gx = p->grid_x, gy = p->grid_y, gl = p->grid_l;
  s->gx = gx;
  s->gy = gy;
  s->gl = gl;
  ora_hfbs_free_grids(s);
  if (gx > s->max_gx || gy > s->max_gy || gl > s->max_gl) {
    /* hfbs.cu:594-611: report and copy target to the output. */
    memcpy(s->optim, s->target, (size_t)W * H * sizeof(REAL));
    return 1;
  }
  const size_t ng = (size_t)gx * gy * gl;
  for (int i = 0; i < ORA_G_COUNT; ++i) s->grids[i] = ora_alloc_real(ng);
  s->overflow_count = ora_alloc_real((size_t)gx * gy);
  REAL* count = s->grids[ORA_G_SPLAT_SUM];
  REAL* csum = s->grids[ORA_G_SPLAT_C];
  REAL* b = s->grids[ORA_G_B];
  REAL* norm = s->grids[ORA_G_SPLAT_NORM];
  REAL* invA = s->grids[ORA_G_INV_DIAG_A];
  REAL* blur_c = s->grids[ORA_G_BLUR_C];
  REAL* zinit = s->grids[ORA_G_Z_INIT];
  REAL* zfin = s->grids[ORA_G_Z_FINAL];
  const int ovf_stored = gl < s->max_gl;

  /* a12. SplatBAndC + BistochastasizeSetup, hfbs.cu:72-120 (nearest bin;
   * bin of luma from the .x channel). */
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t k = (size_t)y * W + x;
      const int bx = (int)floorf((float)x * 1.0f / p->sigma_x);
      const int by = (int)floorf((float)y * 1.0f / p->sigma_y);
      const int bl = (int)floorf((float)s->color[4 * k] * 1.0f / p->sigma_l);
      const REAL c = s->conf[k];
      const REAL ct = c * s->target[k];
      if (bl < gl) {
        const size_t g = GI(bx, by, bl);
        b[g] += ct;
        csum[g] += c;
        count[g] += 1;
      } else if (ovf_stored) {
        s->overflow_count[(size_t)by * gx + bx] += 1;
      }
    }

  /* a13. bistochastization, hfbs.cu:126-155 and :644-666. */
  const int cov_x = (gx % 8 != 0) && (gx < s->max_gx);
  const int cov_y = (gy % 8 != 0) && (gy < s->max_gy);
  const int cov_l = (gl % 8 != 0) && (gl < s->max_gl);
  REAL* src = ora_alloc_real(ng);
  REAL* dst = ora_alloc_real(ng);
  for (size_t i = 0; i < ng; ++i) src[i] = 1;
  for (int it = 0; it < p->bistoch_iter_max; ++it) {
    const REAL pad = (it % 2 == 0) ? (REAL)1 : (REAL)0;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < gl; ++z)
      for (int y = 0; y < gy; ++y)
        for (int x = 0; x < gx; ++x) {
          REAL nb = 0;
          nb += x > 0 ? src[GI(x - 1, y, z)] : (REAL)0;
          nb += x + 1 < gx ? src[GI(x + 1, y, z)] : (cov_x ? pad : (REAL)0);
          nb += y > 0 ? src[GI(x, y - 1, z)] : (REAL)0;
          nb += y + 1 < gy ? src[GI(x, y + 1, z)] : (cov_y ? pad : (REAL)0);
          nb += z > 0 ? src[GI(x, y, z - 1)] : (REAL)0;
          nb += z + 1 < gl ? src[GI(x, y, z + 1)] : (cov_l ? pad : (REAL)0);
          const REAL v = src[GI(x, y, z)];
          const REAL blurred = 2 * v + nb;
          dst[GI(x, y, z)] =
              R_SQRT(v * (count[GI(x, y, z)] + (REAL)0.00001f) /
                     (blurred + (REAL)0.00001f));
        }
    REAL* t = src;
    src = dst;
    dst = t;
  }
  memcpy(norm, src, ng * sizeof(REAL));

  /* a14. CalcInvDiagA, hfbs.cu:159-195 (the splat of c was saved in
   * inv_diag_A by BistochastasizeSetup). */
  for (size_t i = 0; i < ng; ++i) {
    const REAL diag = (REAL)p->lambda * (count[i] - 2 * norm[i] * norm[i]) + csum[i];
    const REAL m = diag > (REAL)1e-3 ? diag : (REAL)1e-3;
    invA[i] = (REAL)1 / m;
  }

  /* a15. Laplace blur of c (-> blur_c) and of b (-> z), InitZ<true>,
   * hfbs.cu:676-719. */
  const REAL nb_beta = p->neg_exp_beta;
  ora_laplace(csum, dst, gx, gy, gl, 0, nb_beta);
  ora_laplace(dst, src, gx, gy, gl, 1, nb_beta);
  ora_laplace(src, blur_c, gx, gy, gl, 2, nb_beta);
  ora_laplace(b, dst, gx, gy, gl, 0, nb_beta);
  ora_laplace(dst, src, gx, gy, gl, 1, nb_beta);
  ora_laplace(src, zinit, gx, gy, gl, 2, nb_beta);
  for (size_t i = 0; i < ng; ++i) zinit[i] = zinit[i] / (blur_c[i] + (REAL)1e-7);

  /* a16. SolveHFBS heavy-ball iterations, hfbs.cu:201-239 and :720-732. */
  REAL* h = ora_alloc_real(ng);
  REAL* zs = src;
  REAL* zd = dst;
  memcpy(zs, zinit, ng * sizeof(REAL));
  for (int it = 0; it < p->optim_iter_max; ++it) {
    ora_hfbs_step(zs, zd, h, norm, b, invA, gx, gy, gl, p);
    REAL* t = zs;
    zs = zd;
    zd = t;
  }
  memcpy(zfin, zs, ng * sizeof(REAL));
  free(h);
  free(src);
  free(dst);

  /* a17. SliceSolution<true>, hfbs.cu:246-330: count-weighted trilinear
   * interpolation; positions and weights in float as in the reference. */
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t k = (size_t)y * W + x;
      const float fxp = (float)x * 1.0f / p->sigma_x;
      const float fyp = (float)y * 1.0f / p->sigma_y;
      const float fzp = (float)s->color[4 * k] * 1.0f / p->sigma_l;
      const float x0 = floorf(fxp), y0 = floorf(fyp), z0 = floorf(fzp);
      const REAL wx = (REAL)(fxp - x0), wy = (REAL)(fyp - y0), wz = (REAL)(fzp - z0);
      REAL num[2][2], den[2][2];
      for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy) {
          REAL nsum = 0, dsum = 0;
          for (int dx = 0; dx < 2; ++dx) {
            const int ix = (int)x0 + dx, iy = (int)y0 + dy, iz = (int)z0 + dz;
            REAL cnt = 0, zv = 0;
            if (ix < gx && iy < gy && iz < gl) {
              cnt = count[GI(ix, iy, iz)];
              zv = zfin[GI(ix, iy, iz)];
            } else if (ix < gx && iy < gy && iz == gl && ovf_stored) {
              cnt = s->overflow_count[(size_t)iy * gx + ix];
            }
            const REAL wxx = dx ? wx : (REAL)1 - wx;
            nsum += cnt * zv * wxx;
            dsum += cnt * wxx;
          }
          num[dz][dy] = nsum;
          den[dz][dy] = dsum;
        }
      const REAL c0 = num[0][0] * ((REAL)1 - wy) + num[0][1] * wy;
      const REAL c1 = num[1][0] * ((REAL)1 - wy) + num[1][1] * wy;
      const REAL c0m = den[0][0] * ((REAL)1 - wy) + den[0][1] * wy;
      const REAL c1m = den[1][0] * ((REAL)1 - wy) + den[1][1] * wy;
      s->optim[k] = (c0 * ((REAL)1 - wz) + c1 * wz) / (c0m * ((REAL)1 - wz) + c1m * wz);
    }
  return 0;
}

/* Three-axis Laplace blur (X -> Y -> Z) of src into dst; t0, t1 scratch. */
static void ora_laplace3(const REAL* src, REAL* dst, REAL* t0, REAL* t1, int gx,
                         int gy, int gl, REAL beta) {
  ora_laplace(src, t0, gx, gy, gl, 0, beta);
  ora_laplace(t0, t1, gx, gy, gl, 1, beta);
  ora_laplace(t1, dst, gx, gy, gl, 2, beta);
}

/* Adjoint of HFBS::Optimize (src/hfbs.cu:586-743) with respect to the
 * target and the confidence, for an upstream gradient grad_out = dL/d(output)
 * (W*H).  Bins, splat counts and the bistochastized normalisation do not
 * depend on target or confidence; the Huber clamp of the heavy-ball step
 * enters by its mask (|grad| <= 1.345), the invA floor (diag <= 1e-3) by a
 * zero derivative.  Steps, last to first:
 *  slice^T:  gz += gout * w * count / den at each in-grid corner (den = 0:
 *            the pixel contributes nothing);
 *  step^T:   u = gh - alpha*gz;  gg = mask*u;  gh = beta*u;
 *            gb -= invA*gg;  ginvA -= (b + lambda*norm*d)*gg;
 *            gz += gg - lambda*norm*N(norm*invA*gg)   (N symmetric);
 *  InitZ^T:  z0 = blur_b / (blur_c + 1e-7);
 *  blur^T:   the three-axis Laplace blur is symmetric;
 *  invA^T:   dinvA/dcsum = -invA^2 where diag > 1e-3;
 *  splat^T:  b = S(c*t), csum = S(c): gt = c*gb[bin], gc = t*gb[bin] + gcsum[bin]
 *            (pixels in the overflow bin get 0).
 * Needs the grids of a completed ora_hfbs_optimize of the same frame; the
 * forward iterates are recomputed and all kept. */
EXPORT int ora_hfbs_backward(ora_hfbs* s, const REAL* grad_out, REAL* grad_t,
                             REAL* grad_c) {
  if (!s->grids[ORA_G_B]) return -1;
  const int W = s->w, H = s->h, gx = s->gx, gy = s->gy, gl = s->gl;
  const ora_hfbs_params* p = &s->p;
  const size_t ng = (size_t)gx * gy * gl;
  const int K = p->optim_iter_max;
  const REAL* count = s->grids[ORA_G_SPLAT_SUM];
  const REAL* csum = s->grids[ORA_G_SPLAT_C];
  const REAL* b = s->grids[ORA_G_B];
  const REAL* norm = s->grids[ORA_G_SPLAT_NORM];
  const REAL* invA = s->grids[ORA_G_INV_DIAG_A];
  const REAL* blur_c = s->grids[ORA_G_BLUR_C];
  const REAL* zinit = s->grids[ORA_G_Z_INIT];
  const int ovf_stored = gl < s->max_gl;
  const REAL lam = p->lambda, alpha = p->alpha, beta = p->beta;
  /* forward iterates z_0 .. z_{K-1} */
  REAL* zh = ora_alloc_real(ng * (size_t)(K > 0 ? K : 1));
  REAL* hv = ora_alloc_real(ng);
  REAL* ztmp = ora_alloc_real(ng);
  memcpy(zh, zinit, ng * sizeof(REAL));
  for (int it = 0; it + 1 < K; ++it)
    ora_hfbs_step(zh + ng * it, zh + ng * (it + 1), hv, norm, b, invA, gx, gy, gl, p);
  REAL* gz = ora_alloc_real(ng);
  REAL* gh = ora_alloc_real(ng);
  REAL* gb = ora_alloc_real(ng);
  REAL* ginv = ora_alloc_real(ng);
  REAL* gg = ora_alloc_real(ng);
  REAL* wv = ora_alloc_real(ng);
  /* slice^T (same positions and weights as the forward slice) */
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t k = (size_t)y * W + x;
      const float fxp = (float)x * 1.0f / p->sigma_x;
      const float fyp = (float)y * 1.0f / p->sigma_y;
      const float fzp = (float)s->color[4 * k] * 1.0f / p->sigma_l;
      const float x0 = floorf(fxp), y0 = floorf(fyp), z0 = floorf(fzp);
      const REAL wx = (REAL)(fxp - x0), wy = (REAL)(fyp - y0), wz = (REAL)(fzp - z0);
      REAL wgt[8], cnt[8];
      size_t gidx[8];
      int in[8];
      REAL den = 0;
      for (int c = 0; c < 8; ++c) {
        const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
        const int ix = (int)x0 + dx, iy = (int)y0 + dy, iz = (int)z0 + dz;
        wgt[c] = (dx ? wx : 1 - wx) * (dy ? wy : 1 - wy) * (dz ? wz : 1 - wz);
        cnt[c] = 0;
        in[c] = 0;
        gidx[c] = 0;
        if (ix < gx && iy < gy && iz < gl) {
          gidx[c] = GI(ix, iy, iz);
          cnt[c] = count[gidx[c]];
          in[c] = 1;
        } else if (ix < gx && iy < gy && iz == gl && ovf_stored) {
          cnt[c] = s->overflow_count[(size_t)iy * gx + ix];
        }
        den += wgt[c] * cnt[c];
      }
      if (den == 0) continue;
      for (int c = 0; c < 8; ++c)
        if (in[c]) gz[gidx[c]] += grad_out[k] * wgt[c] * cnt[c] / den;
    }
  /* heavy-ball steps, last to first */
  for (int it = K - 1; it >= 0; --it) {
    const REAL* z = zh + ng * it;
#pragma omp parallel for schedule(static)
    for (int zz = 0; zz < gl; ++zz)
      for (int y = 0; y < gy; ++y)
        for (int x = 0; x < gx; ++x) {
          REAL d = 0;
          if (x > 0) d += z[GI(x - 1, y, zz)] * norm[GI(x - 1, y, zz)];
          if (x + 1 < gx) d += z[GI(x + 1, y, zz)] * norm[GI(x + 1, y, zz)];
          if (y > 0) d += z[GI(x, y - 1, zz)] * norm[GI(x, y - 1, zz)];
          if (y + 1 < gy) d += z[GI(x, y + 1, zz)] * norm[GI(x, y + 1, zz)];
          if (zz > 0) d += z[GI(x, y, zz - 1)] * norm[GI(x, y, zz - 1)];
          if (zz + 1 < gl) d += z[GI(x, y, zz + 1)] * norm[GI(x, y, zz + 1)];
          const size_t g = GI(x, y, zz);
          const REAL bq = b[g] + lam * norm[g] * d;
          const REAL grad = z[g] - bq * invA[g];
          const REAL u = gh[g] - alpha * gz[g];
          const REAL v = fabs((double)grad) > 1.345 ? (REAL)0 : u;
          gh[g] = beta * u;
          gb[g] -= invA[g] * v;
          ginv[g] -= bq * v;
          gg[g] = v;
          wv[g] = norm[g] * invA[g] * v;
        }
#pragma omp parallel for schedule(static)
    for (int zz = 0; zz < gl; ++zz)
      for (int y = 0; y < gy; ++y)
        for (int x = 0; x < gx; ++x) {
          REAL a = 0;
          if (x > 0) a += wv[GI(x - 1, y, zz)];
          if (x + 1 < gx) a += wv[GI(x + 1, y, zz)];
          if (y > 0) a += wv[GI(x, y - 1, zz)];
          if (y + 1 < gy) a += wv[GI(x, y + 1, zz)];
          if (zz > 0) a += wv[GI(x, y, zz - 1)];
          if (zz + 1 < gl) a += wv[GI(x, y, zz + 1)];
          const size_t g = GI(x, y, zz);
          gz[g] += gg[g] - lam * norm[g] * a;
        }
  }
  /* InitZ^T: gg = d/d blur_b, wv = d/d blur_c */
  for (size_t i = 0; i < ng; ++i) {
    const REAL e = blur_c[i] + (REAL)1e-7;
    gg[i] = gz[i] / e;
    wv[i] = -gz[i] * zinit[i] / e;
  }
  /* blur^T (symmetric): gb += blur(gg); gcsum = blur(wv) (into gh) */
  ora_laplace3(gg, ztmp, gz, hv, gx, gy, gl, p->neg_exp_beta);
  for (size_t i = 0; i < ng; ++i) gb[i] += ztmp[i];
  ora_laplace3(wv, gh, gz, hv, gx, gy, gl, p->neg_exp_beta);
  /* invA^T */
  for (size_t i = 0; i < ng; ++i) {
    const REAL diag = lam * (count[i] - 2 * norm[i] * norm[i]) + csum[i];
    if (diag > (REAL)1e-3) gh[i] -= ginv[i] * invA[i] * invA[i];
  }
  /* splat^T */
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t k = (size_t)y * W + x;
      const int bx = (int)floorf((float)x * 1.0f / p->sigma_x);
      const int by = (int)floorf((float)y * 1.0f / p->sigma_y);
      const int bl = (int)floorf((float)s->color[4 * k] * 1.0f / p->sigma_l);
      if (bl < gl) {
        const size_t g = GI(bx, by, bl);
        if (grad_t) grad_t[k] = s->conf[k] * gb[g];
        if (grad_c) grad_c[k] = s->target[k] * gb[g] + gh[g];
      } else {
        if (grad_t) grad_t[k] = 0;
        if (grad_c) grad_c[k] = 0;
      }
    }
  free(zh);
  free(hv);
  free(ztmp);
  free(gz);
  free(gh);
  free(gb);
  free(ginv);
  free(gg);
  free(wv);
  return 0;
}

/* HFBS::Download -- src/hfbs.cu:555-576. */
EXPORT void ora_hfbs_download(const ora_hfbs* s, int type, REAL* dst) {
  const size_t n = (size_t)s->w * s->h;
  switch (type) {
    case ORA_TARGET:
      memcpy(dst, s->target, n * sizeof(REAL));
      break;
    case ORA_CONFIDENCE:
      memcpy(dst, s->conf, n * sizeof(REAL));
      break;
    case ORA_OPTIMIZED_QUANTITY:
      memcpy(dst, s->optim, n * sizeof(REAL));
      break;
    default:
      break;
  }
}

EXPORT void ora_hfbs_grid_dims(const ora_hfbs* s, int* gx, int* gy, int* gl) {
  *gx = s->gx;
  *gy = s->gy;
  *gl = s->gl;
}

EXPORT void ora_hfbs_grid(const ora_hfbs* s, int which, REAL* dst) {
  if (which < 0 || which >= ORA_G_COUNT || !s->grids[which]) return;
  memcpy(dst, s->grids[which], (size_t)s->gx * s->gy * s->gl * sizeof(REAL));
}

/* ======================================================================
 * Soft-window DTS: the project's relaxation of the reference's integer
 * windows (src/domain_transform_filter.cuh:7-28), for gradients with
 * respect to the edge weights dH / dV (Compute_dHdx / Compute_dVdy,
 * src/domain_transform_common_kernels.cuh:81-116).  Along a line the
 * transformed distance D_pq is the sum of the edge weights over
 * (min(p,q), max(p,q)] and q weighs w_pq = ramp((sigma - D_pq) / tau),
 * ramp(x) = clamp(x + 1/2, 0, 1), in p's window (clipped at the line ends,
 * the Y window running to the height).  The iteration is
 * src/domain_transform_solver.cuh:12-116 with B = sum w v / n, n = sum w.
 * The adjoint here scatters each window pair's derivative onto the edge
 * weights between the pair, pair by pair.
 * ====================================================================== */
static REAL soft_ramp(REAL x) {
  const REAL r = x + (REAL)0.5;
  return r < 0 ? 0 : (r > 1 ? 1 : r);
}

typedef struct {
  int i, L;
  size_t st, base;
} soft_line;

static soft_line soft_line_of(int W, int H, int axis, size_t k) {
  const int y = (int)(k / (size_t)W), x = (int)(k - (size_t)y * W);
  soft_line l;
  if (axis == 0) {
    l.i = x; l.L = W; l.st = 1; l.base = (size_t)y * W;
  } else {
    l.i = y; l.L = H; l.st = (size_t)W; l.base = (size_t)x;
  }
  return l;
}

/* n and sum w*val over pixel k's soft window */
static void soft_window_sum(const soft_line* l, const REAL* e, const REAL* val, REAL sigma,
                            REAL tau, REAL* n_out, REAL* s_out) {
  const REAL wc = soft_ramp(sigma / tau), stop = sigma + tau / 2;
  REAL n = wc, S = wc * val[l->base + l->i * l->st], D = 0;
  for (int q = l->i + 1; q < l->L; ++q) {
    D += e[l->base + q * l->st];
    if (!(D < stop)) break;
    const REAL w = soft_ramp((sigma - D) / tau);
    n += w;
    S += w * val[l->base + q * l->st];
  }
  D = 0;
  for (int q = l->i - 1; q >= 0; --q) {
    D += e[l->base + (q + 1) * l->st];
    if (!(D < stop)) break;
    const REAL w = soft_ramp((sigma - D) / tau);
    n += w;
    S += w * val[l->base + q * l->st];
  }
  *n_out = n;
  *s_out = S;
}

static void soft_data(int loss, REAL v, REAL t, REAL c, REAL n, REAL* h, REAL* hd, REAL* hc) {
  const REAL d = v - t, eps = (REAL)0.000001;
  if (loss == ORA_L2) {
    *h = c / n * d;
    *hd = c / n;
    *hc = d / n;
  } else {
    const REAL r = R_SQRT(d * d + eps);
    *h = (REAL)0.5 * (c / n) * d / r;
    *hd = (REAL)0.5 * (c / n) * eps / (r * r * r);
    *hc = (REAL)0.5 * d / (n * r);
  }
}

static void soft_half(int W, int H, int axis, const REAL* e, const REAL* vin, REAL* vout,
                      const REAL* t, const REAL* c, int data, int loss, REAL lam,
                      REAL sigma, REAL step, REAL tau) {
  const size_t N = (size_t)W * H;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < N; ++k) {
    const soft_line l = soft_line_of(W, H, axis, k);
    REAL n, S, h = 0, hd, hc;
    soft_window_sum(&l, e, vin, sigma, tau, &n, &S);
    if (data) soft_data(loss, vin[k], t[k], c ? c[k] : 1, n, &h, &hd, &hc);
    vout[k] = vin[k] - step * (lam * (vin[k] - S / n) + h);
  }
}

/* adjoint of one half-step: a = dL/dvout -> ain = dL/dvin, ge += dL/de,
 * gt / gc += the data term's (X only) */
static void soft_half_adjoint(int W, int H, int axis, const REAL* e, const REAL* vin,
                              const REAL* t, const REAL* c, int data, int loss, REAL lam,
                              REAL sigma, REAL step, REAL tau, const REAL* a, REAL* ain,
                              REAL* ge, REAL* gt, REAL* gc) {
  const size_t N = (size_t)W * H;
  const REAL stop = sigma + tau / 2;
  for (size_t k = 0; k < N; ++k) ain[k] = 0;
  for (size_t k = 0; k < N; ++k) {
    const soft_line l = soft_line_of(W, H, axis, k);
    REAL n, S, h = 0, hd = 0, hc = 0;
    soft_window_sum(&l, e, vin, sigma, tau, &n, &S);
    const REAL B = S / n;
    if (data) {
      soft_data(loss, vin[k], t[k], c ? c[k] : 1, n, &h, &hd, &hc);
      gt[k] += a[k] * step * hd;
      gc[k] -= a[k] * step * hc;
    }
    ain[k] += a[k] * (1 - step * lam - step * hd);
    const REAL coef = a[k] * step / n;
    ain[k] += coef * lam * soft_ramp(sigma / tau);
    for (int dir = -1; dir <= 1; dir += 2) {
      REAL D = 0;
      for (int q = l.i + dir; q >= 0 && q < l.L; q += dir) {
        const int jnew = dir > 0 ? q : q + 1;  /* the edge weight D just took */
        D += e[l.base + jnew * l.st];
        if (!(D < stop)) break;
        const REAL x = (sigma - D) / tau;
        const size_t kq = l.base + q * l.st;
        ain[kq] += coef * lam * soft_ramp(x);
        if (x > (REAL)-0.5 && x < (REAL)0.5) {
          /* dL/dw_pq times dw/dD = -1/tau, onto every edge weight of D */
          const REAL gD = -coef * (lam * (vin[kq] - B) + h) / tau;
          const int lo = dir > 0 ? l.i + 1 : q + 1, hi = dir > 0 ? q : l.i;
          for (int j = lo; j <= hi; ++j) ge[l.base + j * l.st] += gD;
        }
      }
    }
  }
}

EXPORT void ora_soft_solve(int W, int H, const REAL* eh, const REAL* ev, const REAL* t,
                           const REAL* c, int num_iterations, int loss, float lambda,
                           float sigma_z, float step, float tau, REAL* out) {
  const size_t N = (size_t)W * H;
  const int iters = loss == ORA_L1 ? 0 : num_iterations;
  REAL* v = ora_alloc_real(N);
  REAL* u = ora_alloc_real(N);
  memcpy(v, t, N * sizeof(REAL));
  for (int it = 0; it < iters; ++it) {
    soft_half(W, H, 0, eh, v, u, t, c, 1, loss, lambda, sigma_z, step, tau);
    soft_half(W, H, 1, ev, u, v, NULL, NULL, 0, loss, lambda, sigma_z, step, tau);
  }
  memcpy(out, v, N * sizeof(REAL));
  free(v);
  free(u);
}

EXPORT void ora_soft_backward(int W, int H, const REAL* eh, const REAL* ev, const REAL* t,
                              const REAL* c, int num_iterations, int loss, float lambda,
                              float sigma_z, float step, float tau, const REAL* grad_out,
                              REAL* grad_t, REAL* grad_c, REAL* grad_eh, REAL* grad_ev) {
  const size_t N = (size_t)W * H;
  const int iters = loss == ORA_L1 ? 0 : num_iterations;
  REAL* vs = ora_alloc_real(N * (size_t)(iters + 1));
  REAL* u = ora_alloc_real(N);
  REAL* a = ora_alloc_real(N);
  REAL* b = ora_alloc_real(N);
  memcpy(vs, t, N * sizeof(REAL));
  for (int it = 0; it < iters; ++it) {
    soft_half(W, H, 0, eh, vs + N * it, u, t, c, 1, loss, lambda, sigma_z, step, tau);
    soft_half(W, H, 1, ev, u, vs + N * (it + 1), NULL, NULL, 0, loss, lambda, sigma_z, step,
              tau);
  }
  for (size_t k = 0; k < N; ++k) grad_t[k] = grad_c[k] = grad_eh[k] = grad_ev[k] = 0;
  memcpy(a, grad_out, N * sizeof(REAL));
  for (int it = iters - 1; it >= 0; --it) {
    const REAL* v = vs + N * it;
    soft_half(W, H, 0, eh, v, u, t, c, 1, loss, lambda, sigma_z, step, tau);
    soft_half_adjoint(W, H, 1, ev, u, NULL, NULL, 0, loss, lambda, sigma_z, step, tau, a, b,
                      grad_ev, NULL, NULL);
    soft_half_adjoint(W, H, 0, eh, v, t, c, 1, loss, lambda, sigma_z, step, tau, b, a,
                      grad_eh, grad_t, grad_c);
  }
  for (size_t k = 0; k < N; ++k) grad_t[k] += a[k];
  free(vs);
  free(u);
  free(a);
  free(b);
}
