/*
 * CPU oracle for the DTS / HFBS hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A line-by-line restatement, in plain C, of the reference algorithms of
 * akashbapat/domain_transform_solver.  It exists to check the CUDA product
 * path (tests/, __graft_entry__.smoke()) and to time the CPU baseline leg of
 * bench.py.  Nothing in the product library links, loads or calls it.
 *
 * PARITY UNPINNED: the reference ships no golden vectors and cannot be built
 * or run here (empty libcua/CUB submodules, no OpenCV/GTest, CUDA 8/9 era).
 * The restatement is anchored on the reference's source (file:line cited per
 * function) plus known-answer tests in tests/test_oracle.py, and on one
 * GPU-side pin: the colour-conversion expression compiled by nvcc.
 *
 * The same source is compiled twice:
 *   REAL=double  -> liboracle_f64.so   (the FP64 oracle)
 *   REAL=float   -> liboracle_f32.so   (the FP32 CPU baseline, OpenMP)
 * Decisions the reference takes in FP32 on purpose (bin indices, grid sizes,
 * sigma ratios, sigma schedules) stay in float in both builds.
 */
#ifndef DTS_ORACLE_H_
#define DTS_ORACLE_H_

#include <stdint.h>

#ifndef REAL
#define REAL double
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ImageType (src/domain_transform_common.h:20-28). */
enum { ORA_COLOR_IMAGE = 0, ORA_DIFFERENTIAL, ORA_INTEGRAL, ORA_TARGET,
       ORA_CONFIDENCE, ORA_OPTIMIZED_QUANTITY, ORA_TEST };
/* COLOR_SPACE (src/domain_transform_common.h:32). */
enum { ORA_RGB = 0, ORA_YCBCR = 1, ORA_YYY = 2 };
/* RobustLoss (src/domain_transform_optimize.h:8). */
enum { ORA_L1 = 0, ORA_L2 = 1, ORA_CHARBONNIER = 2 };

/* Colour-conversion evaluation orders of the double expressions in
 * src/color_space.cuh:18-21,35.  0 = every operation rounded separately,
 * 1 = mul+add contracted to fma as nvcc does by default (see oracle.c). */
enum { ORA_CONTRACT_NONE = 0, ORA_CONTRACT_NVCC = 1 };

int ora_real_bytes(void);
/* OpenMP worker threads of the loops below (n <= 0: all host threads). */
void ora_set_threads(int n);
int ora_get_threads(void);

/* ---- a1: colour conversion of n RGBA pixels (in may equal out). -------- */
void ora_color_convert(int color_space, int contract, const uint8_t* in,
                       uint8_t* out, int64_t n);

/* ---- DTS: mirror of DomainTransformFilter + DomainTransformSolver. ------ */
typedef struct ora_dts ora_dts;
ora_dts* ora_dts_create(int max_w, int max_h);
void ora_dts_destroy(ora_dts* s);
/* ref_y_limit=1 reproduces the Y-pass search limit quirk (loop bound is the
 * image width in both passes, src/domain_transform_filter.cuh:22).  */
void ora_dts_set_compat(ora_dts* s, int ref_y_limit, int color_contract);
int ora_dts_set_image_dim(ora_dts* s, int w, int h);
void ora_dts_clear_all(ora_dts* s);
void ora_dts_init_frame(ora_dts* s, int color_space, const uint8_t* rgba,
                        const float* target, const float* confidence);
/* target / confidence at REAL precision (NULL keeps a plane) */
void ora_dts_set_target_conf(ora_dts* s, const REAL* target,
                             const REAL* confidence);
void ora_dts_differential(ora_dts* s, float sigma_x, float sigma_y,
                          float sigma_r);
void ora_dts_integrate(ora_dts* s);
void ora_dts_filter(ora_dts* s, float sigma_x, float sigma_y, float sigma_r,
                    const float* in, REAL* out, int num_iter);
void ora_dts_compute_confidence(ora_dts* s, float sigma_x, float sigma_y,
                                float sigma_r, float sigma0, int left_clear);
void ora_dts_optimize(ora_dts* s, int num_iterations, int loss, float lambda,
                      float sigma_z, float step_size, float overwrite);
/* DomainTransformStereo (src/domain_transform_stereo.h:93-114). */
void ora_dts_init_right_frame(ora_dts* s, float center_offset, int color_space,
                              const uint8_t* rgba);
void ora_dts_process_right_frame(ora_dts* s);
void ora_dts_optimize_stereo(ora_dts* s, int num_iterations, int loss,
                             float lambda, float sigma_z, float step_size,
                             float photo_lambda, float overwrite);
/* Adjoint of Optimize with the windows fixed: dL/dt and dL/dc for an
 * upstream gradient dL/dv of the result (L2 or Charbonnier; returns -1 for
 * other losses). */
int ora_dts_backward(ora_dts* s, int num_iterations, int loss, float lambda,
                     float sigma_z, float step_size, const REAL* grad_out,
                     REAL* grad_t, REAL* grad_c);
/* Download: COLOR_IMAGE -> uint8 RGBA, everything else -> REAL. */
void ora_dts_download(const ora_dts* s, int image_type, void* dst);
/* Window bounds of the current domain transform for one sigma.
 * axis 0 = X pass (ct_H), 1 = Y pass (ct_V).  l/u are absolute indices along
 * the axis; margin is the smallest |ct(i) - (ct(p) -+ sigma)| over the two
 * comparisons that decided the bounds (ties have margin ~ 0).  */
void ora_dts_bounds(const ora_dts* s, int axis, float sigma, int32_t* l,
                    int32_t* u, REAL* margin);
/* Bounds override: when set for (axis, sigma), every pass with that sigma
 * uses these bounds instead of searching.  Used to evaluate the value path
 * on the exact windows the GPU chose.  */
void ora_dts_add_bounds_override(ora_dts* s, int axis, float sigma,
                                 const int32_t* l, const int32_t* u);
void ora_dts_clear_bounds_override(ora_dts* s);

/* ---- Soft-window DTS (the project's relaxation of the integer windows for
 * gradients with respect to the edge weights; see oracle.c).  eh / ev: the
 * edge weights dH / dV (W*H), c may be NULL (ones).  -------------------- */
void ora_soft_solve(int w, int h, const REAL* eh, const REAL* ev, const REAL* t,
                    const REAL* c, int num_iterations, int loss, float lambda,
                    float sigma_z, float step, float tau, REAL* out);
void ora_soft_backward(int w, int h, const REAL* eh, const REAL* ev, const REAL* t,
                       const REAL* c, int num_iterations, int loss, float lambda,
                       float sigma_z, float step, float tau, const REAL* grad_out,
                       REAL* grad_t, REAL* grad_c, REAL* grad_eh, REAL* grad_ev);

/* ---- HFBS: mirror of class HFBS (src/hfbs.h:99-150). -------------------- */
typedef struct {
  float sigma_x, sigma_y, sigma_l, lambda, alpha, beta;
  int bistoch_iter_max, optim_iter_max;
  float neg_exp_beta;
  int grid_x, grid_y, grid_l;
} ora_hfbs_params; /* field order of HFBSGridParams, src/hfbs.h:18-60 */

enum { ORA_G_SPLAT_SUM = 0, ORA_G_SPLAT_C, ORA_G_B, ORA_G_SPLAT_NORM,
       ORA_G_INV_DIAG_A, ORA_G_BLUR_C, ORA_G_Z_INIT, ORA_G_Z_FINAL,
       ORA_G_COUNT };

typedef struct ora_hfbs ora_hfbs;
ora_hfbs* ora_hfbs_create(int max_w, int max_h, int max_gx, int max_gy,
                          int max_gl);
void ora_hfbs_destroy(ora_hfbs* s);
void ora_hfbs_set_compat(ora_hfbs* s, int color_contract);
int ora_hfbs_set_image_dim(ora_hfbs* s, int w, int h);
void ora_hfbs_set_params(ora_hfbs* s, const ora_hfbs_params* p);
void ora_hfbs_clear_all(ora_hfbs* s);
void ora_hfbs_init_frame(ora_hfbs* s, int color_space, const uint8_t* rgba,
                         const float* target, const float* confidence);
/* returns 0 on a solve, 1 when the grid exceeded the allocation and the
 * target was copied to the output (src/hfbs.cu:594-611). */
int ora_hfbs_optimize(ora_hfbs* s);
/* target / confidence at REAL precision (NULL keeps a plane) */
void ora_hfbs_set_target_conf(ora_hfbs* s, const REAL* target, const REAL* confidence);
/* adjoint of the last optimize w.r.t. target and confidence (0 on success,
 * -1 without a completed optimize); grad_t / grad_c may be NULL */
int ora_hfbs_backward(ora_hfbs* s, const REAL* grad_out, REAL* grad_t, REAL* grad_c);
void ora_hfbs_download(const ora_hfbs* s, int image_type, REAL* dst);
/* grid dims of the last Optimize (gx, gy, gl). */
void ora_hfbs_grid_dims(const ora_hfbs* s, int* gx, int* gy, int* gl);
/* intermediate grid (gx*gy*gl, x fastest then y then l) of the last solve. */
void ora_hfbs_grid(const ora_hfbs* s, int which, REAL* dst);

#ifdef __cplusplus
}
#endif
#endif
