/*
 * libdtsgb -- C ABI of the GB300-native Domain Transform Solver (DTS) and
 * Hardware-Friendly Bilateral Solver (HFBS).
 *
 * Every entry point returns an int status (DTSGB_OK = 0); no call prints,
 * exits or aborts.  dtsgb_last_error() returns a description of the last
 * failure on the calling thread.  Arguments are plain pointers and sizes:
 *   - "host" pointers are ordinary (pageable or pinned) host memory, copied
 *     synchronously like the reference's libcua View/CopyTo;
 *   - "device" pointers are CUDA device memory of the current device;
 *   - compute calls are asynchronous on the handle's stream (set with
 *     *_set_stream; by default a stream owned by the handle), exactly like
 *     the reference's kernel launches, and every download synchronises.
 *
 * Each declaration names the reference interface it replaces.  The reference
 * paths are relative to akashbapat/domain_transform_solver.
 */
#ifndef DTSGB_H_
#define DTSGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DTSGB_API __attribute__((visibility("default")))

/* ---- status codes -------------------------------------------------------*/
#define DTSGB_OK 0
#define DTSGB_ERR_INVALID_ARGUMENT 1 /* null handle / pointer, bad enum      */
#define DTSGB_ERR_INVALID_DIMS 2     /* SetImageDim outside the allocation   */
#define DTSGB_ERR_UNSUPPORTED 3      /* parameter outside the kernels' range */
#define DTSGB_ERR_CUDA 4             /* a CUDA runtime call failed           */
#define DTSGB_ERR_OUT_OF_MEMORY 5
#define DTSGB_ERR_TOO_SMALL 6        /* image below the supported minimum    */
/* HFBS grid larger than the allocation: target copied to the output
 * (src/hfbs.cu:594-611).  A warning: the call still completed. */
#define DTSGB_WARN_GRID_TOO_LARGE 100

/* ---- enums, values identical to the reference -----------------------------
 * ImageType    src/domain_transform_common.h:20-28
 * COLOR_SPACE  src/domain_transform_common.h:32
 * RobustLoss   src/domain_transform_optimize.h:8                          */
enum {
  DTSGB_COLOR_IMAGE = 0,
  DTSGB_DIFFERENTIAL = 1,
  DTSGB_INTEGRAL = 2,
  DTSGB_TARGET = 3,
  DTSGB_CONFIDENCE = 4,
  DTSGB_OPTIMIZED_QUANTITY = 5,
  DTSGB_TEST = 6
};
enum { DTSGB_RGB = 0, DTSGB_YCBCR = 1, DTSGB_YYY = 2 };
enum { DTSGB_L1 = 0, DTSGB_L2 = 1, DTSGB_CHARBONNIER = 2 };

/* ---- creation flags -------------------------------------------------------*/
/* Store target and confidence as BF16 (rounded once at upload); all
 * arithmetic stays FP32. */
#define DTSGB_FLAG_BF16_STORAGE 0x1u
/* Search the Y-pass window up to the image height instead of reproducing the
 * reference's width limit (src/domain_transform_filter.cuh:22). */
#define DTSGB_FLAG_FIX_Y_LIMIT 0x2u
/* Keep the filter-only (DomainTransformFilter) download set. */
#define DTSGB_FLAG_FILTER_ONLY 0x4u
/* DomainTransformStereo (src/domain_transform_stereo.h:93-114): the handle
 * holds a right image and Optimize adds the photometric term. */
#define DTSGB_FLAG_STEREO 0x8u

/* ---- parameter structs, field order of the reference ----------------------*/
/* DomainFilterParams = DomainFilterParamsVec<0>,
 * src/domain_transform_filter_params.h:8-27 (sigmas[] unused at N=0). */
typedef struct {
  float sigma_x, sigma_y, sigma_r;
} dtsgb_filter_params;

/* DomainFilterParamsVec<1>: sigmas[0] is the confidence sigma. */
typedef struct {
  float sigma_x, sigma_y, sigma_r;
  float sigmas[2];
} dtsgb_conf_params;

/* DomainOptimizeParams, src/domain_transform_optimize.h:29-50. */
typedef struct {
  int num_iterations;
  int loss;
  float lambda;
  float sigma_z;
  float step_size;
  float photo_consis_lambda;
  float DT_lambda;
} dtsgb_optimize_params;

/* HFBSGridParams, src/hfbs.h:18-60 (grid_* are outputs of optimize). */
typedef struct {
  float sigma_x, sigma_y, sigma_l, lambda, alpha, beta;
  int bistoch_iter_max, optim_iter_max;
  float neg_exp_beta;
  int grid_x, grid_y, grid_l;
} dtsgb_hfbs_params;

DTSGB_API const char* dtsgb_last_error(void);
DTSGB_API int dtsgb_version(void);

/* ---- kernel timing (new; no reference counterpart) ------------------------
 * When enabled, every launch of the kernels below is bracketed by CUDA
 * events recorded on the stream it is launched on; read() synchronises on
 * those events and returns the launch count and summed duration. */
enum {
  DTSGB_K_BOUNDS = 0,   /* window-bound search from the guide          */
  DTSGB_K_DTS_ITER = 1, /* fused X+Y solver iteration                  */
  DTSGB_K_FILTER = 2,   /* filter / confidence box pass                */
  DTSGB_K_HFBS_SPLAT = 3,
  DTSGB_K_HFBS_BISTOCH = 4,
  DTSGB_K_HFBS_SOLVE = 5,
  DTSGB_K_HFBS_OTHER = 6,
  DTSGB_K_HFBS_SLICE = 7,
  DTSGB_K_DTS_OTHER = 8, /* iterate init, conversions                 */
  DTSGB_K_DTS_ADJOINT = 9, /* adjoint of one fused iteration          */
  DTSGB_K_HFBS_ADJOINT = 10, /* the whole HFBS adjoint                  */
  DTSGB_K_SOFT = 11,         /* soft-window plans, line scans, unplanned forms */
  DTSGB_K_SOFT_HALF_X = 12,  /* planned soft X half-step                    */
  DTSGB_K_SOFT_ADJ_X = 13,   /* planned soft adjoint of the X half-step     */
  DTSGB_K_SOFT_ADJ_Y = 14,   /* planned soft adjoint of the Y half-step     */
  DTSGB_K_SOFT_HALF_Y = 15,  /* planned soft Y half-step                    */
  DTSGB_K_COUNT = 16
};
/* (new) Thread blocks of the library's kernels that gave up waiting for an
 * asynchronous (TMA) copy of their tile since the library was loaded: each
 * wait polls a bounded number of times, and a block that gives up records
 * it here and leaves its tile unwritten.  0 on a healthy run. */
DTSGB_API int dtsgb_wait_timeouts(unsigned long long* count);
DTSGB_API int dtsgb_profile_enable(int enable);
DTSGB_API int dtsgb_profile_reset(void);
DTSGB_API int dtsgb_profile_read(int kernel_id, int* launches, double* total_ms);

/* ===========================================================================
 * DTS: DomainTransformFilter (src/domain_transform_filter.h:19-70) and
 * DomainTransformSolver (src/domain_transform_solver.h:34-85) over one handle.
 * ===========================================================================*/
typedef struct dtsgb_dts_s* dtsgb_dts_t;

/* DomainTransformFilter(const ImageDim&) / DomainTransformSolver(const
 * ImageDim&): allocates every buffer at max_w x max_h. */
DTSGB_API int dtsgb_dts_create(int max_w, int max_h, unsigned flags,
                               dtsgb_dts_t* out);
/* ~DomainTransformSolver */
DTSGB_API int dtsgb_dts_destroy(dtsgb_dts_t h);
/* (new) stream for all later work of this handle; NULL = own stream. */
DTSGB_API int dtsgb_dts_set_stream(dtsgb_dts_t h, void* cuda_stream);
/* (new) wait for all work queued on the handle's stream. */
DTSGB_API int dtsgb_dts_synchronize(dtsgb_dts_t h);
/* SetImageDim, src/domain_transform_filter.h:31 (invalid dims: error, the
 * previous dims stay, as the reference ignores them). */
DTSGB_API int dtsgb_dts_set_image_dim(dtsgb_dts_t h, int width, int height);
/* InitFrame(color_space, color_image)            filter.h:36
 * InitFrame(color_space, color, target, conf)    solver.h:52
 * rgba: host W*H*4 bytes; target may be NULL (filter only); confidence NULL
 * means all ones. */
DTSGB_API int dtsgb_dts_init_frame(dtsgb_dts_t h, int color_space,
                                   const void* rgba, const float* target,
                                   const float* confidence);
/* (new) same with device pointers (dense rows, no pitch). */
DTSGB_API int dtsgb_dts_init_frame_device(dtsgb_dts_t h, int color_space,
                                          const void* rgba,
                                          const float* target,
                                          const float* confidence);
/* Guide-state reuse (no reference counterpart; its InitFrame always
 * re-uploads the guide, src/domain_transform_solver.cu:46-60): a new target
 * and confidence (null: all ones) for the guide already in place, as for
 * video frames with a fixed guide.  The guide, its domain transform and the
 * window bounds of the last Optimize stay, so the next Optimize with the
 * same sigma_z skips the window-bound search; results equal InitFrame with
 * the same guide. */
DTSGB_API int dtsgb_dts_upload_targets(dtsgb_dts_t h, const float* target,
                                       const float* confidence);
DTSGB_API int dtsgb_dts_upload_targets_device(dtsgb_dts_t h, const float* target,
                                              const float* confidence);
/* ComputeColorSpaceDifferential, filter.h:53 / solver.h:57. */
DTSGB_API int dtsgb_dts_compute_differential(dtsgb_dts_t h,
                                             const dtsgb_filter_params* p);
/* IntegrateColorDifferentials, filter.h:57 / solver.h:60. */
DTSGB_API int dtsgb_dts_integrate(dtsgb_dts_t h);
/* Filter(params, input, output, num_iter), filter.h:41: host in/out. */
DTSGB_API int dtsgb_dts_filter(dtsgb_dts_t h, const dtsgb_filter_params* p,
                               const float* input, float* output,
                               int num_iter);
/* ComputeConfidence(conf_params, left_side_clear_width), solver.h:74. */
DTSGB_API int dtsgb_dts_compute_confidence(dtsgb_dts_t h,
                                           const dtsgb_conf_params* p,
                                           int left_side_clear_width);
/* Optimize(optimize_params, overwrite_target_above_conf), solver.h:66. */
DTSGB_API int dtsgb_dts_optimize(dtsgb_dts_t h,
                                 const dtsgb_optimize_params* p,
                                 float overwrite_target_above_conf);
/* Download(image_type, image), filter.h:46 / solver.h:69: host dst.
 * COLOR_IMAGE -> W*H*4 bytes, other types -> W*H floats. */
DTSGB_API int dtsgb_dts_download(dtsgb_dts_t h, int image_type, void* image);
/* (new) same into device memory (async on the handle's stream). */
DTSGB_API int dtsgb_dts_download_device(dtsgb_dts_t h, int image_type,
                                        void* image);
/* ClearAll, filter.h:49 / solver.h:78. */
DTSGB_API int dtsgb_dts_clear_all(dtsgb_dts_t h);
/* DomainTransformStereo::InitRightFrame(center_offset, color_space, image),
 * src/domain_transform_stereo.h:98 (handle created with DTSGB_FLAG_STEREO). */
DTSGB_API int dtsgb_dts_init_right_frame(dtsgb_dts_t h, float center_offset,
                                         int color_space, const void* rgba);
DTSGB_API int dtsgb_dts_init_right_frame_device(dtsgb_dts_t h,
                                                float center_offset,
                                                int color_space,
                                                const void* rgba);
/* DomainTransformStereo::ProcessRightFrame, stereo.h:102: the right image's
 * domain transform for the solver's current filter params. */
DTSGB_API int dtsgb_dts_process_right_frame(dtsgb_dts_t h);
/* (new, tests) window bounds the kernels use for one sigma on the current
 * domain transform; axis 0 = X, 1 = Y.  l, u: host W*H int32 each; the
 * window is the index range (l, u] along the axis. */
DTSGB_API int dtsgb_dts_debug_bounds(dtsgb_dts_t h, int axis, float sigma,
                                     int32_t* l, int32_t* u);
/* (new, tests) colour conversion of n host RGBA pixels through the GPU. */
DTSGB_API int dtsgb_debug_color_convert(int color_space, const void* in,
                                        void* out, long long n);

/* ===========================================================================
 * HFBS: class HFBS, src/hfbs.h:99-150.
 * ===========================================================================*/
typedef struct dtsgb_hfbs_s* dtsgb_hfbs_t;

/* HFBS(max_image_dims, max_grid_x, max_grid_y, max_grid_l), hfbs.h:107. */
DTSGB_API int dtsgb_hfbs_create(int max_w, int max_h, int max_grid_x,
                                int max_grid_y, int max_grid_l,
                                unsigned flags, dtsgb_hfbs_t* out);
DTSGB_API int dtsgb_hfbs_destroy(dtsgb_hfbs_t h);
DTSGB_API int dtsgb_hfbs_set_stream(dtsgb_hfbs_t h, void* cuda_stream);
DTSGB_API int dtsgb_hfbs_synchronize(dtsgb_hfbs_t h);
/* SetImageDim, hfbs.h:115. */
DTSGB_API int dtsgb_hfbs_set_image_dim(dtsgb_hfbs_t h, int width, int height);
/* InitFrame(color_space, color_image, target, confidence), hfbs.h:121. */
DTSGB_API int dtsgb_hfbs_init_frame(dtsgb_hfbs_t h, int color_space,
                                    const void* rgba, const float* target,
                                    const float* confidence);
DTSGB_API int dtsgb_hfbs_init_frame_device(dtsgb_hfbs_t h, int color_space,
                                           const void* rgba,
                                           const float* target,
                                           const float* confidence);
/* Guide-state reuse for HFBS (src/hfbs.cu:540-554 re-uploads the guide
 * with every InitFrame): a new target and confidence for the guide in
 * place.  The next Optimize with the same grid parameters keeps the
 * bistochastized normalisation of the last one (it depends only on the
 * guide's bins, src/hfbs.cu:626-665); results equal InitFrame with the same
 * guide. */
DTSGB_API int dtsgb_hfbs_upload_targets(dtsgb_hfbs_t h, const float* target,
                                        const float* confidence);
DTSGB_API int dtsgb_hfbs_upload_targets_device(dtsgb_hfbs_t h, const float* target,
                                               const float* confidence);
/* SetFilterParams, hfbs.h:125. */
DTSGB_API int dtsgb_hfbs_set_filter_params(dtsgb_hfbs_t h,
                                           const dtsgb_hfbs_params* p);
/* ClearAll, hfbs.h:129. */
DTSGB_API int dtsgb_hfbs_clear_all(dtsgb_hfbs_t h);
/* Optimize, hfbs.h:132.  Returns DTSGB_WARN_GRID_TOO_LARGE when the grid
 * exceeds the allocation (the target is copied to the output). */
DTSGB_API int dtsgb_hfbs_optimize(dtsgb_hfbs_t h);
/* Download(image_type, image), hfbs.h:136: TARGET, CONFIDENCE,
 * OPTIMIZED_QUANTITY (W*H floats, host). */
DTSGB_API int dtsgb_hfbs_download(dtsgb_hfbs_t h, int image_type, float* image);
DTSGB_API int dtsgb_hfbs_download_device(dtsgb_hfbs_t h, int image_type,
                                         float* image);
/* (new) grid dims of the last optimize. */
DTSGB_API int dtsgb_hfbs_grid_dims(dtsgb_hfbs_t h, int* gx, int* gy, int* gl);
/* (new, tests) one intermediate grid of the last optimize into host memory,
 * gx*gy*gl floats, x fastest: 0 splat count, 1 splat of c, 2 b,
 * 3 splat_norm, 4 inv_diag_A, 5 blurred c, 6 initial z, 7 final z. */
DTSGB_API int dtsgb_hfbs_debug_grid(dtsgb_hfbs_t h, int which, float* dst);

/* Gradients of the HFBS solve (an addition: the reference has no gradients).
 * With gradients enabled, dtsgb_hfbs_optimize keeps what the adjoint needs:
 * every heavy-ball iterate (segment 1), or z and h at every segment-th step
 * with the segment's iterates recomputed by the backward (segment > 1);
 * segment 0 chooses every iterate when those optim_iter_max planes fit in a
 * quarter of the free device memory, else about sqrt(optim_iter_max) steps
 * per segment.  The forward then runs one heavy-ball step per launch.
 * dtsgb_hfbs_backward maps dL/d(output) of the last optimize (W*H floats) to
 * dL/dtarget and dL/dconfidence (W*H floats each; either may be NULL).  Bins,
 * splat counts and the bistochastized normalisation are held fixed (the
 * guide gets no gradient), the Huber clamp of the heavy-ball step enters by
 * its mask.  InitFrame, SetImageDim, SetFilterParams or ClearAll after the
 * optimize make the backward return DTSGB_ERR_INVALID_ARGUMENT. */
DTSGB_API int dtsgb_hfbs_enable_grad(dtsgb_hfbs_t h, int enable, int segment);
/* the segment and the number of grid planes of the last optimize */
DTSGB_API int dtsgb_hfbs_grad_info(dtsgb_hfbs_t h, int* segment, int* planes);
DTSGB_API int dtsgb_hfbs_backward(dtsgb_hfbs_t h, const float* grad_out,
                                  float* grad_target, float* grad_confidence);
DTSGB_API int dtsgb_hfbs_backward_device(dtsgb_hfbs_t h, const float* grad_out,
                                         float* grad_target, float* grad_confidence);

/* ===========================================================================
 * Soft-window DTS: gradients with respect to the edge weights (new; no
 * reference counterpart).
 *
 * The reference's windows are integer (LinearSearchLowerAndUpperBound2DX,
 * src/domain_transform_filter.cuh:7-28): a pixel q belongs to p's window when
 * the transformed distance D_pq (the sum of the edge weights dH / dV,
 * Compute_dHdx / Compute_dVdy, src/domain_transform_common_kernels.cuh:81-116,
 * between them) is at most sigma_z.  The result is therefore piecewise
 * constant in the edge weights and their gradient is zero almost everywhere.
 * This mode relaxes membership to the weight ramp((sigma_z - D_pq) / tau),
 * ramp(x) = clamp(x + 1/2, 0, 1) -- fractional window ends of width tau in
 * transformed-domain units -- and solves the Optimize iteration
 * (src/domain_transform_solver.cuh:12-116) with the weighted box mean and
 * the summed weights as n.  tau -> 0 gives the integer windows clipped at the
 * image borders; unlike the reference, windows are clipped (not collapsed to
 * one side) at the borders and the Y window runs to the image height.
 *
 * A handle holds n instances (dense W*H rows).  All image arguments are
 * host arrays of n DEVICE pointers (W*H floats, or W*H*4 bytes of RGBA);
 * calls are asynchronous on the handle's stream except where noted.
 * ===========================================================================*/
typedef struct dtsgb_soft_s* dtsgb_soft_t;
DTSGB_API int dtsgb_soft_create(int n, const int* widths, const int* heights,
                                dtsgb_soft_t* out);
DTSGB_API int dtsgb_soft_destroy(dtsgb_soft_t s);
DTSGB_API int dtsgb_soft_set_stream(dtsgb_soft_t s, void* cuda_stream);
/* The guide-derived edge weights dH, dV of ComputeColorSpaceDifferential
 * (filter.cu:92-110; colour conversion as InitFrame) for the filter sigmas,
 * written to dH[i], dV[i]; synchronises. */
DTSGB_API int dtsgb_soft_edge_weights(dtsgb_soft_t s, int color_space,
                                      const void* const* rgba,
                                      const dtsgb_filter_params* filter,
                                      float* const* dH, float* const* dV);
/* Soft-window Optimize from given edge weights (finite, > 0; the guide's
 * are >= 1), target and confidence (NULL: ones) into out.  Keeps every
 * iterate for dtsgb_soft_backward.  tau in (0, 2 sigma_z]; L1 and zero
 * iterations return the target.  No confidence overwrite. */
DTSGB_API int dtsgb_soft_solve(dtsgb_soft_t s, const float* const* dH,
                               const float* const* dV, const float* const* target,
                               const float* const* confidence,
                               const dtsgb_optimize_params* optimize, float tau,
                               float* const* out);
/* Adjoint of the last dtsgb_soft_solve: dL/dtarget, dL/dconfidence, dL/ddH,
 * dL/ddV for the upstream gradient dL/dout (any output array may be NULL);
 * synchronises. */
DTSGB_API int dtsgb_soft_backward(dtsgb_soft_t s, const float* const* grad_out,
                                  float* const* grad_target,
                                  float* const* grad_confidence,
                                  float* const* grad_dH, float* const* grad_dV);

/* ===========================================================================
 * Allocation-free DTS solve (no counterpart in the reference).
 *
 * For callers that cannot call cudaMalloc: code that runs inside a CUDA-graph
 * capture owned by another framework, real-time pipelines that forbid device
 * allocation after start-up, or hosts whose own allocator must own every
 * device allocation.  One call is ComputeColorSpaceDifferential +
 * IntegrateColorDifferentials + Optimize of DomainTransformSolver on device
 * buffers the caller owns: rgba (W*H*4 bytes, RGBA, dense rows), target and
 * confidence (W*H floats; confidence may be NULL = all ones) and output (W*H
 * floats, must not alias an input), all enqueued on cuda_stream.
 *
 * The solve's scratch (8 bytes per pixel: window bounds and one iterate) is a
 * static device array of DTSGB_NOALLOC_MAX_PIXELS pixels (8 MiB) inside the
 * library, which every GPU that loads the library holds until the process
 * exits.  Larger images return DTSGB_ERR_UNSUPPORTED.  The first call on a
 * device looks the array up with cudaGetSymbolAddress, so make it before any
 * stream capture.  All calls on a device share the array and it keeps the
 * previous call's contents; nothing in it needs to start at zero, since a
 * call writes every element it reads before reading it.  Calls that overlap
 * on the GPU race on the array and must be serialised by the caller.  The
 * call allocates nothing: no cudaMalloc, cudaFree, stream creation or
 * allocating library routine.
 *
 * Limits beyond the allocating path: sigma_z below DTSGB_NOALLOC_MAX_SIGMA_Z
 * (97; the iteration keeps its 32x32 tile plus a floor(sigma_z) halo on each
 * side in shared memory, (32 + 2h) * (64 + 2h) * 4 bytes for h =
 * floor(sigma_z), which must fit in 227 KiB; the allocating path takes any
 * sigma_z below 254); rgba, target, confidence and output 4-byte aligned
 * (DTSGB_ERR_INVALID_ARGUMENT otherwise).  The array's address is looked up
 * once per device ordinal in the primary context: use the call from the
 * primary context (the runtime API's default) and not across
 * cudaDeviceReset.  The window bounds sum the edge weights in float, one by
 * one, where the allocating path takes exact fixed-point prefix
 * differences: the two agree except at windows whose sum lies within
 * rounding of sigma_z, so results match the allocating path within the
 * parity tolerance rather than bit for bit.
 * ===========================================================================*/
#define DTSGB_NOALLOC_MAX_PIXELS (1LL << 20)
#define DTSGB_NOALLOC_MAX_SIGMA_Z 97.0f
DTSGB_API int dtsgb_dts_solve_noalloc(int width, int height, int color_space,
                                      const void* rgba, const float* target,
                                      const float* confidence,
                                      const dtsgb_filter_params* filter,
                                      const dtsgb_optimize_params* optimize,
                                      float overwrite_target_above_conf,
                                      float* output, void* cuda_stream);

/* ===========================================================================
 * Batched solves (new; no reference counterpart): n independent instances of
 * uneven size in one HBM arena, each solved with DTS and/or HFBS by single
 * launches that cover every instance (the reference solves one image per
 * object, src/edge_aware_solver.h:59-90).  A batch reuses the per-image
 * semantics of the classes above: dtsgb_batch_solve_dts is
 * ComputeColorSpaceDifferential + IntegrateColorDifferentials + Optimize on
 * every instance, dtsgb_batch_solve_hfbs is HFBS::Optimize on every instance.
 * ===========================================================================*/
typedef struct dtsgb_batch_s* dtsgb_batch_t;

DTSGB_API int dtsgb_batch_create(int n, const int* widths, const int* heights,
                                 unsigned flags, dtsgb_batch_t* out);
DTSGB_API int dtsgb_batch_destroy(dtsgb_batch_t b);
DTSGB_API int dtsgb_batch_set_stream(dtsgb_batch_t b, void* cuda_stream);
/* Capture each solve as a CUDA graph on first use and replay it while the
 * parameters stay the same (default on). */
DTSGB_API int dtsgb_batch_use_graphs(dtsgb_batch_t b, int enable);
/* Host arrays of n pointers: rgba (W*H*4 bytes each), target and confidence
 * (W*H floats each).  confidence may be NULL, or hold NULL entries: ones. */
DTSGB_API int dtsgb_batch_upload(dtsgb_batch_t b, int color_space,
                                 const void* const* rgba,
                                 const float* const* target,
                                 const float* const* confidence);
DTSGB_API int dtsgb_batch_upload_device(dtsgb_batch_t b, int color_space,
                                        const void* const* rgba,
                                        const float* const* target,
                                        const float* const* confidence);
/* Replace target and confidence only; the guide (and the state derived
 * from it) is kept.  n host / device pointers as in dtsgb_batch_upload. */
DTSGB_API int dtsgb_batch_upload_targets(dtsgb_batch_t b, const float* const* target,
                                         const float* const* confidence);
DTSGB_API int dtsgb_batch_upload_targets_device(dtsgb_batch_t b,
                                                const float* const* target,
                                                const float* const* confidence);
DTSGB_API int dtsgb_batch_solve_dts(dtsgb_batch_t b,
                                    const dtsgb_filter_params* filter,
                                    const dtsgb_optimize_params* optimize,
                                    float overwrite_target_above_conf);
DTSGB_API int dtsgb_batch_solve_hfbs(dtsgb_batch_t b,
                                     const dtsgb_hfbs_params* params);
/* which: 0 = DTS result, 1 = HFBS result; dst: n pointers (W*H floats). */
DTSGB_API int dtsgb_batch_download(dtsgb_batch_t b, int which,
                                   float* const* dst);
DTSGB_API int dtsgb_batch_download_device(dtsgb_batch_t b, int which,
                                          float* const* dst);
/* Intermediate state of instance i after the last solve, for parity checks
 * (new; the reference's FilterStructPtr() exposes the same state through
 * its device structs, src/domain_transform_filter.h:64).  which:
 *   DTSGB_BATCH_PLANE_BOUNDS  W*H uint32 packed window offsets of the last
 *                             DTS solve (bits 0-7 dl_x, 8-15 du_x, 16-23
 *                             dl_y, 24-31 du_y; the window along an axis is
 *                             the pixels p-dl+1 .. p+du)
 *   DTSGB_BATCH_PLANE_COUNT   gx*gy*gl floats, the HFBS splat counts
 *   DTSGB_BATCH_PLANE_CSUM    gx*gy*gl floats, the splatted confidences
 *   DTSGB_BATCH_PLANE_B       gx*gy*gl floats, the splatted c * t
 * (grids x fastest, then y, then luma).  dst_bytes must cover the plane. */
#define DTSGB_BATCH_PLANE_BOUNDS 0
#define DTSGB_BATCH_PLANE_COUNT 1
#define DTSGB_BATCH_PLANE_CSUM 2
#define DTSGB_BATCH_PLANE_B 3
DTSGB_API int dtsgb_batch_debug_plane(dtsgb_batch_t b, int i, int which, void* dst,
                                      long long dst_bytes);

/* ---- Tuning (new).  DTSGB_TUNE_DTS_TILE: tile width of the fused DTS
 * iteration and its adjoint, 64 (64 x 128 tiles) or 32 (32 x 32 tiles;
 * the default when the batch holds under 4 x 152 x 64 x 64 pixels).
 * DTSGB_TUNE_HFBS_GROUP_VOXELS:
 * the HFBS iterations run over groups of consecutive instances holding at
 * most this many grid voxels, all iterations of one group before the next,
 * so that a group's grids can stay in L2 (0, the default: all instances at
 * once).  Neither changes results beyond the last bits of the DTS iterate
 * (HFBS: bitwise identical). */
#define DTSGB_TUNE_DTS_TILE 0
#define DTSGB_TUNE_HFBS_GROUP_VOXELS 1
/* DTSGB_TUNE_REUSE_GUIDE_STATE (default 1): while the guide is unchanged
 * (dtsgb_batch_upload_targets between solves, as for video frames whose
 * target changes), a DTS solve with the same sigmas keeps the window bounds
 * and an HFBS solve with the same grid keeps the bistochastized
 * normalisation instead of recomputing them; results are identical. */
#define DTSGB_TUNE_REUSE_GUIDE_STATE 2
/* DTSGB_TUNE_HFBS_SOLVE_STEPS: heavy-ball steps per launch, 4 (default:
 * a temporally blocked kernel, each launch four steps on 24 x 24-column
 * blocks staged in shared memory, for grids of at most 16 levels) or 1
 * (one step per launch, any grid; with a group budget its grids can stay in
 * L2).  The two add a voxel's six neighbour products in different roundings:
 * results agree to FP32 rounding, and each is differentiated exactly. */
#define DTSGB_TUNE_HFBS_SOLVE_STEPS 3
/* DTSGB_TUNE_BOUNDS_SEGMENT: pixels each thread of the window-bound search
 * walks per axis with its two pointers (4, 8 or 16; default 8).  Longer
 * segments restart the walk less often, shorter ones spread a tile's lines
 * over more threads; the windows are identical. */
#define DTSGB_TUNE_BOUNDS_SEGMENT 4
DTSGB_API int dtsgb_batch_set_tuning(dtsgb_batch_t b, int knob, long long value);
DTSGB_API int dtsgb_batch_get_tuning(dtsgb_batch_t b, int knob, long long* value);
/* Times the uploaded batch's solves (reps runs each on the batch's stream,
 * with the guide state recomputed every run) under each DTS tile shape, then
 * each bounds segment (filter and optimize given), and under every pair of
 * HFBS steps per launch (4, 1) and group budget (0, 1M, 2M, 4M, 8M voxels;
 * hfbs given); keeps the fastest setting of each and leaves the results of
 * one solve with it. */
DTSGB_API int dtsgb_batch_autotune(dtsgb_batch_t b, const dtsgb_filter_params* filter,
                                   const dtsgb_optimize_params* optimize,
                                   float overwrite_target_above_conf,
                                   const dtsgb_hfbs_params* hfbs, int reps);
/* dtsgb_batch_autotune with a cache file: a line per tuned case (a hash of
 * the device name and SM count, the batch's sizes and flags and the solve
 * parameters, then the chosen DTS tile, bounds segment, HFBS steps per
 * launch and HFBS group budget).  A case found there is applied without
 * timing (*from_cache = 1); otherwise it is tuned and appended.  The file is
 * created when missing; failing to write it is not an error. */
DTSGB_API int dtsgb_batch_autotune_cached(dtsgb_batch_t b,
                                          const dtsgb_filter_params* filter,
                                          const dtsgb_optimize_params* optimize,
                                          float overwrite_target_above_conf,
                                          const dtsgb_hfbs_params* hfbs, int reps,
                                          const char* cache_path, int* from_cache);

/* ---- Overlapped host-to-host solves (new; the reference copies, solves
 * and copies back one image at a time).  A pipeline splits n instances into
 * n_chunks runs of consecutive instances of about equal pixel count, each a
 * batch with its own stream (created with `flags`), and dtsgb_pipeline_run
 * enqueues every chunk's upload, solves and downloads without waiting, so
 * the copy engines move one chunk while another is solved.  The copies are
 * asynchronous only from pinned host memory (cudaHostAlloc /
 * cudaHostRegister); run returns when every result is on the host or, after
 * a failure, when nothing enqueued is still running.  Arrays hold n
 * pointers, as for dtsgb_batch_upload / dtsgb_batch_download.
 * ===========================================================================*/
typedef struct dtsgb_pipeline_s* dtsgb_pipeline_t;

DTSGB_API int dtsgb_pipeline_create(int n, const int* widths, const int* heights,
                                    unsigned flags, int n_chunks,
                                    dtsgb_pipeline_t* out);
DTSGB_API int dtsgb_pipeline_destroy(dtsgb_pipeline_t p);
/* Number of chunks (min(n_chunks, n)). */
DTSGB_API int dtsgb_pipeline_chunks(dtsgb_pipeline_t p);
/* Chunk k's batch, owned by the pipeline (for dtsgb_batch_set_tuning and
 * the like). */
DTSGB_API int dtsgb_pipeline_batch(dtsgb_pipeline_t p, int k, dtsgb_batch_t* out);
/* Upload, then DTS (when filter and optimize are both given; results into
 * out_dts) and HFBS (when hfbs is given; results into out_hfbs), then
 * download, for every instance. */
DTSGB_API int dtsgb_pipeline_run(dtsgb_pipeline_t p, int color_space,
                                 const void* const* rgba, const float* const* target,
                                 const float* const* confidence,
                                 const dtsgb_filter_params* filter,
                                 const dtsgb_optimize_params* optimize,
                                 float overwrite_target_above_conf,
                                 const dtsgb_hfbs_params* hfbs, float* const* out_dts,
                                 float* const* out_hfbs);
/* The same for a differentiable solve: upload, DTS with gradients on (the
 * automatic checkpoint choice of dtsgb_batch_enable_grad), download of the
 * results into out_v, then the backward of the upstream gradients grad_out
 * into grad_target / grad_confidence (either may be NULL or hold NULL
 * entries), chunk by chunk without waiting. */
DTSGB_API int dtsgb_pipeline_run_grad(dtsgb_pipeline_t p, int color_space,
                                      const void* const* rgba, const float* const* target,
                                      const float* const* confidence,
                                      const dtsgb_filter_params* filter,
                                      const dtsgb_optimize_params* optimize,
                                      const float* const* grad_out, float* const* out_v,
                                      float* const* grad_target,
                                      float* const* grad_confidence);

/* ---- Gradients of the batched DTS solve (new; the reference has no
 * gradients).  With gradients enabled, dtsgb_batch_solve_dts also keeps the
 * iterate v_k every `segment` iterations (0 = automatic: every iterate, so
 * that the backward recomputes nothing, when those num_iterations + 4 planes
 * fit in a quarter of the free device memory; else the length that holds
 * the fewest planes, near sqrt(num_iterations), and of those the shortest),
 * and dtsgb_batch_dts_backward maps an upstream gradient dL/dv of each DTS
 * result to dL/dtarget and dL/dconfidence of the same solve.  The window
 * bounds found from the guide are held fixed: they are piecewise constant in
 * the guide, so the solve's derivative with respect to the guide's edge
 * weights is zero almost everywhere.  The iterates between checkpoints are
 * recomputed, so the solve holds ceil(N/segment) - 1 + segment + 4 planes of
 * W*H floats per instance, not N.  L2 and Charbonnier; L1 and zero iterations
 * return the target, so dL/dtarget = dL/dv.  A solve with the confidence
 * overwrite in (0,1) returns DTSGB_ERR_UNSUPPORTED while gradients are on.
 * For BF16 storage the derivative is taken at the BF16-rounded target and
 * confidence.  The adjoint's tile holds sigma_z below 80 (larger values
 * return DTSGB_ERR_UNSUPPORTED from the backward; the forward takes any
 * sigma_z below 254).  grad_target / grad_confidence (n pointers, W*H floats) may be
 * NULL or hold NULL entries to skip an output. */
DTSGB_API int dtsgb_batch_enable_grad(dtsgb_batch_t b, int enable, int segment);
/* segment length and planes held by the last solve (0, 0 before any). */
DTSGB_API int dtsgb_batch_grad_info(dtsgb_batch_t b, int* segment, int* planes);
DTSGB_API int dtsgb_batch_dts_backward(dtsgb_batch_t b, const float* const* grad_out,
                                       float* const* grad_target,
                                       float* const* grad_confidence);
DTSGB_API int dtsgb_batch_dts_backward_device(dtsgb_batch_t b,
                                              const float* const* grad_out,
                                              float* const* grad_target,
                                              float* const* grad_confidence);
/* The HFBS counterpart: with gradients enabled (dtsgb_batch_enable_grad),
 * dtsgb_batch_solve_hfbs keeps its heavy-ball iterates (the same segment
 * choice; the forward result is unchanged) and dtsgb_batch_hfbs_backward maps
 * the upstream gradients of its results to dL/dtarget and dL/dconfidence of
 * every instance, as dtsgb_hfbs_backward does for one. */
DTSGB_API int dtsgb_batch_hfbs_backward(dtsgb_batch_t b, const float* const* grad_out,
                                        float* const* grad_target,
                                        float* const* grad_confidence);
DTSGB_API int dtsgb_batch_hfbs_backward_device(dtsgb_batch_t b,
                                               const float* const* grad_out,
                                               float* const* grad_target,
                                               float* const* grad_confidence);
/* segment and grid planes of the last differentiable HFBS solve (0, 0: none) */
DTSGB_API int dtsgb_batch_hfbs_grad_info(dtsgb_batch_t b, int* segment, int* planes);

/* ---- Host-side image helper (no counterpart: the reference's drivers decode
 * PNG with OpenCV).  Undoes the PNG row filters (types 0-4) of `height` rows
 * of `stride` bytes, each preceded by its filter byte in `raw`, with `bpp`
 * bytes per pixel; writes height * stride bytes to `out`. */
DTSGB_API int dtsgb_png_unfilter(const unsigned char* raw, int height, int stride,
                                 int bpp, unsigned char* out);

#ifdef __cplusplus
}
#endif
#endif /* DTSGB_H_ */
