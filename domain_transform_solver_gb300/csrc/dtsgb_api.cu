// C ABI of libdtsgb: handle objects that mirror the reference classes
// DomainTransformFilter / DomainTransformSolver
// (src/domain_transform_filter.cu, src/domain_transform_solver.cu) and HFBS
// (src/hfbs.cu), on top of the sm_103a kernels of dts_kernels.cu and
// hfbs_kernels.cu.
//
// Differences of form, not of results, from the reference classes:
//  * no call prints or exits: every call returns a status;
//  * each handle owns one CUDA stream (or borrows one, *_set_stream);
//  * the domain transform is evaluated lazily: ComputeColorSpaceDifferential
//    records the sigma ratios and the window bounds are built from the guide
//    when a pass needs them, straight from the guide without materialising
//    dH, dV or their prefix sums (Download(DIFFERENTIAL / INTEGRAL) computes
//    them on demand).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dtsgb.h"
#include "color.cuh"
#include "dtsgb_internal.cuh"
#include "tma.cuh"
#include "hfbs_internal.cuh"

namespace dtsgb {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return DTSGB_ERR_CUDA;
}

float filter_sigma_multiplier(int it, int n) {
  if (it == 0) return 1.f;
  return (float)(3 * std::pow(2.0, (double)(n - (it + 1))) /
                 std::sqrt(std::pow(4.0, (double)n) - 1));
}

namespace {

std::vector<Tile> make_tiles(int w, int h, int tw, int th) {
  std::vector<Tile> t;
  for (int y = 0; y < h; y += th)
    for (int x = 0; x < w; x += tw) t.push_back(Tile{0, x, y, 0});
  return t;
}

}  // namespace
}  // namespace dtsgb

using namespace dtsgb;

// ===========================================================================
// DTS handle
// ===========================================================================
struct dtsgb_dts_s {
  int max_w = 0, max_h = 0, pitch = 0;
  int w = 0, h = 0;
  unsigned flags = 0;
  Storage st = Storage::F32;
  int ref_y = 1;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  size_t plane = 0;  // elements per plane

  uchar4* guide = nullptr;
  void* target = nullptr;
  void* conf = nullptr;
  uint32_t* bounds = nullptr;
  float* v[4] = {nullptr, nullptr, nullptr, nullptr};
  float* scr[2] = {nullptr, nullptr};

  Inst h_inst{};
  Inst* d_inst = nullptr;
  Tile* d_tb = nullptr;  // bounds tiles
  Tile* d_ti = nullptr;  // iteration tiles
  Tile* d_ti_small = nullptr;  // small iteration tiles when d_ti holds big ones
  int ntb = 0, nti = 0, nti_small = 0;

  bool diff_valid = false;
  float ratio_x = 0.f, ratio_y = 0.f;
  // the solver's filter_params_ (set only by ComputeColorSpaceDifferential)
  bool solver_fp_valid = false;
  float solver_sx = 0.f, solver_sr = 0.f;
  // DomainTransformStereo: right guide (converted), centre offset and the
  // sigma ratio of its dHdx (-1: ProcessRightFrame not called)
  uchar4* right = nullptr;
  float center_offset = 0.f;
  float right_ratio = -1.f;
  bool bounds_valid = false;
  float b_sx = 0.f, b_sy = 0.f;
  int var_idx = -1;

  // tensor maps of the iterate planes (TMA staging of the iteration),
  // rebuilt when the image dims change
  mutable TmaCache tma;

  size_t tsize() const { return st == Storage::F32 ? 4 : 2; }
  DtsLaunch launch_b() const { return DtsLaunch{d_inst, d_tb, ntb, 1}; }
  bool small = false;
  DtsLaunch launch_i() const {
    return DtsLaunch{d_inst, d_ti, nti, 1, small, small ? nullptr : d_ti_small, nti_small,
                     &tma, &h_inst};
  }
};

static int dts_layout(dtsgb_dts_t h) {
  h->h_inst = Inst{h->w, h->h, h->pitch, 0, 0};
  h->tma.clear();
  std::vector<Tile> tb = make_tiles(h->w, h->h, kBoundsTW, kBoundsTH);
  const long long t64 = (long long)((h->w + kIterTW - 1) / kIterTW) *
                        ((h->h + kIterTH - 1) / kIterTH);
  h->small = use_small_iter_tiles(t64);
  std::vector<Tile> ti =
      h->small ? make_tiles(h->w, h->h, kIterSmallTW, kIterSmallTH)
               : make_tiles(h->w, h->h, kIterTW, kIterTH);
  h->ntb = (int)tb.size();
  h->nti = (int)ti.size();
  if (!h->small) {
    // small tiles too, for halos that do not fit the big tiles' shared memory
    std::vector<Tile> ts = make_tiles(h->w, h->h, kIterSmallTW, kIterSmallTH);
    h->nti_small = (int)ts.size();
    DTSGB_CUDA(cudaMemcpyAsync(h->d_ti_small, ts.data(), ts.size() * sizeof(Tile),
                               cudaMemcpyHostToDevice, h->stream));
    DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  }
  DTSGB_CUDA(cudaMemcpyAsync(h->d_inst, &h->h_inst, sizeof(Inst),
                             cudaMemcpyHostToDevice, h->stream));
  DTSGB_CUDA(cudaMemcpyAsync(h->d_tb, tb.data(), tb.size() * sizeof(Tile),
                             cudaMemcpyHostToDevice, h->stream));
  DTSGB_CUDA(cudaMemcpyAsync(h->d_ti, ti.data(), ti.size() * sizeof(Tile),
                             cudaMemcpyHostToDevice, h->stream));
  DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  h->bounds_valid = false;
  return DTSGB_OK;
}

static void dts_free(dtsgb_dts_t h) {
  dfree(h->right);
  dfree(h->guide);
  dfree(h->target);
  dfree(h->conf);
  dfree(h->bounds);
  for (auto& p : h->v) dfree(p);
  for (auto& p : h->scr) dfree(p);
  dfree(h->d_inst);
  dfree(h->d_tb);
  dfree(h->d_ti);
  dfree(h->d_ti_small);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  h->stream = nullptr;
}

extern "C" {

DTSGB_API const char* dtsgb_last_error(void) { return g_last_error.c_str(); }
DTSGB_API int dtsgb_version(void) { return 1; }

DTSGB_API int dtsgb_dts_create(int max_w, int max_h, unsigned flags,
                               dtsgb_dts_t* out) {
  if (!out) return fail(DTSGB_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  if (max_w <= 0 || max_h <= 0)
    return fail(DTSGB_ERR_INVALID_DIMS, "max dims must be positive");
  dtsgb_dts_t h = new dtsgb_dts_s();
  h->max_w = h->w = max_w;
  h->max_h = h->h = max_h;
  h->pitch = round_up(max_w, 32);
  h->flags = flags;
  h->st = (flags & DTSGB_FLAG_BF16_STORAGE) ? Storage::BF16 : Storage::F32;
  h->ref_y = (flags & DTSGB_FLAG_FIX_Y_LIMIT) ? 0 : 1;
  h->plane = (size_t)h->pitch * max_h;
  int st = DTSGB_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "cudaStreamCreate");
  }
  h->own_stream = true;
  const size_t ntiles_b = (size_t)((max_w + kBoundsTW - 1) / kBoundsTW) *
                          ((max_h + kBoundsTH - 1) / kBoundsTH);
  const size_t ntiles_i = (size_t)((max_w + kIterSmallTW - 1) / kIterSmallTW) *
                          ((max_h + kIterSmallTH - 1) / kIterSmallTH);
  if (!st) st = dalloc(&h->guide, h->plane);
  if (!st && (flags & DTSGB_FLAG_STEREO)) st = dalloc(&h->right, h->plane);
  if (!st) st = dalloc((char**)&h->target, h->plane * h->tsize());
  if (!st) st = dalloc((char**)&h->conf, h->plane * h->tsize());
  if (!st) st = dalloc(&h->bounds, h->plane);
  for (int i = 0; i < 4 && !st; ++i) st = dalloc(&h->v[i], h->plane);
  for (int i = 0; i < 2 && !st; ++i) st = dalloc(&h->scr[i], h->plane);
  if (!st) st = dalloc(&h->d_inst, 1);
  if (!st) st = dalloc(&h->d_tb, ntiles_b);
  if (!st) st = dalloc(&h->d_ti, ntiles_i);
  if (!st) st = dalloc(&h->d_ti_small, ntiles_i);
  if (!st) st = dts_layout(h);
  if (st) {
    if (st == DTSGB_ERR_CUDA && g_last_error.find("memory") != std::string::npos)
      st = DTSGB_ERR_OUT_OF_MEMORY;
    dts_free(h);
    delete h;
    return st;
  }
  *out = h;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_destroy(dtsgb_dts_t h) {
  if (!h) return DTSGB_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  dts_free(h);
  delete h;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_set_stream(dtsgb_dts_t h, void* stream) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->own_stream = false;
  h->stream = (cudaStream_t)stream;
  if (!stream) {
    DTSGB_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
  }
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_synchronize(dtsgb_dts_t h) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_set_image_dim(dtsgb_dts_t h, int w, int hh) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if (!(w > 0 && w <= h->max_w && hh > 0 && hh <= h->max_h))
    return fail(DTSGB_ERR_INVALID_DIMS,
                "Invalid image dims WxH:" + std::to_string(w) + " x " +
                    std::to_string(hh));
  h->w = w;
  h->h = hh;
  return dts_layout(h);
}

static int dts_upload_plane(dtsgb_dts_t h, const float* src, void* dst,
                            cudaMemcpyKind kind) {
  const size_t wb = (size_t)h->w * sizeof(float);
  if (h->st == Storage::F32) {
    DTSGB_CUDA(cudaMemcpy2DAsync(dst, (size_t)h->pitch * 4, src, wb, wb, h->h,
                                 kind, h->stream));
    return DTSGB_OK;
  }
  DTSGB_CUDA(cudaMemcpy2DAsync(h->scr[0], (size_t)h->pitch * 4, src, wb, wb,
                               h->h, kind, h->stream));
  return launch_storage_from_float(&h->h_inst, 1, h->st, h->scr[0], dst,
                                   (long long)h->pitch * h->h, h->stream);
}

static int dts_init_frame(dtsgb_dts_t h, int cs, const void* rgba,
                          const float* target, const float* conf,
                          cudaMemcpyKind kind) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if (!rgba) return fail(DTSGB_ERR_INVALID_ARGUMENT, "color image is null");
  if (cs < DTSGB_RGB || cs > DTSGB_YYY)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid color space");
  const size_t wb = (size_t)h->w * 4;
  DTSGB_CUDA(cudaMemcpy2DAsync(h->guide, (size_t)h->pitch * 4, rgba, wb, wb,
                               h->h, kind, h->stream));
  int st = launch_color_convert_flat(h->guide, (long long)h->pitch * h->h, cs,
                                     h->stream);
  if (st) return st;
  if (target) {
    st = dts_upload_plane(h, target, h->target, kind);
    if (st) return st;
  }
  if (target || conf) {
    if (conf) {
      st = dts_upload_plane(h, conf, h->conf, kind);
    } else {
      st = launch_fill_storage(h->st, h->conf, (long long)h->plane, 1.f,
                               h->stream);
    }
    if (st) return st;
  }
  h->bounds_valid = false;
  if (kind == cudaMemcpyHostToDevice) DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_init_frame(dtsgb_dts_t h, int cs, const void* rgba,
                                   const float* target, const float* conf) {
  return dts_init_frame(h, cs, rgba, target, conf, cudaMemcpyHostToDevice);
}

DTSGB_API int dtsgb_dts_init_frame_device(dtsgb_dts_t h, int cs,
                                          const void* rgba, const float* target,
                                          const float* conf) {
  return dts_init_frame(h, cs, rgba, target, conf, cudaMemcpyDeviceToDevice);
}

// A new target and confidence for the guide already in place (video frames
// with a fixed guide): the guide, its domain transform and the cached window
// bounds stay, so the next Optimize with the same sigma_z skips the
// window-bound search.  Results equal InitFrame with the same guide.
static int dts_upload_targets(dtsgb_dts_t h, const float* target, const float* conf,
                              cudaMemcpyKind kind) {
  if (!h || !target) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  int st = dts_upload_plane(h, target, h->target, kind);
  if (st) return st;
  st = conf ? dts_upload_plane(h, conf, h->conf, kind)
            : launch_fill_storage(h->st, h->conf, (long long)h->plane, 1.f, h->stream);
  if (st) return st;
  if (kind == cudaMemcpyHostToDevice) DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_upload_targets(dtsgb_dts_t h, const float* target,
                                       const float* conf) {
  return dts_upload_targets(h, target, conf, cudaMemcpyHostToDevice);
}

DTSGB_API int dtsgb_dts_upload_targets_device(dtsgb_dts_t h, const float* target,
                                              const float* conf) {
  return dts_upload_targets(h, target, conf, cudaMemcpyDeviceToDevice);
}

static int check_filter_params(float sx, float sy, float sr) {
  if (!finite_pos(sx) || !finite_pos(sy) || !finite_pos(sr))
    return fail(DTSGB_ERR_INVALID_ARGUMENT,
                "sigma_x, sigma_y and sigma_r must be finite and positive");
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_compute_differential(dtsgb_dts_t h,
                                             const dtsgb_filter_params* p) {
  if (!h || !p) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  int st = check_filter_params(p->sigma_x, p->sigma_y, p->sigma_r);
  if (st) return st;
  h->ratio_x = p->sigma_x / p->sigma_r;
  h->ratio_y = p->sigma_y / p->sigma_r;
  h->diff_valid = true;
  h->bounds_valid = false;
  h->solver_fp_valid = true;
  h->solver_sx = p->sigma_x;
  h->solver_sr = p->sigma_r;
  return DTSGB_OK;
}

static int dts_init_right(dtsgb_dts_t h, float offset, int cs, const void* rgba,
                          cudaMemcpyKind kind) {
  if (!h || !rgba) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (!h->right)
    return fail(DTSGB_ERR_INVALID_ARGUMENT,
                "InitRightFrame needs a handle created with DTSGB_FLAG_STEREO");
  if (cs < DTSGB_RGB || cs > DTSGB_YYY)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid color space");
  if (!std::isfinite(offset))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "center offset must be finite");
  const size_t wb = (size_t)h->w * 4;
  DTSGB_CUDA(cudaMemcpy2DAsync(h->right, (size_t)h->pitch * 4, rgba, wb, wb, h->h,
                               kind, h->stream));
  int st = launch_color_convert_flat(h->right, (long long)h->pitch * h->h, cs,
                                     h->stream);
  if (st) return st;
  h->center_offset = offset;
  if (kind == cudaMemcpyHostToDevice) DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_init_right_frame(dtsgb_dts_t h, float offset, int cs,
                                         const void* rgba) {
  return dts_init_right(h, offset, cs, rgba, cudaMemcpyHostToDevice);
}

DTSGB_API int dtsgb_dts_init_right_frame_device(dtsgb_dts_t h, float offset,
                                                int cs, const void* rgba) {
  return dts_init_right(h, offset, cs, rgba, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_dts_process_right_frame(dtsgb_dts_t h) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if (!h->right)
    return fail(DTSGB_ERR_INVALID_ARGUMENT,
                "ProcessRightFrame needs a handle created with DTSGB_FLAG_STEREO");
  if (!h->solver_fp_valid)
    return fail(DTSGB_ERR_INVALID_ARGUMENT,
                "ProcessRightFrame uses the filter params of "
                "ComputeColorSpaceDifferential: call that first");
  // the right image's dHdx is evaluated from its guide when a pass needs it
  h->right_ratio = h->solver_sx / h->solver_sr;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_integrate(dtsgb_dts_t h) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  return DTSGB_OK;
}

// Window bounds for (sx, sy) on the current domain transform.  Without a
// differential (after ClearAll) the reference's dH / ct buffers are zero and
// every window collapses to the pixel itself.
static int dts_bounds(dtsgb_dts_t h, float sx, float sy, bool use_cache) {
  if (use_cache && h->bounds_valid && h->b_sx == sx && h->b_sy == sy)
    return DTSGB_OK;
  if (!finite_pos(sx) || !finite_pos(sy))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "sigma must be finite and positive");
  int st = launch_bounds(h->launch_b(), h->guide, h->bounds,
                         h->diff_valid ? h->ratio_x : -1.f,
                         h->diff_valid ? h->ratio_y : -1.f, sx, sy, h->ref_y,
                         h->stream);
  if (st) return st;
  h->bounds_valid = use_cache;
  h->b_sx = sx;
  h->b_sy = sy;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_optimize(dtsgb_dts_t h, const dtsgb_optimize_params* p,
                                 float overwrite) {
  if (!h || !p) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (p->loss < DTSGB_L1 || p->loss > DTSGB_CHARBONNIER)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid loss");
  if (p->num_iterations < 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "num_iterations < 0");
  if (!finite_pos(p->sigma_z) || p->sigma_z >= 254.f)
    return fail(DTSGB_ERR_UNSUPPORTED, "sigma_z must be in (0, 254)");
  if (!std::isfinite(p->lambda) || !std::isfinite(p->step_size))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "lambda / step_size not finite");
  int st = launch_init_var(h->launch_i(), h->st, h->target, h->v[0], h->stream);
  if (st) return st;
  h->var_idx = 0;
  // RobustLoss::L1 has no kernel in the reference's switches, so the
  // iterate stays the target (src/domain_transform_solver.cu:133-153).
  if (p->loss == DTSGB_L1 || p->num_iterations == 0) return DTSGB_OK;
  st = dts_bounds(h, p->sigma_z, p->sigma_z, true);
  if (st) return st;
  const int halo = (int)std::floor(p->sigma_z);
  const IterMode mode = p->loss == DTSGB_L2 ? IterMode::L2 : IterMode::CHARB;
  // DomainTransformStereo::Optimize adds PhotometricL2LossTerm with
  // alpha = (sigma_r / sigma_x)^2 of filter_params_, beta = -1
  // (src/domain_transform_stereo.cu:77-88)
  StereoArgs sa{};
  const StereoArgs* sp = nullptr;
  if (h->flags & DTSGB_FLAG_STEREO) {
    if (!h->solver_fp_valid)
      return fail(DTSGB_ERR_INVALID_ARGUMENT,
                  "stereo Optimize needs ComputeColorSpaceDifferential first");
    const float sxr = h->solver_sr / h->solver_sx;
    sa = StereoArgs{h->guide, h->right, h->center_offset, p->photo_consis_lambda,
                    sxr * sxr, h->right_ratio};
    sp = &sa;
  }
  int a = 0, b = 1;
  for (int it = 0; it < p->num_iterations; ++it) {
    st = launch_dts_iter(h->launch_i(), h->st, mode, h->v[a], h->v[b],
                         h->target, h->conf, h->bounds, p->lambda, p->step_size,
                         overwrite, halo, halo, h->stream, sp);
    if (st) return st;
    std::swap(a, b);
  }
  h->var_idx = a;
  return DTSGB_OK;
}

// num_iter X/Y box passes of the current v[src] with the sigma schedule of
// DomainTransformFilter::Filter; returns the index of the result buffer.
static int dts_filter_device(dtsgb_dts_t h, float sx, float sy, int num_iter,
                             int* result_idx) {
  int a = 0, b = 1;
  for (int it = 0; it < num_iter; ++it) {
    const float m = filter_sigma_multiplier(it, num_iter);
    const float six = sx * m, siy = sy * m;
    if (six >= 254.f || siy >= 254.f)
      return fail(DTSGB_ERR_UNSUPPORTED, "filter sigma must be below 254");
    int st = dts_bounds(h, six, siy, false);
    if (st) return st;
    st = launch_filter_pass(h->launch_i(), 1, h->v[a], nullptr, h->v[b], nullptr,
                            h->bounds, (int)std::floor(six), (int)std::floor(siy),
                            h->st, nullptr, 0.f, 0, h->stream);
    if (st) return st;
    std::swap(a, b);
  }
  *result_idx = a;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_filter(dtsgb_dts_t h, const dtsgb_filter_params* p,
                               const float* input, float* output, int num_iter) {
  if (!h || !p || !input || !output)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (num_iter < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "num_iter < 0");
  int st = check_filter_params(p->sigma_x, p->sigma_y, p->sigma_r);
  if (st) return st;
  const size_t wb = (size_t)h->w * 4;
  DTSGB_CUDA(cudaMemcpy2DAsync(h->v[0], (size_t)h->pitch * 4, input, wb, wb,
                               h->h, cudaMemcpyHostToDevice, h->stream));
  // Filter recomputes the DT with its own sigmas (filter.cu:128-129).
  h->ratio_x = p->sigma_x / p->sigma_r;
  h->ratio_y = p->sigma_y / p->sigma_r;
  h->diff_valid = true;
  h->bounds_valid = false;
  int res = 0;
  st = dts_filter_device(h, p->sigma_x, p->sigma_y, num_iter, &res);
  if (st) return st;
  if (res != 0)
    DTSGB_CUDA(cudaMemcpyAsync(h->v[0], h->v[res], h->plane * 4,
                               cudaMemcpyDeviceToDevice, h->stream));
  h->var_idx = 0;
  DTSGB_CUDA(cudaMemcpy2DAsync(output, wb, h->v[0], (size_t)h->pitch * 4, wb,
                               h->h, cudaMemcpyDeviceToHost, h->stream));
  DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_compute_confidence(dtsgb_dts_t h,
                                           const dtsgb_conf_params* p,
                                           int left_clear) {
  if (!h || !p) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  int st = check_filter_params(p->sigma_x, p->sigma_y, p->sigma_r);
  if (st) return st;
  if (!std::isfinite(p->sigmas[0]) || p->sigmas[0] == 0.f)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "sigmas[0] must be finite, nonzero");
  h->ratio_x = p->sigma_x / p->sigma_r;
  h->ratio_y = p->sigma_y / p->sigma_r;
  h->diff_valid = true;
  h->bounds_valid = false;
  // (v0, v1) = (t, t^2); three passes ping-pong between (v0,v1) and (v2,v3)
  st = launch_target_to_float(h->launch_i(), h->st, h->target, h->v[0], h->v[1],
                              h->stream);
  if (st) return st;
  const int kIters = 3;  // kNimDTFilterIteration, solver.cu:225
  const float scale = 0.5f / (p->sigmas[0] * p->sigmas[0]);
  int a = 0;
  for (int it = 0; it < kIters; ++it) {
    const float m = filter_sigma_multiplier(it, kIters);
    const float six = p->sigma_x * m, siy = p->sigma_y * m;
    if (six >= 254.f || siy >= 254.f)
      return fail(DTSGB_ERR_UNSUPPORTED, "filter sigma must be below 254");
    st = dts_bounds(h, six, siy, false);
    if (st) return st;
    const int b = 2 - a;
    const bool last = it == kIters - 1;
    st = launch_filter_pass(h->launch_i(), 2, h->v[a], h->v[a + 1], h->v[b],
                            h->v[b + 1], h->bounds, (int)std::floor(six),
                            (int)std::floor(siy), h->st, last ? h->conf : nullptr,
                            scale, left_clear, h->stream);
    if (st) return st;
    a = b;
  }
  // the reference leaves DT(t^2) in its var buffer
  h->var_idx = a + 1;
  return DTSGB_OK;
}

static int dts_download_impl(dtsgb_dts_t h, int type, void* dst,
                             cudaMemcpyKind kind) {
  if (!h || !dst) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  const bool filter_only = (h->flags & DTSGB_FLAG_FILTER_ONLY) != 0;
  const size_t fw = (size_t)h->w * 4, fp = (size_t)h->pitch * 4;
  const float* src = nullptr;
  int st = DTSGB_OK;
  switch (type) {
    case DTSGB_COLOR_IMAGE:
      DTSGB_CUDA(cudaMemcpy2DAsync(dst, fw, h->guide, fp, fw, h->h, kind,
                                   h->stream));
      break;
    case DTSGB_DIFFERENTIAL:
    case DTSGB_INTEGRAL:
      if (!h->diff_valid) {
        DTSGB_CUDA(cudaMemsetAsync(h->scr[0], 0, h->plane * 4, h->stream));
      } else {
        st = launch_differential(h->launch_i(), h->guide, h->ratio_x, 0,
                                 h->scr[0], h->stream);
        if (st) return st;
      }
      src = h->scr[0];
      if (type == DTSGB_INTEGRAL) {
        st = launch_row_prefix(&h->h_inst, h->d_inst, 1, h->scr[0], h->scr[1],
                               h->stream);
        if (st) return st;
        src = h->scr[1];
      }
      break;
    case DTSGB_TARGET:
    case DTSGB_CONFIDENCE:
      if (filter_only) return DTSGB_OK;
      if (h->st == Storage::F32) {
        src = (const float*)(type == DTSGB_TARGET ? h->target : h->conf);
      } else {
        st = launch_target_to_float(h->launch_i(), h->st,
                                    type == DTSGB_TARGET ? h->target : h->conf,
                                    h->scr[0], nullptr, h->stream);
        if (st) return st;
        src = h->scr[0];
      }
      break;
    case DTSGB_OPTIMIZED_QUANTITY:
      if (filter_only) return DTSGB_OK;
      if (h->var_idx < 0) {
        DTSGB_CUDA(cudaMemsetAsync(h->scr[0], 0, h->plane * 4, h->stream));
        src = h->scr[0];
      } else {
        src = h->v[h->var_idx];
      }
      break;
    default:
      return DTSGB_OK;  // the reference ignores other image types
  }
  if (src)
    DTSGB_CUDA(cudaMemcpy2DAsync(dst, fw, src, fp, fw, h->h, kind, h->stream));
  if (kind == cudaMemcpyDeviceToHost) DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_download(dtsgb_dts_t h, int type, void* image) {
  return dts_download_impl(h, type, image, cudaMemcpyDeviceToHost);
}

DTSGB_API int dtsgb_dts_download_device(dtsgb_dts_t h, int type, void* image) {
  return dts_download_impl(h, type, image, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_dts_clear_all(dtsgb_dts_t h) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  DTSGB_CUDA(cudaMemsetAsync(h->guide, 0, h->plane * 4, h->stream));
  DTSGB_CUDA(cudaMemsetAsync(h->target, 0, h->plane * h->tsize(), h->stream));
  DTSGB_CUDA(cudaMemsetAsync(h->conf, 0, h->plane * h->tsize(), h->stream));
  DTSGB_CUDA(cudaMemsetAsync(h->bounds, 0, h->plane * 4, h->stream));
  for (auto* p : h->v) DTSGB_CUDA(cudaMemsetAsync(p, 0, h->plane * 4, h->stream));
  h->diff_valid = false;
  h->bounds_valid = false;
  h->var_idx = -1;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_dts_debug_bounds(dtsgb_dts_t h, int axis, float sigma,
                                     int32_t* l, int32_t* u) {
  if (!h || !l || !u) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (axis != 0 && axis != 1) return fail(DTSGB_ERR_INVALID_ARGUMENT, "axis");
  if (!finite_pos(sigma) || sigma >= 254.f)
    return fail(DTSGB_ERR_UNSUPPORTED, "sigma must be in (0, 254)");
  int st = dts_bounds(h, sigma, sigma, false);
  if (st) return st;
  const size_t n = (size_t)h->w * h->h;
  int32_t* dl = (int32_t*)h->scr[0];
  int32_t* du = (int32_t*)h->scr[1];
  st = launch_unpack_bounds(h->launch_i(), h->bounds, axis, dl, du, h->stream);
  if (st) return st;
  DTSGB_CUDA(cudaMemcpyAsync(l, dl, n * 4, cudaMemcpyDeviceToHost, h->stream));
  DTSGB_CUDA(cudaMemcpyAsync(u, du, n * 4, cudaMemcpyDeviceToHost, h->stream));
  DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  h->bounds_valid = false;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_wait_timeouts(unsigned long long* count) {
  if (!count) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  *count = dts_wait_timeouts() + hfbs_wait_timeouts();
  return DTSGB_OK;
}

DTSGB_API int dtsgb_debug_color_convert(int cs, const void* in, void* out,
                                        long long n) {
  if (!in || !out || n < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "bad args");
  if (cs < DTSGB_RGB || cs > DTSGB_YYY)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid color space");
  uchar4* d = nullptr;
  int st = dalloc(&d, (size_t)n);
  if (st) return st;
  cudaError_t e = cudaMemcpy(d, in, (size_t)n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    st = launch_color_convert_flat(d, n, cs, 0);
    if (!st) e = cudaMemcpy(out, d, (size_t)n * 4, cudaMemcpyDeviceToHost);
  }
  cudaFree(d);
  if (st) return st;
  if (e != cudaSuccess) return cuda_fail(e, "debug_color_convert");
  return DTSGB_OK;
}

}  // extern "C"

// ===========================================================================
// HFBS handle
// ===========================================================================
struct dtsgb_hfbs_s {
  int max_w = 0, max_h = 0, pitch = 0, max_gx = 0, max_gy = 0, max_gl = 0;
  int w = 0, h = 0;
  unsigned flags = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  size_t plane = 0, gsize = 0;
  uchar4* guide = nullptr;
  float *target = nullptr, *conf = nullptr, *out = nullptr;
  float* g[16] = {};
  // tensor maps of the grid planes and the grid they describe
  TmaCache tma;
  HInst tma_inst{};
  float* ovf = nullptr;
  float2* sgrid = nullptr;  // (max_gx + 1) x (max_gy + 1) x (max_gl + 2)
  HInst* d_inst = nullptr;
  dtsgb_hfbs_params p{};
  int gx = 0, gy = 0, gl = 0;
  bool solved = false;
  // gradients (dtsgb_hfbs_enable_grad): the requested and the chosen
  // checkpoint segment, one arena for the kept iterates, the adjoint's grids
  // and three pixel planes (upstream gradient, dL/dtarget, dL/dconfidence)
  bool grad = false;
  int grad_seg_req = 0, grad_seg = 0, grad_planes = 0;
  float* gbuf = nullptr;
  size_t gbuf_cap = 0;  // floats
  float *gout = nullptr, *gtgt = nullptr, *gcnf = nullptr;
  HfbsGradState gs{};
  HInst inst{};
  bool grad_ready = false;  // the last optimize kept its iterates
  // guide-state reuse: the bistochastized normalisation depends only on the
  // guide's bins, so a solve whose guide (generation), grid and
  // bistochastization parameters equal the last one's keeps it
  struct NormKey {
    unsigned long long guide_gen;
    HInst inst;
    float sigma_x, sigma_y, sigma_l;
    int bistoch_iter_max;
  };
  unsigned long long guide_gen = 0;
  NormKey nkey{};
  bool nkey_valid = false;
};

enum {
  G_COUNT = 0, G_CSUM, G_B, G_N0, G_N1, G_INVA, G_Z0, G_Z1, G_H, G_T0, G_T1,
  G_T2, G_DBG_NORM, G_DBG_BLUR_C, G_DBG_Z_INIT, G_DBG_Z_FINAL, G_NUM
};

static void hfbs_free(dtsgb_hfbs_t h) {
  dfree(h->guide);
  dfree(h->target);
  dfree(h->conf);
  dfree(h->out);
  for (auto& p : h->g) dfree(p);
  dfree(h->ovf);
  dfree(h->sgrid);
  dfree(h->d_inst);
  dfree(h->gbuf);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  h->stream = nullptr;
}

// The single-instance batch of a handle (instance table already on the device).
static void hfbs_fill_batch(dtsgb_hfbs_t h, const HInst* hi, HfbsBatch& B) {
  const HInst& I = *hi;
  B.d_inst = h->d_inst;
  B.h_inst = hi;
  B.n_inst = 1;
  B.max_voxels = (long long)I.gx * I.gy * I.gl;
  // grid rows of px voxels; planes (and the kept iterates carved from one
  // arena) start every 32 voxels, as in a batch, so that every grid row
  // starts on a 16-byte boundary
  B.total_voxels = round_up_ll((long long)I.px * I.gy * I.gl, 32);
  B.max_pixels = (long long)I.w * I.h;
  B.max_cells = (long long)I.gx * I.gy;
  B.max_rows = (long long)I.gy * I.gl;
  B.max_lines = std::max({(long long)I.gy * I.gl, (long long)I.gx * I.gl,
                          (long long)I.gx * I.gy});
  B.max_gl = I.gl;
  B.guide = h->guide;
  B.target = h->target;
  B.conf = h->conf;
  B.st = Storage::F32;
  B.out = h->out;
  B.count = h->g[G_COUNT];
  B.csum = h->g[G_CSUM];
  B.b = h->g[G_B];
  B.n0 = h->g[G_N0];
  B.n1 = h->g[G_N1];
  B.invA = h->g[G_INVA];
  B.z0 = h->g[G_Z0];
  B.z1 = h->g[G_Z1];
  B.h = h->g[G_H];
  B.t0 = h->g[G_T0];
  B.t1 = h->g[G_T1];
  B.t2 = h->g[G_T2];
  B.sgrid = h->sgrid;
  B.ovf = h->ovf;
  B.keep_debug = true;
  B.grid_bytes = (size_t)I.px * I.gy * I.gl * 4;  // pitched
  B.dbg_norm = h->g[G_DBG_NORM];
  B.dbg_blur_c = h->g[G_DBG_BLUR_C];
  B.dbg_z_init = h->g[G_DBG_Z_INIT];
  B.dbg_z_final = h->g[G_DBG_Z_FINAL];
}

// Carve the gradient arena for K heavy-ball steps over tv voxels: the kept
// iterates and the adjoint's grids (hfbs_grad_planes) and three pixel planes.
// Segment 0 (automatic): every iterate when that fits in a quarter of the
// free device memory (the arena already held counts as free), else about
// sqrt(K) steps per segment.
static int hfbs_prepare_grad(dtsgb_hfbs_t h, int K, long long tv) {
  const long long pix = 3 * (long long)h->plane;
  int S = h->grad_seg_req;
  if (K <= 1) S = 1;
  if (S <= 0 && h->grad_seg == 1 &&
      h->gbuf_cap >= (size_t)(hfbs_grad_planes(K, 1) * tv + pix))
    S = 1;  // every iterate already held: no memory query
  if (S <= 0) {
    size_t fr = 0, tot = 0;
    DTSGB_CUDA(cudaMemGetInfo(&fr, &tot));
    const double avail = (double)fr + (double)h->gbuf_cap * 4.0;
    const double need1 = ((double)hfbs_grad_planes(K, 1) * tv + pix) * 4.0;
    S = need1 <= avail / 4 ? 1 : std::max(2, (int)std::ceil(std::sqrt((double)K)));
  }
  S = std::min(S, std::max(K, 1));
  const long long need = hfbs_grad_planes(K, S) * tv + pix;
  if ((size_t)need > h->gbuf_cap) {
    DTSGB_CUDA(cudaStreamSynchronize(h->stream));  // a backward may still read it
    dfree(h->gbuf);
    h->gbuf_cap = 0;
    int st = dalloc(&h->gbuf, (size_t)need);
    if (st) return st;
    h->gbuf_cap = (size_t)need;
  }
  float* q = h->gbuf;
  hfbs_carve_grad(h->gs, q, K, S, tv);
  q += hfbs_grad_planes(K, S) * tv;
  h->gout = q;
  h->gtgt = q + h->plane;
  h->gcnf = q + 2 * h->plane;
  h->grad_seg = S;
  h->grad_planes = (int)hfbs_grad_planes(K, S);
  return DTSGB_OK;
}

extern "C" {

DTSGB_API int dtsgb_hfbs_create(int max_w, int max_h, int max_gx, int max_gy,
                                int max_gl, unsigned flags, dtsgb_hfbs_t* out) {
  if (!out) return fail(DTSGB_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  if (max_w <= 0 || max_h <= 0 || max_gx <= 0 || max_gy <= 0 || max_gl <= 0)
    return fail(DTSGB_ERR_INVALID_DIMS, "max dims must be positive");
  dtsgb_hfbs_t h = new dtsgb_hfbs_s();
  h->max_w = h->w = max_w;
  h->max_h = h->h = max_h;
  h->pitch = round_up(max_w, 32);
  h->max_gx = max_gx;
  h->max_gy = max_gy;
  h->max_gl = max_gl;
  h->flags = flags;
  h->plane = (size_t)h->pitch * max_h;
  h->gsize = (size_t)round_up_ll((long long)round_up(max_gx, 4) * max_gy * max_gl, 32);
  // HFBSGridParams defaults, src/hfbs.h:18-60
  h->p = dtsgb_hfbs_params{8.f, 8.f, 4.f, 8.f, 1.f, 0.9f, 20, 140, 0.9f, 1, 1, 1};
  int st = DTSGB_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "cudaStreamCreate");
  }
  h->own_stream = true;
  if (!st) st = dalloc(&h->guide, h->plane);
  if (!st) st = dalloc(&h->target, h->plane);
  if (!st) st = dalloc(&h->conf, h->plane);
  if (!st) st = dalloc(&h->out, h->plane);
  for (int i = 0; i < G_NUM && !st; ++i) st = dalloc(&h->g[i], h->gsize);
  if (!st) st = dalloc(&h->ovf, (size_t)max_gx * max_gy);
  if (!st)
    st = dalloc(&h->sgrid, (size_t)(max_gx + 1) * (max_gy + 1) * (max_gl + 2));
  if (!st) st = dalloc(&h->d_inst, 1);
  if (st) {
    if (g_last_error.find("memory") != std::string::npos)
      st = DTSGB_ERR_OUT_OF_MEMORY;
    hfbs_free(h);
    delete h;
    return st;
  }
  *out = h;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_destroy(dtsgb_hfbs_t h) {
  if (!h) return DTSGB_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  hfbs_free(h);
  delete h;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_set_stream(dtsgb_hfbs_t h, void* stream) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->own_stream = false;
  h->stream = (cudaStream_t)stream;
  if (!stream) {
    DTSGB_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
  }
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_synchronize(dtsgb_hfbs_t h) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_set_image_dim(dtsgb_hfbs_t h, int w, int hh) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  // src/hfbs.cu:527-538 only guards against dims above the allocation
  if (w <= 0 || hh <= 0 || w > h->max_w || hh > h->max_h)
    return fail(DTSGB_ERR_INVALID_DIMS,
                "Image size is more than the reserved Cuda memory in constructor.");
  h->w = w;
  h->h = hh;
  h->grad_ready = false;
  ++h->guide_gen;
  return DTSGB_OK;
}

static int hfbs_init_frame(dtsgb_hfbs_t h, int cs, const void* rgba,
                           const float* target, const float* conf,
                           cudaMemcpyKind kind) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if (!rgba || !target)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "color image / target is null");
  if (cs < DTSGB_RGB || cs > DTSGB_YYY)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid color space");
  const size_t wb = (size_t)h->w * 4, pb = (size_t)h->pitch * 4;
  DTSGB_CUDA(cudaMemcpy2DAsync(h->guide, pb, rgba, wb, wb, h->h, kind, h->stream));
  int st = launch_color_convert_flat(h->guide, (long long)h->pitch * h->h, cs,
                                     h->stream);
  if (st) return st;
  DTSGB_CUDA(cudaMemcpy2DAsync(h->target, pb, target, wb, wb, h->h, kind,
                               h->stream));
  if (conf) {
    DTSGB_CUDA(cudaMemcpy2DAsync(h->conf, pb, conf, wb, wb, h->h, kind,
                                 h->stream));
  } else {
    st = launch_fill_storage(Storage::F32, h->conf, (long long)h->plane, 1.f,
                             h->stream);
    if (st) return st;
  }
  h->grad_ready = false;
  ++h->guide_gen;
  if (kind == cudaMemcpyHostToDevice) DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

// A new target and confidence for the guide already in place: the next
// Optimize with the same grid parameters keeps the bistochastized
// normalisation (results equal InitFrame with the same guide).
static int hfbs_upload_targets(dtsgb_hfbs_t h, const float* target, const float* conf,
                               cudaMemcpyKind kind) {
  if (!h || !target) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  const size_t wb = (size_t)h->w * 4, pb = (size_t)h->pitch * 4;
  DTSGB_CUDA(cudaMemcpy2DAsync(h->target, pb, target, wb, wb, h->h, kind, h->stream));
  if (conf) {
    DTSGB_CUDA(cudaMemcpy2DAsync(h->conf, pb, conf, wb, wb, h->h, kind, h->stream));
  } else {
    int st = launch_fill_storage(Storage::F32, h->conf, (long long)h->plane, 1.f,
                                 h->stream);
    if (st) return st;
  }
  h->grad_ready = false;
  if (kind == cudaMemcpyHostToDevice) DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_upload_targets(dtsgb_hfbs_t h, const float* target,
                                        const float* conf) {
  return hfbs_upload_targets(h, target, conf, cudaMemcpyHostToDevice);
}

DTSGB_API int dtsgb_hfbs_upload_targets_device(dtsgb_hfbs_t h, const float* target,
                                               const float* conf) {
  return hfbs_upload_targets(h, target, conf, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_hfbs_init_frame(dtsgb_hfbs_t h, int cs, const void* rgba,
                                    const float* target, const float* conf) {
  return hfbs_init_frame(h, cs, rgba, target, conf, cudaMemcpyHostToDevice);
}

DTSGB_API int dtsgb_hfbs_init_frame_device(dtsgb_hfbs_t h, int cs,
                                           const void* rgba, const float* target,
                                           const float* conf) {
  return hfbs_init_frame(h, cs, rgba, target, conf, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_hfbs_set_filter_params(dtsgb_hfbs_t h,
                                           const dtsgb_hfbs_params* p) {
  if (!h || !p) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  h->p = *p;
  h->grad_ready = false;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_clear_all(dtsgb_hfbs_t h) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  DTSGB_CUDA(cudaMemsetAsync(h->guide, 0, h->plane * 4, h->stream));
  DTSGB_CUDA(cudaMemsetAsync(h->target, 0, h->plane * 4, h->stream));
  DTSGB_CUDA(cudaMemsetAsync(h->conf, 0, h->plane * 4, h->stream));
  DTSGB_CUDA(cudaMemsetAsync(h->out, 0, h->plane * 4, h->stream));
  for (auto* p : h->g) DTSGB_CUDA(cudaMemsetAsync(p, 0, h->gsize * 4, h->stream));
  DTSGB_CUDA(cudaMemsetAsync(h->ovf, 0, (size_t)h->max_gx * h->max_gy * 4,
                             h->stream));
  h->solved = false;
  h->grad_ready = false;
  ++h->guide_gen;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_optimize(dtsgb_hfbs_t h) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  dtsgb_hfbs_params& p = h->p;
  if (!finite_pos(p.sigma_x) || !finite_pos(p.sigma_y) || !finite_pos(p.sigma_l))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "grid sigmas must be finite, positive");
  if (p.bistoch_iter_max < 0 || p.optim_iter_max < 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "iteration counts must be >= 0");
  // grid size, src/hfbs.cu:589-591
  p.grid_x = (int)std::ceil((float)h->w / p.sigma_x);
  p.grid_y = (int)std::ceil((float)h->h / p.sigma_y);
  p.grid_l = (int)std::ceil(255.0 / (double)p.sigma_l);
  h->gx = p.grid_x;
  h->gy = p.grid_y;
  h->gl = p.grid_l;
  h->solved = false;
  const bool had_norm = h->nkey_valid;
  h->nkey_valid = false;
  if (p.grid_x > h->max_gx || p.grid_y > h->max_gy || p.grid_l > h->max_gl) {
    // src/hfbs.cu:594-611: the target becomes the output
    const size_t pb = (size_t)h->pitch * 4;
    DTSGB_CUDA(cudaMemcpy2DAsync(h->out, pb, h->target, pb, (size_t)h->w * 4,
                                 h->h, cudaMemcpyDeviceToDevice, h->stream));
    return fail(DTSGB_WARN_GRID_TOO_LARGE,
                "Trying to use too large a bilateral space. Increase the blur "
                "sigmas or allocate more memory via constructor.");
  }
  if (p.grid_l > 256)
    return fail(DTSGB_ERR_UNSUPPORTED, "more than 256 luma bins (sigma_l < 1)");
  HInst I{};
  I.w = h->w;
  I.h = h->h;
  I.pitch = h->pitch;
  I.gx = p.grid_x;
  I.gy = p.grid_y;
  I.gl = p.grid_l;
  I.px = round_up(I.gx, 4);
  I.cov_x = (I.gx % 8 != 0) && (I.gx < h->max_gx);
  I.cov_y = (I.gy % 8 != 0) && (I.gy < h->max_gy);
  I.cov_l = (I.gl % 8 != 0) && (I.gl < h->max_gl);
  I.ovf_stored = I.gl < h->max_gl;
  I.pix_off = 0;
  I.grid_off = 0;
  I.plane_off = 0;
  I.slice_off = 0;
  DTSGB_CUDA(cudaMemcpyAsync(h->d_inst, &I, sizeof(HInst),
                             cudaMemcpyHostToDevice, h->stream));
  HfbsBatch B{};
  hfbs_fill_batch(h, &I, B);
  if (std::memcmp(&I, &h->tma_inst, sizeof I) != 0) {  // other grid: other tensor maps
    h->tma.clear();
    h->tma_inst = I;
  }
  B.tma = &h->tma;
  h->grad_ready = false;
  if (h->grad) {
    int gst = hfbs_prepare_grad(h, p.optim_iter_max, B.total_voxels);
    if (gst) return gst;
    B.grad = &h->gs;
  }
  HParams hp{p.sigma_x, p.sigma_y, p.sigma_l, p.lambda, p.alpha, p.beta,
             p.bistoch_iter_max, p.optim_iter_max, p.neg_exp_beta};
  dtsgb_hfbs_s::NormKey nk{};  // zero padding, so that memcmp compares fields
  nk.guide_gen = h->guide_gen;
  nk.inst = I;
  nk.sigma_x = p.sigma_x;
  nk.sigma_y = p.sigma_y;
  nk.sigma_l = p.sigma_l;
  nk.bistoch_iter_max = p.bistoch_iter_max;
  B.reuse_norm = had_norm && std::memcmp(&nk, &h->nkey, sizeof nk) == 0;
  int st = hfbs_enqueue_solve(B, hp, h->stream);
  if (st) return st;
  h->nkey = nk;
  h->nkey_valid = true;
  h->inst = I;
  h->solved = true;
  h->grad_ready = h->grad;
  return DTSGB_OK;
}

static int hfbs_download_impl(dtsgb_hfbs_t h, int type, float* dst,
                              cudaMemcpyKind kind) {
  if (!h || !dst) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  const float* src = nullptr;
  switch (type) {
    case DTSGB_TARGET: src = h->target; break;
    case DTSGB_CONFIDENCE: src = h->conf; break;
    case DTSGB_OPTIMIZED_QUANTITY: src = h->out; break;
    default: return DTSGB_OK;  // the reference ignores other types
  }
  const size_t wb = (size_t)h->w * 4, pb = (size_t)h->pitch * 4;
  DTSGB_CUDA(cudaMemcpy2DAsync(dst, wb, src, pb, wb, h->h, kind, h->stream));
  if (kind == cudaMemcpyDeviceToHost) DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_download(dtsgb_hfbs_t h, int type, float* image) {
  return hfbs_download_impl(h, type, image, cudaMemcpyDeviceToHost);
}

DTSGB_API int dtsgb_hfbs_download_device(dtsgb_hfbs_t h, int type,
                                         float* image) {
  return hfbs_download_impl(h, type, image, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_hfbs_grid_dims(dtsgb_hfbs_t h, int* gx, int* gy, int* gl) {
  if (!h || !gx || !gy || !gl) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null");
  *gx = h->gx;
  *gy = h->gy;
  *gl = h->gl;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_debug_grid(dtsgb_hfbs_t h, int which, float* dst) {
  if (!h || !dst) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  static const int map[8] = {G_COUNT,      G_CSUM,       G_B,
                             G_DBG_NORM,   G_INVA,       G_DBG_BLUR_C,
                             G_DBG_Z_INIT, G_DBG_Z_FINAL};
  if (which < 0 || which >= 8) return fail(DTSGB_ERR_INVALID_ARGUMENT, "which");
  if (!h->solved) return fail(DTSGB_ERR_INVALID_ARGUMENT, "no solve yet");
  // rows of round_up(gx, 4) voxels on the device, of gx in dst
  DTSGB_CUDA(cudaMemcpy2DAsync(dst, (size_t)h->gx * 4, h->g[map[which]],
                               (size_t)round_up(h->gx, 4) * 4, (size_t)h->gx * 4,
                               (size_t)h->gy * h->gl, cudaMemcpyDeviceToHost, h->stream));
  DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_enable_grad(dtsgb_hfbs_t h, int enable, int segment) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if (segment < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "segment must be >= 0");
  h->grad = enable != 0;
  h->grad_seg_req = segment;
  h->grad_ready = false;
  if (!h->grad) {
    DTSGB_CUDA(cudaStreamSynchronize(h->stream));
    dfree(h->gbuf);
    h->gbuf_cap = 0;
    h->grad_seg = h->grad_planes = 0;
  }
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_grad_info(dtsgb_hfbs_t h, int* segment, int* planes) {
  if (!h) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if (segment) *segment = h->grad_seg;
  if (planes) *planes = h->grad_planes;
  return DTSGB_OK;
}

static int hfbs_backward_impl(dtsgb_hfbs_t h, const float* grad_out, float* grad_target,
                              float* grad_confidence, cudaMemcpyKind up,
                              cudaMemcpyKind down) {
  if (!h || !grad_out) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (!h->grad_ready)
    return fail(DTSGB_ERR_INVALID_ARGUMENT,
                "no optimize with gradients enabled since the last change of frame, "
                "dims or parameters");
  const size_t wb = (size_t)h->w * 4, pb = (size_t)h->pitch * 4;
  DTSGB_CUDA(cudaMemcpy2DAsync(h->gout, pb, grad_out, wb, wb, h->h, up, h->stream));
  HfbsBatch B{};
  hfbs_fill_batch(h, &h->inst, B);
  B.grad = &h->gs;
  const dtsgb_hfbs_params& p = h->p;
  HParams hp{p.sigma_x, p.sigma_y, p.sigma_l, p.lambda, p.alpha, p.beta,
             p.bistoch_iter_max, p.optim_iter_max, p.neg_exp_beta};
  int st = hfbs_enqueue_backward(B, hp, h->gout, grad_target ? h->gtgt : nullptr,
                                 grad_confidence ? h->gcnf : nullptr, h->stream);
  if (st) return st;
  if (grad_target)
    DTSGB_CUDA(cudaMemcpy2DAsync(grad_target, wb, h->gtgt, pb, wb, h->h, down, h->stream));
  if (grad_confidence)
    DTSGB_CUDA(cudaMemcpy2DAsync(grad_confidence, wb, h->gcnf, pb, wb, h->h, down,
                                 h->stream));
  if (down == cudaMemcpyDeviceToHost) DTSGB_CUDA(cudaStreamSynchronize(h->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_hfbs_backward(dtsgb_hfbs_t h, const float* grad_out, float* grad_target,
                                  float* grad_confidence) {
  return hfbs_backward_impl(h, grad_out, grad_target, grad_confidence,
                            cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost);
}

DTSGB_API int dtsgb_hfbs_backward_device(dtsgb_hfbs_t h, const float* grad_out,
                                         float* grad_target, float* grad_confidence) {
  return hfbs_backward_impl(h, grad_out, grad_target, grad_confidence,
                            cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice);
}

}  // extern "C"
