// C++ facade of libdtsgb with the reference's API: the types and classes of
// akashbapat/domain_transform_solver (namespace domain_transform) as thin
// header-only wrappers over the C ABI in dtsgb.h.  Code written against
//   src/domain_transform_common.h, src/domain_transform_filter_params.h,
//   src/domain_transform_optimize.h, src/domain_transform_filter.h,
//   src/domain_transform_solver.h, src/hfbs.h, src/edge_aware_solver.h
// compiles against this header and links -ldtsgb instead.
//
// Error behaviour follows the reference: an invalid SetImageDim is reported on
// stderr and ignored; a CUDA failure is reported and ends the process with
// std::exit (the reference's GPU_CHECK).  Define DTSGB_FACADE_THROW before
// including this header to get std::runtime_error instead of the exit.
// EdgeAwareOptimize takes raw host buffers instead of cv::Mat.
#ifndef DOMAIN_TRANSFORM_GB300_HPP_
#define DOMAIN_TRANSFORM_GB300_HPP_

#include <chrono>
#include <cstdlib>
#include <iostream>
#include <stdexcept>
#include <string>

#include "dtsgb.h"

namespace domain_transform {

// ---- src/domain_transform_common.h ----------------------------------------
struct ImageDim {
  int width = 100;
  int height = 200;
  ImageDim Transpose() const {
    ImageDim d;
    d.width = height;
    d.height = width;
    return d;
  }
};
enum class ImageType { COLOR_IMAGE, DIFFERENTIAL, INTEGRAL, TARGET, CONFIDENCE,
                       OPTIMIZED_QUANTITY, TEST };
enum class COLOR_SPACE { RGB, YCbCr, YYY };

// ---- src/domain_transform_filter_params.h ----------------------------------
template <int N>
struct DomainFilterParamsVec {
  float sigma_x;
  float sigma_y;
  float sigma_r;
  float sigmas[N + 1];
  std::string ToString() const {
    std::string s = "DomainFilterParamsVec<" + std::to_string(N) + ">:\n";
    s += "sigma_x = " + std::to_string(sigma_x) + "\n";
    s += "sigma_y = " + std::to_string(sigma_y) + "\n";
    s += "sigma_r = " + std::to_string(sigma_r) + "\n";
    for (int i = 0; i < N; i++)
      s += "sigmas[" + std::to_string(i) + "] = " + std::to_string(sigmas[i]) + "\n";
    return s;
  }
};
using DomainFilterParams = DomainFilterParamsVec<0>;

// ---- src/domain_transform_optimize.h ---------------------------------------
enum class RobustLoss { L1, L2, CHARBONNIER };
inline std::string RobustLossToString(const RobustLoss& loss) {
  switch (loss) {
    case RobustLoss::L2: return "RobustLoss::L2";
    case RobustLoss::L1: return "RobustLoss::L1";
    default: return "RobustLoss::CHARBONNIER";
  }
}
struct DomainOptimizeParams {
  int num_iterations = 3;
  RobustLoss loss = RobustLoss::L2;
  float lambda = 1.0f;
  float sigma_z = 100;
  float step_size = 0.99;
  float photo_consis_lambda = 1.0f;
  float DT_lambda = 0.2f;
};

// ---- src/hfbs.h --------------------------------------------------------------
struct HFBSGridParams {
  float sigma_x = 8.0f;
  float sigma_y = 8.0f;
  float sigma_l = 4.0f;
  float lambda = 8.0f;
  float alpha = 1.0f;
  float beta = 0.9f;
  int bistoch_iter_max = 20;
  int optim_iter_max = 140;
  float neg_exp_beta = 0.9;
  int grid_x = 1;
  int grid_y = 1;
  int grid_l = 1;
};

namespace detail {
inline void on_status(int status, bool continue_on_dims = false) {
  if (status == DTSGB_OK) return;
  const std::string msg = dtsgb_last_error();
  std::cerr << msg << std::endl;
  if (status >= 100) return;  // warnings (HFBS grid too large)
  if (continue_on_dims && status == DTSGB_ERR_INVALID_DIMS) return;
#ifdef DTSGB_FACADE_THROW
  throw std::runtime_error(msg);
#else
  std::exit(status);
#endif
}
inline dtsgb_filter_params to_c(const DomainFilterParams& p) {
  return dtsgb_filter_params{p.sigma_x, p.sigma_y, p.sigma_r};
}
}  // namespace detail

// ---- src/domain_transform_filter.h -----------------------------------------
class DomainTransformFilter {
 public:
  explicit DomainTransformFilter(const ImageDim& max_image_dims)
      : DomainTransformFilter(max_image_dims, DTSGB_FLAG_FILTER_ONLY) {}
  virtual ~DomainTransformFilter() { dtsgb_dts_destroy(h_); }
  DomainTransformFilter(const DomainTransformFilter&) = delete;
  DomainTransformFilter& operator=(const DomainTransformFilter&) = delete;

  virtual void SetImageDim(const ImageDim& image_dim) {
    const int st = dtsgb_dts_set_image_dim(h_, image_dim.width, image_dim.height);
    if (st == DTSGB_OK) image_dims_ = image_dim;
    detail::on_status(st, true);
  }
  void InitFrame(const COLOR_SPACE& color_space, void* color_image) {
    detail::on_status(dtsgb_dts_init_frame(h_, static_cast<int>(color_space),
                                           color_image, nullptr, nullptr));
  }
  void Filter(const DomainFilterParams& filter_params, const float* input,
              float* output, const int num_iter = 3) {
    const dtsgb_filter_params p = detail::to_c(filter_params);
    detail::on_status(dtsgb_dts_filter(h_, &p, input, output, num_iter));
  }
  virtual void Download(const ImageType& image_type, void* image) const {
    detail::on_status(dtsgb_dts_download(h_, static_cast<int>(image_type), image));
  }
  void ClearAll() { detail::on_status(dtsgb_dts_clear_all(h_)); }
  void ComputeColorSpaceDifferential(const DomainFilterParams& domain_filter_params) {
    const dtsgb_filter_params p = detail::to_c(domain_filter_params);
    detail::on_status(dtsgb_dts_compute_differential(h_, &p));
  }
  void IntegrateColorDifferentials() { detail::on_status(dtsgb_dts_integrate(h_)); }
  // (new) CUDA stream for this object's work; nullptr = its own stream.
  void SetStream(void* cuda_stream) {
    detail::on_status(dtsgb_dts_set_stream(h_, cuda_stream));
  }
  dtsgb_dts_t handle() const { return h_; }

 protected:
  DomainTransformFilter(const ImageDim& max_image_dims, unsigned flags)
      : max_image_dims_(max_image_dims), image_dims_(max_image_dims) {
    detail::on_status(dtsgb_dts_create(max_image_dims.width, max_image_dims.height,
                                       flags, &h_));
  }
  dtsgb_dts_t h_ = nullptr;
  ImageDim max_image_dims_;
  ImageDim image_dims_;
};

// ---- src/domain_transform_solver.h -----------------------------------------
class DomainTransformSolver : public DomainTransformFilter {
 public:
  explicit DomainTransformSolver(const ImageDim& max_image_dims, unsigned flags = 0)
      : DomainTransformFilter(max_image_dims, flags & ~DTSGB_FLAG_FILTER_ONLY) {}
  // Guide-state reuse (extension): a new target / confidence for the guide
  // in place; the next Optimize with the same sigma_z keeps its windows.
  void UploadTargets(const float* target, const float* confidence = nullptr) {
    detail::on_status(dtsgb_dts_upload_targets(h_, target, confidence));
  }
  void InitFrame(const COLOR_SPACE& color_space, void* color_image, float* target,
                 float* confidence = nullptr) {
    detail::on_status(dtsgb_dts_init_frame(h_, static_cast<int>(color_space),
                                           color_image, target, confidence));
  }
  void ComputeColorSpaceDifferential(const DomainFilterParams& filter_params) {
    filter_params_ = filter_params;
    DomainTransformFilter::ComputeColorSpaceDifferential(filter_params);
  }
  void IntegrateColorDifferentials() { DomainTransformFilter::IntegrateColorDifferentials(); }
  virtual void Optimize(const DomainOptimizeParams& optimize_params,
                        const float overwrite_target_above_conf = -1) {
    const dtsgb_optimize_params p{optimize_params.num_iterations,
                                  static_cast<int>(optimize_params.loss),
                                  optimize_params.lambda, optimize_params.sigma_z,
                                  optimize_params.step_size,
                                  optimize_params.photo_consis_lambda,
                                  optimize_params.DT_lambda};
    detail::on_status(dtsgb_dts_optimize(h_, &p, overwrite_target_above_conf));
  }
  void Download(const ImageType& image_type, void* image) const override {
    detail::on_status(dtsgb_dts_download(h_, static_cast<int>(image_type), image));
  }
  void ComputeConfidence(const DomainFilterParamsVec<1>& conf_params,
                         const int left_side_clear_width) {
    const dtsgb_conf_params p{conf_params.sigma_x, conf_params.sigma_y,
                              conf_params.sigma_r,
                              {conf_params.sigmas[0], conf_params.sigmas[1]}};
    detail::on_status(dtsgb_dts_compute_confidence(h_, &p, left_side_clear_width));
  }
  void ClearAll() { DomainTransformFilter::ClearAll(); }

 protected:
  DomainFilterParams filter_params_{};
};

// ---- src/domain_transform_stereo.h:93-114 ------------------------------------
class DomainTransformStereo : public DomainTransformSolver {
 public:
  explicit DomainTransformStereo(const ImageDim& max_image_dims, unsigned flags = 0)
      : DomainTransformSolver(max_image_dims, flags | DTSGB_FLAG_STEREO) {}
  void InitRightFrame(const float center_offset, const COLOR_SPACE& color_space,
                      void* color_image) {
    detail::on_status(dtsgb_dts_init_right_frame(h_, center_offset,
                                                 static_cast<int>(color_space),
                                                 color_image));
  }
  // Always call this after ComputeColorSpaceDifferential().
  void ProcessRightFrame() { detail::on_status(dtsgb_dts_process_right_frame(h_)); }
  // Optimize (inherited) adds the photometric term on a stereo handle.
};

// ---- class HFBS, src/hfbs.h:99-150 -------------------------------------------
class HFBS {
 public:
  HFBS(const ImageDim& max_image_dims, const int max_grid_x, const int max_grid_y,
       const int max_grid_l) {
    detail::on_status(dtsgb_hfbs_create(max_image_dims.width, max_image_dims.height,
                                        max_grid_x, max_grid_y, max_grid_l, 0, &h_));
  }
  ~HFBS() { dtsgb_hfbs_destroy(h_); }
  HFBS(const HFBS&) = delete;
  HFBS& operator=(const HFBS&) = delete;

  void SetImageDim(const ImageDim& image_dim) {
    const int st = dtsgb_hfbs_set_image_dim(h_, image_dim.width, image_dim.height);
    if (st == DTSGB_OK) image_dim_ = image_dim;
    detail::on_status(st, true);
  }
  // Guide-state reuse (extension): a new target / confidence for the guide
  // in place; the next Optimize with the same grid keeps the normalisation.
  void UploadTargets(const float* target, const float* confidence = nullptr) {
    detail::on_status(dtsgb_hfbs_upload_targets(h_, target, confidence));
  }
  void InitFrame(const COLOR_SPACE& color_space, void* color_image, float* target,
                 float* confidence = nullptr) {
    detail::on_status(dtsgb_hfbs_init_frame(h_, static_cast<int>(color_space),
                                            color_image, target, confidence));
  }
  void SetFilterParams(const HFBSGridParams& grid_params) {
    grid_params_ = grid_params;
    const dtsgb_hfbs_params p{grid_params.sigma_x, grid_params.sigma_y,
                              grid_params.sigma_l, grid_params.lambda,
                              grid_params.alpha, grid_params.beta,
                              grid_params.bistoch_iter_max, grid_params.optim_iter_max,
                              grid_params.neg_exp_beta, grid_params.grid_x,
                              grid_params.grid_y, grid_params.grid_l};
    detail::on_status(dtsgb_hfbs_set_filter_params(h_, &p));
  }
  void ClearAll() { detail::on_status(dtsgb_hfbs_clear_all(h_)); }
  void Optimize() {
    detail::on_status(dtsgb_hfbs_optimize(h_));
    dtsgb_hfbs_grid_dims(h_, &grid_params_.grid_x, &grid_params_.grid_y,
                         &grid_params_.grid_l);
  }
  void Download(const ImageType& image_type, float* image) const {
    detail::on_status(dtsgb_hfbs_download(h_, static_cast<int>(image_type), image));
  }
  void SetStream(void* cuda_stream) {
    detail::on_status(dtsgb_hfbs_set_stream(h_, cuda_stream));
  }
  // Gradients (an addition: the reference has none; dtsgb_hfbs_enable_grad).
  // segment 0 chooses the checkpoint segment; Backward maps dL/d(output) of
  // the last Optimize to dL/dtarget and dL/dconfidence (either may be null).
  void EnableGrad(bool enable = true, int segment = 0) {
    detail::on_status(dtsgb_hfbs_enable_grad(h_, enable ? 1 : 0, segment));
  }
  void Backward(const float* grad_out, float* grad_target, float* grad_confidence) {
    detail::on_status(dtsgb_hfbs_backward(h_, grad_out, grad_target, grad_confidence));
  }
  dtsgb_hfbs_t handle() const { return h_; }

 protected:
  dtsgb_hfbs_t h_ = nullptr;
  ImageDim image_dim_;
  HFBSGridParams grid_params_;
};

// ---- src/edge_aware_solver.h (cv::Mat-free) ---------------------------------
struct DtsOptions {
  DomainFilterParams filter_options;
  DomainOptimizeParams optim_options;
  DomainFilterParamsVec<1> conf_params;
  COLOR_SPACE color_space;
  ImageDim image_dims;
  float overwrite_target_above_conf = -1;
};
struct HfbsOptions {
  HFBSGridParams grid_params;
  domain_transform::COLOR_SPACE color_space;
  ImageDim image_dims;
  float overwrite_target_above_conf = -1;
};

template <typename SolverOptions, typename SolverType>
void Solve(const SolverOptions& solver_options, const bool compute_confidence,
           SolverType* solver);

template <>
inline void Solve(const DtsOptions& solver_options, const bool compute_confidence,
                  DomainTransformSolver* solver) {
  solver->ComputeColorSpaceDifferential(solver_options.filter_options);
  solver->IntegrateColorDifferentials();
  if (compute_confidence) solver->ComputeConfidence(solver_options.conf_params, 0);
  solver->Optimize(solver_options.optim_options, solver_options.overwrite_target_above_conf);
}

template <>
inline void Solve(const HfbsOptions&, const bool, HFBS* solver) {
  solver->Optimize();
}

namespace detail {
inline void sync(DomainTransformSolver* s) { on_status(dtsgb_dts_synchronize(s->handle())); }
inline void sync(HFBS* s) { on_status(dtsgb_hfbs_synchronize(s->handle())); }
}  // namespace detail

// EdgeAwareOptimize without OpenCV: rgba W*H*4 bytes, target / confidence W*H
// floats (confidence may be null), optim_image W*H floats.  Returns the solve
// time in ms over the same window as the reference (after the upload, before
// the download), measured on the host between two synchronisations of the
// solver's stream.
template <typename SolverOptions, typename SolverType>
float EdgeAwareOptimize(const void* rgba_image, const float* target_image,
                        const float* confidence, const SolverOptions& solver_options,
                        SolverType* solver, float* optim_image) {
  solver->SetImageDim(solver_options.image_dims);
  solver->ClearAll();
  solver->InitFrame(solver_options.color_space, const_cast<void*>(rgba_image),
                    const_cast<float*>(target_image), const_cast<float*>(confidence));
  detail::sync(solver);
  const auto t0 = std::chrono::steady_clock::now();
  Solve(solver_options, confidence == nullptr, solver);
  detail::sync(solver);
  const auto t1 = std::chrono::steady_clock::now();
  solver->Download(ImageType::OPTIMIZED_QUANTITY, optim_image);
  return std::chrono::duration<float, std::milli>(t1 - t0).count();
}

}  // namespace domain_transform

#endif  // DOMAIN_TRANSFORM_GB300_HPP_
