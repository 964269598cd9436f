// C entry points over the reference's own DTS / HFBS classes compiled for
// the CPU (build_ref.py) -- TEST INFRASTRUCTURE ONLY: they produce the
// golden vectors that pin the oracle and the GPU path to the reference.
//
// One translation unit holds the reference's sources (their headers define
// non-inline functions, so the reference itself is a single-TU build too).
// Each entry point follows the reference's call sequence for a solve
// (src/edge_aware_solver.h:59-90: SetImageDim, ClearAll, InitFrame, Solve,
// Download; Solve<DtsOptions> at :38-50) and reads intermediate state
// through the reference's own accessors (FilterStructPtr()) or, for HFBS,
// a subclass that reaches the protected implementation pointer.
#include "domain_transform_filter.cu"
#include "domain_transform_solver.cu"
#include "domain_transform_stereo.cu"
#include "hfbs.cu"
#include "error_types.cpp"

using namespace domain_transform;

namespace {

// The reference's row scan (src/domain_transform_common_functions.h:41-70)
// exits the process below 128 pixels; the transposed scans need the
// height to be that large too.
bool size_ok(int w, int h) { return w >= 128 && h >= 128; }

template <class C>
void download_plane(const C& a, int w, int h, float* dst, bool transposed) {
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x)
      dst[(size_t)y * w + x] = transposed ? a.get(y, x) : a.get(x, y);
}

struct HfbsProbe : HFBS {
  using HFBS::HFBS;
  HFBSImpl* impl() { return solver_impl_.get(); }
  const HFBSGridParams& params() const { return grid_params_; }
};

DomainFilterParams filter_params(float sx, float sy, float sr) {
  DomainFilterParams p;
  p.sigma_x = sx;
  p.sigma_y = sy;
  p.sigma_r = sr;
  return p;
}

}  // namespace

extern "C" {

// One DTS solve (Solve<DtsOptions>): differential, integration, optional
// confidence estimate (conf == nullptr, as EdgeAwareOptimize does), then
// Optimize.  Every output but `result` may be null.
//   color: the guide after InitFrame's colour conversion, w*h RGBA
//   dH, dV: the integrands; ctH, ctV: their integrals (ctV de-transposed)
//   conf_out: the confidence the solve used
//   bounds: 4 ints per pixel -- the X window (lower, upper) and the Y window,
//           from the reference's own LinearSearchLowerAndUpperBound2DX over
//           ct_H / ct_V with sigma_z, as OptimizeX / OptimizeY call it
int dtsref_dts_solve(int w, int h, int color_space, const unsigned char* rgba,
                     const float* target, const float* conf, float sx, float sy,
                     float sr, const float* conf_params /* sx, sy, sr, sigma0 */,
                     int num_iterations, int loss, float lambda, float sigma_z,
                     float step_size, float overwrite, float* result,
                     unsigned char* color, float* dH, float* dV, float* ctH,
                     float* ctV, float* conf_out, int* bounds) {
  if (!size_ok(w, h)) return -1;
  ImageDim dim;
  dim.width = w;
  dim.height = h;
  DomainTransformSolver solver(dim);
  solver.SetImageDim(dim);
  solver.ClearAll();
  std::vector<unsigned char> guide(rgba, rgba + (size_t)w * h * 4);
  std::vector<float> t(target, target + (size_t)w * h);
  std::vector<float> c;
  if (conf) c.assign(conf, conf + (size_t)w * h);
  solver.InitFrame(static_cast<COLOR_SPACE>(color_space), guide.data(), t.data(),
                   conf ? c.data() : nullptr);
  solver.ComputeColorSpaceDifferential(filter_params(sx, sy, sr));
  solver.IntegrateColorDifferentials();
  if (!conf) {
    DomainFilterParamsVec<1> cp;
    cp.sigma_x = conf_params[0];
    cp.sigma_y = conf_params[1];
    cp.sigma_r = conf_params[2];
    cp.sigmas[0] = conf_params[3];
    solver.ComputeConfidence(cp, 0);
  }
  DomainOptimizeParams op;
  op.num_iterations = num_iterations;
  op.loss = static_cast<RobustLoss>(loss);
  op.lambda = lambda;
  op.sigma_z = sigma_z;
  op.step_size = step_size;
  solver.Optimize(op, overwrite);
  solver.Download(ImageType::OPTIMIZED_QUANTITY, result);
  if (conf_out) solver.Download(ImageType::CONFIDENCE, conf_out);
  DomainTransformFilterStruct* fs = solver.FilterStructPtr();
  if (color) solver.Download(ImageType::COLOR_IMAGE, color);
  if (dH) download_plane(fs->dHdx, w, h, dH, false);
  if (dV) download_plane(fs->dVdy, w, h, dV, false);
  if (ctH) download_plane(fs->ct_H, w, h, ctH, false);
  if (ctV) download_plane(fs->ct_V, w, h, ctV, true);
  if (bounds) {
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        int* b = bounds + 4 * ((size_t)y * w + x);
        LinearSearchLowerAndUpperBound2DX(dim, &fs->ct_H, sigma_z, x, y, &b[0], &b[1]);
        LinearSearchLowerAndUpperBound2DX(dim, &fs->ct_V, sigma_z, y, x, &b[2], &b[3]);
      }
  }
  return 0;
}

// DomainTransformFilter::Filter on `input` (num_iter passes).  bounds
// (nullable) receives, per pass, 4 ints per pixel: the X and Y windows of
// that pass's sigmas (the schedule of src/domain_transform_filter.cu:142-152)
// from the reference's own search over ct_H / ct_V.
int dtsref_filter(int w, int h, int color_space, const unsigned char* rgba, float sx,
                  float sy, float sr, const float* input, int num_iter, float* output,
                  int* bounds) {
  if (!size_ok(w, h)) return -1;
  ImageDim dim;
  dim.width = w;
  dim.height = h;
  DomainTransformFilter filter(dim);
  filter.SetImageDim(dim);
  filter.ClearAll();
  std::vector<unsigned char> guide(rgba, rgba + (size_t)w * h * 4);
  filter.InitFrame(static_cast<COLOR_SPACE>(color_space), guide.data());
  filter.Filter(filter_params(sx, sy, sr), input, output, num_iter);
  if (bounds) {
    DomainTransformFilterStruct* fs = filter.FilterStructPtr();
    for (int it = 0; it < num_iter; ++it) {
      float sigma_x = sx, sigma_y = sy;
      if (it != 0) {
        const float multiplier =
            3 * std::pow(2, (num_iter - (it + 1))) / std::sqrt(std::pow(4, num_iter) - 1);
        sigma_x *= multiplier;
        sigma_y *= multiplier;
      }
      for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
          int* b = bounds + 4 * (((size_t)it * h + y) * w + x);
          LinearSearchLowerAndUpperBound2DX(dim, &fs->ct_H, sigma_x, x, y, &b[0], &b[1]);
          LinearSearchLowerAndUpperBound2DX(dim, &fs->ct_V, sigma_y, y, x, &b[2], &b[3]);
        }
    }
  }
  return 0;
}

// DomainTransformStereo: left guide, right guide at center_offset, then a
// solve with the photometric term (src/domain_transform_stereo.cu:43-160).
int dtsref_stereo_solve(int w, int h, int color_space, const unsigned char* left,
                        const unsigned char* right, float center_offset,
                        const float* target, const float* conf, float sx, float sy,
                        float sr, int num_iterations, int loss, float lambda,
                        float sigma_z, float step_size, float photo_lambda,
                        float dt_lambda, float* result) {
  if (!size_ok(w, h)) return -1;
  ImageDim dim;
  dim.width = w;
  dim.height = h;
  DomainTransformStereo solver(dim);
  solver.SetImageDim(dim);
  solver.ClearAll();
  std::vector<unsigned char> gl(left, left + (size_t)w * h * 4);
  std::vector<unsigned char> gr(right, right + (size_t)w * h * 4);
  std::vector<float> t(target, target + (size_t)w * h);
  std::vector<float> c(conf, conf + (size_t)w * h);
  solver.InitFrame(static_cast<COLOR_SPACE>(color_space), gl.data(), t.data(), c.data());
  solver.InitRightFrame(center_offset, static_cast<COLOR_SPACE>(color_space), gr.data());
  solver.ComputeColorSpaceDifferential(filter_params(sx, sy, sr));
  solver.IntegrateColorDifferentials();
  solver.ProcessRightFrame();
  DomainOptimizeParams op;
  op.num_iterations = num_iterations;
  op.loss = static_cast<RobustLoss>(loss);
  op.lambda = lambda;
  op.sigma_z = sigma_z;
  op.step_size = step_size;
  op.photo_consis_lambda = photo_lambda;
  op.DT_lambda = dt_lambda;
  solver.Optimize(op, -1);
  solver.Download(ImageType::OPTIMIZED_QUANTITY, result);
  return 0;
}

// HFBS::Optimize on a max_gx x max_gy x max_gl allocation.  `params` holds
// sigma_x, sigma_y, sigma_l, lambda, alpha, beta, neg_exp_beta (floats) and
// `iters` bistoch_iter_max, optim_iter_max.  grids (nullable) receives five
// max_gx*max_gy*max_gl planes, x fastest: splat_sum, splat_norm,
// inv_diag_A, b, z (the final solution); dims receives grid_x, grid_y,
// grid_l.  Returns 1 when the grid is too large (the target is copied).
int dtsref_hfbs_solve(int w, int h, int color_space, const unsigned char* rgba,
                      const float* target, const float* conf, const float* params,
                      const int* iters, int max_gx, int max_gy, int max_gl,
                      float* result, float* grids, int* dims) {
  ImageDim dim;
  dim.width = w;
  dim.height = h;
  HfbsProbe solver(dim, max_gx, max_gy, max_gl);
  HFBSGridParams gp;
  gp.sigma_x = params[0];
  gp.sigma_y = params[1];
  gp.sigma_l = params[2];
  gp.lambda = params[3];
  gp.alpha = params[4];
  gp.beta = params[5];
  gp.neg_exp_beta = params[6];
  gp.bistoch_iter_max = iters[0];
  gp.optim_iter_max = iters[1];
  solver.SetImageDim(dim);
  solver.SetFilterParams(gp);
  solver.ClearAll();
  std::vector<unsigned char> guide(rgba, rgba + (size_t)w * h * 4);
  std::vector<float> t(target, target + (size_t)w * h);
  std::vector<float> c;
  if (conf) c.assign(conf, conf + (size_t)w * h);
  solver.InitFrame(static_cast<COLOR_SPACE>(color_space), guide.data(), t.data(),
                   conf ? c.data() : nullptr);
  solver.Optimize();
  solver.Download(ImageType::OPTIMIZED_QUANTITY, result);
  const HFBSGridParams& used = solver.params();
  if (dims) {
    dims[0] = used.grid_x;
    dims[1] = used.grid_y;
    dims[2] = used.grid_l;
  }
  const bool too_large = used.grid_x > max_gx || used.grid_y > max_gy || used.grid_l > max_gl;
  if (grids && !too_large) {
    HFBS::HFBSImpl* s = solver.impl();
    const size_t plane = (size_t)max_gx * max_gy * max_gl;
    for (int z = 0; z < max_gl; ++z)
      for (int y = 0; y < max_gy; ++y)
        for (int x = 0; x < max_gx; ++x) {
          const size_t i = ((size_t)z * max_gy + y) * max_gx + x;
          grids[0 * plane + i] = s->splat_sum.get(x, y, z);
          grids[1 * plane + i] = s->splat_norm.get(x, y, z);
          grids[2 * plane + i] = s->inv_diag_A.get(x, y, z);
          grids[3 * plane + i] = s->b.get(x, y, z);
          grids[4 * plane + i] = s->z.get(x, y, z);
        }
  }
  return too_large ? 1 : 0;
}

// RGB2YCbCr / RGB2YYY (src/color_space.cuh) on n pixels, in place, as the
// reference's InitFrame launches them (32x32 blocks over a w x h image).
int dtsref_color_convert(int w, int h, int color_space, unsigned char* rgba) {
  ImageDim dim;
  dim.width = w;
  dim.height = h;
  cua::CudaSurface2D<uchar4> image(w, h);
  image = reinterpret_cast<const uchar4*>(rgba);
  dim3 block, grid;
  ComputeBlockAndGridDim2D<false>(dim, &block, &grid);
  if (color_space == static_cast<int>(COLOR_SPACE::YCbCr))
    ::refemu::launch(grid, block, [&]() { RGB2YCbCr(dim, image); });
  else if (color_space == static_cast<int>(COLOR_SPACE::YYY))
    ::refemu::launch(grid, block, [&]() { RGB2YYY(dim, image); });
  image.View(0, 0, w, h).CopyTo(reinterpret_cast<uchar4*>(rgba));
  return 0;
}

}  // extern "C"
