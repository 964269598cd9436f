// Drop-in check of the C++ facade: the call sequence of the reference's
// tests/domain_transform_solver_test.cpp and tests/domain_transform_filter_test.cpp
// (InitFrame -> ComputeColorSpaceDifferential -> IntegrateColorDifferentials ->
// Optimize -> Download; Filter) and of an HFBS solve, on inputs read from raw
// files, written against domain_transform_gb300.hpp exactly as against the
// reference headers.
//   facade_solver_test <dir>   reads  dir/{rgba.bin,target.bin,conf.bin,dims.txt}
//                              writes dir/{dts.bin,filter.bin,hfbs.bin,color.bin}
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "domain_transform_gb300.hpp"

template <typename T>
static std::vector<T> read_all(const std::string& path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
  return v;
}

template <typename T>
static void write_all(const std::string& path, const std::vector<T>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

int main(int argc, char** argv) {
  using namespace domain_transform;
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  ImageDim dims;
  {
    std::ifstream f(dir + "/dims.txt");
    f >> dims.width >> dims.height;
  }
  const size_t n = (size_t)dims.width * dims.height;
  auto rgba = read_all<unsigned char>(dir + "/rgba.bin", n * 4);
  auto target = read_all<float>(dir + "/target.bin", n);
  auto conf = read_all<float>(dir + "/conf.bin", n);

  // solver, as in domain_transform_solver_test.cpp
  DomainTransformSolver solver(dims);
  solver.SetImageDim(dims);
  solver.ClearAll();
  solver.InitFrame(COLOR_SPACE::YCbCr, rgba.data(), target.data(), conf.data());
  DomainFilterParams fp;
  fp.sigma_x = 8;
  fp.sigma_y = 8;
  fp.sigma_r = 0.1f;
  solver.ComputeColorSpaceDifferential(fp);
  solver.IntegrateColorDifferentials();
  DomainOptimizeParams op;
  op.num_iterations = 10;
  op.lambda = 0.99f;
  op.sigma_z = 8;
  op.step_size = 0.99f;
  op.loss = RobustLoss::L2;
  solver.Optimize(op);
  std::vector<float> out(n);
  solver.Download(ImageType::OPTIMIZED_QUANTITY, out.data());
  write_all(dir + "/dts.bin", out);
  std::vector<unsigned char> color(n * 4);
  solver.Download(ImageType::COLOR_IMAGE, color.data());
  write_all(dir + "/color.bin", color);

  // filter, as in domain_transform_filter_test.cpp
  DomainTransformFilter filter(dims);
  filter.InitFrame(COLOR_SPACE::YCbCr, rgba.data());
  DomainFilterParams ffp;
  ffp.sigma_x = 8;
  ffp.sigma_y = 8;
  ffp.sigma_r = 0.2f;
  std::vector<float> filtered(n);
  filter.Filter(ffp, target.data(), filtered.data(), 5);
  write_all(dir + "/filter.bin", filtered);

  // HFBS through the generic solve API
  HFBS hfbs(dims, (dims.width + 7) / 8 + 1, (dims.height + 7) / 8 + 1, 17);
  HfbsOptions ho;
  ho.grid_params.sigma_l = 16;
  ho.grid_params.optim_iter_max = 20;
  ho.color_space = COLOR_SPACE::YCbCr;
  ho.image_dims = dims;
  hfbs.SetFilterParams(ho.grid_params);
  std::vector<float> hout(n);
  const float ms = EdgeAwareOptimize(rgba.data(), target.data(), conf.data(), ho, &hfbs,
                                     hout.data());
  write_all(dir + "/hfbs.bin", hout);
  // the HFBS adjoint through the facade (an addition): dL/d(output) = target
  hfbs.EnableGrad(true, 0);
  hfbs.Optimize();
  std::vector<float> hgt(n), hgc(n);
  hfbs.Backward(target.data(), hgt.data(), hgc.data());
  write_all(dir + "/hfbs_gt.bin", hgt);
  write_all(dir + "/hfbs_gc.bin", hgc);
  std::printf("facade ok: hfbs solve %.3f ms\n", ms);
  return 0;
}
