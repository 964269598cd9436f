// dtsgb_dts_solve_noalloc: one DTS solve (ComputeColorSpaceDifferential +
// IntegrateColorDifferentials + Optimize of DomainTransformSolver) for
// callers that cannot allocate device memory, such as code running inside
// another framework's CUDA-graph capture, real-time pipelines that forbid
// allocation after start-up, or hosts whose own allocator must own every
// cudaMalloc.  The caller passes device inputs and the device output; the
// solve's scratch (packed window bounds and one iterate buffer) lives in the
// file-scope array below, which every GPU that loads the library holds until
// the process exits.
//
// Contract (also in include/dtsgb.h):
//  * at most kNoAllocMaxPixels pixels per call; larger images are rejected;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress while that device is current, so make that first
//    call before any stream capture;
//  * every call on a device shares the one array and it keeps the previous
//    call's contents: calls that overlap on the GPU (other streams, other
//    host threads) race on it and must be serialised by the caller.  Nothing
//    in it needs to start at zero: every element a call reads is written
//    earlier in the same call;
//  * no cudaMalloc, cudaFree, stream creation or any allocating routine;
//  * sigma_z below DTSGB_NOALLOC_MAX_SIGMA_Z (the iteration's tile and halo
//    live in shared memory) and 4-byte aligned buffers;
//  * the array's address is cached per device ordinal: primary context
//    only, and not across cudaDeviceReset.
#include <cstdint>
#include <mutex>

#include "../../include/dtsgb.h"
#include "color.cuh"
#include "dtsgb_internal.cuh"

namespace dtsgb {
namespace {

constexpr long long kNoAllocMaxPixels = DTSGB_NOALLOC_MAX_PIXELS;
constexpr int kNaThreads = 256;
constexpr int kNaTile = 32;  // output tile of the bounds and iteration kernels

// bounds (u32 per pixel) followed by one f32 iterate plane
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocMaxPixels * 8];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

__device__ __forceinline__ uchar4 na_guide(const uchar4* g, int W, int x, int y,
                                           int cs) {
  return convert_pixel(g[(long long)y * W + x], cs);
}

// Window bounds from the caller's RGBA guide (converted on the fly), dense
// rows of width W; tile index from blockIdx.  Same search as the batched
// bounds kernel: lower = largest i < p with sum_{i+1..p} w > sigma (else
// p-1), upper = (smallest i > p, i < limit, with sum_{p+1..i} w > sigma) - 1
// (else p).
__global__ void __launch_bounds__(kNaThreads)
    k_na_bounds(const uchar4* __restrict__ guide, int W, int H, int cs,
                float ratio_x, float ratio_y, float sigma, int r,
                int ref_y_limit, uint32_t* __restrict__ bounds) {
  extern __shared__ float sm[];
  const int ntx = (W + kNaTile - 1) / kNaTile;
  const int x0 = (blockIdx.x % ntx) * kNaTile, y0 = (blockIdx.x / ntx) * kNaTile;
  const int DW = kNaTile + 2 * r - 1;
  float* sH = sm;
  float* sV = sm + kNaTile * DW;
  const uchar4 zero = make_uchar4(0, 0, 0, 0);
  for (int i = threadIdx.x; i < kNaTile * DW; i += blockDim.x) {
    const int rr = i / DW, c = i - rr * DW;
    const int x = x0 - r + 1 + c, y = y0 + rr;
    float w = 0.f;
    if (x >= 0 && x < W && y < H)
      w = edge_weight(na_guide(guide, W, x, y, cs),
                  x > 0 ? na_guide(guide, W, x - 1, y, cs) : zero, ratio_x);
    sH[i] = w;
  }
  for (int i = threadIdx.x; i < DW * kNaTile; i += blockDim.x) {
    const int rr = i / kNaTile, c = i - rr * kNaTile;
    const int x = x0 + c, y = y0 - r + 1 + rr;
    float w = 0.f;
    if (x < W && y >= 0 && y < H)
      w = edge_weight(na_guide(guide, W, x, y, cs),
                  y > 0 ? na_guide(guide, W, x, y - 1, cs) : zero, ratio_y);
    sV[i] = w;
  }
  __syncthreads();
  const int ylim = ref_y_limit ? min(W, H) : H;
  for (int i = threadIdx.x; i < kNaTile * kNaTile; i += blockDim.x) {
    const int rr = i / kNaTile, c = i - rr * kNaTile;
    const int x = x0 + c, y = y0 + rr;
    if (x >= W || y >= H) continue;
    const float* row = sH + rr * DW + (c + r - 1);
    const float* col = sV + (rr + r - 1) * kNaTile + c;
    int dlx = 1, dux = 0, dly = 1, duy = 0;
    float acc = 0.f;
    for (int k = 1; k <= r && x - k >= 0; ++k) {
      acc += row[1 - k];
      if (acc > sigma) { dlx = k; break; }
    }
    acc = 0.f;
    for (int k = 1; k <= r && x + k < W; ++k) {
      acc += row[k];
      if (acc > sigma) { dux = k - 1; break; }
    }
    acc = 0.f;
    for (int k = 1; k <= r && y - k >= 0; ++k) {
      acc += col[(1 - k) * kNaTile];
      if (acc > sigma) { dly = k; break; }
    }
    acc = 0.f;
    for (int k = 1; k <= r && y + k < ylim; ++k) {
      acc += col[k * kNaTile];
      if (acc > sigma) { duy = k - 1; break; }
    }
    bounds[(long long)y * W + x] = pack_bounds(dlx, dux, dly, duy);
  }
}

// One X+Y iteration over dense rows (src/domain_transform_solver.cuh:37-116),
// direct window sums over a tile + halo in shared memory; conf == nullptr
// means confidence 1 everywhere.
template <int MODE>
__global__ void __launch_bounds__(kNaThreads)
    k_na_iter(const float* __restrict__ vin, float* __restrict__ vout,
              const float* __restrict__ tgt, const float* __restrict__ cnf,
              const uint32_t* __restrict__ bnd, int W, int H, float lambda,
              float step, float overwrite, int hx) {
  extern __shared__ float sm[];
  const int ntx = (W + kNaTile - 1) / kNaTile;
  const int x0 = (blockIdx.x % ntx) * kNaTile, y0 = (blockIdx.x / ntx) * kNaTile;
  const int hy = hx;
  const int SW = kNaTile + 2 * hx, SR = kNaTile + 2 * hy;
  float* sv = sm;
  float* sx = sm + SR * SW;
  const bool over = overwrite > 0.f && overwrite < 1.f;
  for (int i = threadIdx.x; i < SR * SW; i += blockDim.x) {
    const int rr = i / SW, c = i - rr * SW;
    const int x = x0 - hx + c, y = y0 - hy + rr;
    float v = 0.f;
    if (x >= 0 && x < W && y >= 0 && y < H) {
      const long long p = (long long)y * W + x;
      v = vin[p];
      const float cv = cnf ? cnf[p] : 1.f;
      if (over && cv > overwrite) v = tgt[p];
    }
    sv[i] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < SR * kNaTile; i += blockDim.x) {
    const int rr = i / kNaTile, c = i - rr * kNaTile;
    const int x = x0 + c, y = y0 - hy + rr;
    float o = 0.f;
    if (x < W && y >= 0 && y < H) {
      const long long p = (long long)y * W + x;
      const uint32_t b = bnd[p];
      const int dl = min((int)(b & 0xff), hx + 1), du = min((int)((b >> 8) & 0xff), hx);
      const float* row = sv + rr * SW + c + hx;
      float s = 0.f;
      for (int k = 1 - dl; k <= du; ++k) s += row[k];
      const float nf = (float)(dl + du);
      const float v = row[0], tv = tgt[p], cv = cnf ? cnf[p] : 1.f;
      const float cn = __fdiv_rn(cv, nf), d = v - tv;
      const float g = MODE == 0 ? 2.f * cn * d
                                : __fdiv_rn(cn * d, __fsqrt_rn(__fmaf_rn(d, d, 1e-6f)));
      o = __fmaf_rn(step, -__fmaf_rn(lambda, v - __fdiv_rn(s, nf), 0.5f * g), v);
      if (over && cv > overwrite) o = tv;
    }
    sx[i] = o;
  }
  __syncthreads();
  const float slam = step * lambda;
  for (int i = threadIdx.x; i < kNaTile * kNaTile; i += blockDim.x) {
    const int rr = i / kNaTile, c = i - rr * kNaTile;
    const int x = x0 + c, y = y0 + rr;
    if (x >= W || y >= H) continue;
    const long long p = (long long)y * W + x;
    const uint32_t b = bnd[p];
    const int dl = min((int)((b >> 16) & 0xff), hy + 1), du = min((int)(b >> 24), hy);
    const float* col = sx + (rr + hy) * kNaTile + c;
    float s = 0.f;
    for (int k = 1 - dl; k <= du; ++k) s += col[k * kNaTile];
    const float v = col[0];
    vout[p] = __fmaf_rn(-slam, v - __fdiv_rn(s, (float)(dl + du)), v);
  }
}

int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  DTSGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(DTSGB_ERR_UNSUPPORTED, "device ordinal beyond the no-alloc table");
  std::lock_guard<std::mutex> g(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    DTSGB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_addr[dev] = p;
  }
  *out = (unsigned char*)g_scratch_addr[dev];
  return DTSGB_OK;
}

}  // namespace
}  // namespace dtsgb

using namespace dtsgb;

extern "C" DTSGB_API int dtsgb_dts_solve_noalloc(
    int width, int height, int color_space, const void* rgba, const float* target,
    const float* confidence, const dtsgb_filter_params* filter,
    const dtsgb_optimize_params* optimize, float overwrite, float* output,
    void* cuda_stream) {
  if (!rgba || !target || !output || !filter || !optimize)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (output == target || (const void*)output == (const void*)confidence)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "output must not alias an input");
  if (((uintptr_t)rgba | (uintptr_t)target | (uintptr_t)confidence | (uintptr_t)output) & 3)
    return fail(DTSGB_ERR_INVALID_ARGUMENT,
                "dtsgb_dts_solve_noalloc: rgba, target, confidence and output must be "
                "4-byte aligned");
  if (width <= 0 || height <= 0)
    return fail(DTSGB_ERR_INVALID_DIMS, "image dims must be positive");
  if ((long long)width * height > kNoAllocMaxPixels)
    return fail(DTSGB_ERR_UNSUPPORTED,
                "dtsgb_dts_solve_noalloc: image of " + std::to_string(width) + "x" +
                    std::to_string(height) + " pixels exceeds its static scratch of " +
                    std::to_string(kNoAllocMaxPixels) + " pixels");
  if (color_space < DTSGB_RGB || color_space > DTSGB_YYY)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid color space");
  if (!finite_pos(filter->sigma_x) || !finite_pos(filter->sigma_y) ||
      !finite_pos(filter->sigma_r))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "filter sigmas must be finite, positive");
  if (optimize->loss < DTSGB_L1 || optimize->loss > DTSGB_CHARBONNIER)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid loss");
  if (optimize->num_iterations < 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "num_iterations < 0");
  if (!finite_pos(optimize->sigma_z) || optimize->sigma_z >= DTSGB_NOALLOC_MAX_SIGMA_Z)
    return fail(DTSGB_ERR_UNSUPPORTED,
                "dtsgb_dts_solve_noalloc: sigma_z must be in (0, 97): its iteration tile "
                "of (32 + 2h) x (64 + 2h) floats, h = floor(sigma_z), must fit in 227 KiB "
                "of shared memory (the allocating entry points take sigma_z below 254)");
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const long long n = (long long)width * height;
  // RobustLoss::L1 runs no kernel in the reference: the result is the target
  if (optimize->loss == DTSGB_L1 || optimize->num_iterations == 0) {
    DTSGB_CUDA(cudaMemcpyAsync(output, target, n * sizeof(float),
                               cudaMemcpyDeviceToDevice, s));
    return DTSGB_OK;
  }
  unsigned char* scratch = nullptr;
  int st = scratch_for_current_device(&scratch);
  if (st) return st;
  uint32_t* bounds = reinterpret_cast<uint32_t*>(scratch);
  float* iterate = reinterpret_cast<float*>(scratch + (size_t)kNoAllocMaxPixels * 4);
  const float sz = optimize->sigma_z;
  const int r = (int)floorf(sz) + 1, hx = r - 1;
  const int tiles = ((width + kNaTile - 1) / kNaTile) * ((height + kNaTile - 1) / kNaTile);
  const size_t smem_b = sizeof(float) * 2 * (size_t)kNaTile * (kNaTile + 2 * r - 1);
  const size_t smem_i = sizeof(float) * ((size_t)(kNaTile + 2 * hx) * (kNaTile + 2 * hx) +
                                         (size_t)(kNaTile + 2 * hx) * kNaTile);
  if (smem_b > 227 * 1024 || smem_i > 227 * 1024)
    return fail(DTSGB_ERR_UNSUPPORTED, "sigma_z too large for the no-alloc kernels");
  if (smem_b > 48 * 1024)
    DTSGB_CUDA(cudaFuncSetAttribute(k_na_bounds, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem_b));
  const float rx = filter->sigma_x / filter->sigma_r, ry = filter->sigma_y / filter->sigma_r;
  k_na_bounds<<<tiles, kNaThreads, smem_b, s>>>((const uchar4*)rgba, width, height,
                                                color_space, rx, ry, sz, r, 1, bounds);
  DTSGB_CUDA(cudaGetLastError());
  // ping-pong between the scratch iterate and the output so that the last
  // iteration writes the output; the first reads the target
  const int N = optimize->num_iterations;
  const float* src = target;
  for (int k = 0; k < N; ++k) {
    float* dst = ((N - 1 - k) % 2 == 0) ? output : iterate;
    if (optimize->loss == DTSGB_L2) {
      if (smem_i > 48 * 1024)
        DTSGB_CUDA(cudaFuncSetAttribute(k_na_iter<0>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem_i));
      k_na_iter<0><<<tiles, kNaThreads, smem_i, s>>>(src, dst, target, confidence, bounds,
                                                     width, height, optimize->lambda,
                                                     optimize->step_size, overwrite, hx);
    } else {
      if (smem_i > 48 * 1024)
        DTSGB_CUDA(cudaFuncSetAttribute(k_na_iter<1>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem_i));
      k_na_iter<1><<<tiles, kNaThreads, smem_i, s>>>(src, dst, target, confidence, bounds,
                                                     width, height, optimize->lambda,
                                                     optimize->step_size, overwrite, hx);
    }
    DTSGB_CUDA(cudaGetLastError());
    src = dst;
  }
  return DTSGB_OK;
}
