// Host side of the TMA staging (tma.cuh): tensor-map encoding through the
// driver entry point resolved at run time (no link against libcuda), and
// the per-owner cache of device tables of tensor maps.
#include <cudaTypedefs.h>

#include <string>

#include <mutex>

#include "../../include/dtsgb.h"
#include "tma.cuh"

namespace dtsgb {
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      (void)cudaGetLastError();
  });
  return fn;
}

}  // namespace

int tma_encode_plane(CUtensorMap* out, const void* base, int w, int h, int pitch, int box_w,
                     int box_h) {
  auto fn = encode_fn();
  if (!fn) return fail(DTSGB_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  if (box_w <= 0 || box_w > 256 || box_h <= 0 || box_h > 256 || (box_w * 4) % 16 != 0 ||
      ((uintptr_t)base & 15) != 0 || (pitch * 4) % 16 != 0)
    return fail(DTSGB_ERR_UNSUPPORTED, "plane or box outside the TMA limits");
  const cuuint64_t dims[2] = {(cuuint64_t)w, (cuuint64_t)h};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch * 4};
  const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(DTSGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return DTSGB_OK;
}

int tma_encode_grid(CUtensorMap* out, const void* base, const TmaGrid& g, int bx, int by,
                    int bl) {
  auto fn = encode_fn();
  if (!fn) return fail(DTSGB_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  if (bx <= 0 || bx > 256 || by <= 0 || by > 256 || bl <= 0 || bl > 256 ||
      (bx * 4) % 16 != 0 || ((uintptr_t)base & 15) != 0 || (g.px * 4) % 16 != 0)
    return fail(DTSGB_ERR_UNSUPPORTED, "grid or box outside the TMA limits");
  const cuuint64_t dims[3] = {(cuuint64_t)g.gx, (cuuint64_t)g.gy, (cuuint64_t)g.gl};
  const cuuint64_t strides[2] = {(cuuint64_t)g.px * 4, (cuuint64_t)g.px * g.gy * 4};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bl};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(DTSGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return DTSGB_OK;
}

TmaCache::~TmaCache() { clear(); }

const CUtensorMap* TmaCache::upload(const std::vector<CUtensorMap>& maps,
                                    const std::tuple<const float*, int, int, int>& key) {
  CUtensorMap* d = nullptr;
  if (cudaMalloc((void**)&d, sizeof(CUtensorMap) * maps.size()) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (cudaMemcpy(d, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    cudaFree(d);
    return nullptr;
  }
  tables_[key] = d;
  return d;
}

// No synchronous copies inside a capture: the caller then stages by loads.
static bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    (void)cudaGetLastError();
    return true;
  }
  return cs != cudaStreamCaptureStatusNone;
}

const CUtensorMap* TmaCache::get_grid(const TmaGrid* grids, int n, const float* plane, int bx,
                                      int by, int bl, cudaStream_t s) {
  if (!grids || n <= 0 || !plane) return nullptr;
  const auto key = std::make_tuple(plane, bx, by, 1000 + bl);
  auto it = tables_.find(key);
  if (it != tables_.end()) return it->second;
  if (capturing(s)) return nullptr;
  std::vector<CUtensorMap> maps(n);
  for (int i = 0; i < n; ++i)
    if (tma_encode_grid(&maps[i], plane + grids[i].off, grids[i], bx, by, bl)) return nullptr;
  return upload(maps, key);
}

void TmaCache::clear() {
  for (auto& kv : tables_) cudaFree(kv.second);
  tables_.clear();
}

const CUtensorMap* TmaCache::get(const Inst* h_inst, int n, const float* plane, int box_w,
                                 int box_h, cudaStream_t s) {
  if (!h_inst || n <= 0 || !plane) return nullptr;
  const auto key = std::make_tuple(plane, box_w, box_h, 0);
  auto it = tables_.find(key);
  if (it != tables_.end()) return it->second;
  if (capturing(s)) return nullptr;
  std::vector<CUtensorMap> maps(n);
  for (int i = 0; i < n; ++i)
    if (tma_encode_plane(&maps[i], plane + h_inst[i].off, h_inst[i].w, h_inst[i].h,
                         h_inst[i].pitch, box_w, box_h))
      return nullptr;
  return upload(maps, key);
}

}  // namespace dtsgb
