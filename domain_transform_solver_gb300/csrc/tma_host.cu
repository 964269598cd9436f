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

TmaCache::~TmaCache() { clear(); }

void TmaCache::clear() {
  for (auto& kv : tables_) cudaFree(kv.second);
  tables_.clear();
}

const CUtensorMap* TmaCache::get(const Inst* h_inst, int n, const float* plane, int box_w,
                                 int box_h, cudaStream_t s) {
  if (!h_inst || n <= 0 || !plane) return nullptr;
  const auto key = std::make_tuple(plane, box_w, box_h);
  auto it = tables_.find(key);
  if (it != tables_.end()) return it->second;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    (void)cudaGetLastError();
    return nullptr;  // no synchronous copies inside a capture: the caller stages itself
  }
  std::vector<CUtensorMap> maps(n);
  for (int i = 0; i < n; ++i)
    if (tma_encode_plane(&maps[i], plane + h_inst[i].off, h_inst[i].w, h_inst[i].h,
                         h_inst[i].pitch, box_w, box_h))
      return nullptr;
  CUtensorMap* d = nullptr;
  if (cudaMalloc((void**)&d, sizeof(CUtensorMap) * n) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (cudaMemcpy(d, maps.data(), sizeof(CUtensorMap) * n, cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    cudaFree(d);
    return nullptr;
  }
  tables_[key] = d;
  return d;
}

}  // namespace dtsgb
