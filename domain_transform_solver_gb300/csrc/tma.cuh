// Tensor-memory-accelerator (TMA) staging for sm_103a kernels: inline PTX
// for mbarriers and cp.async.bulk.tensor, bounded waits, and a host-side
// cache of tensor maps (one per instance of a batch and per source plane).
//
// A tensor map describes one instance's plane as a 2D tensor of W x H
// 4-byte elements with a row pitch of `pitch` elements (a multiple of 32,
// so every row starts on a 128-byte boundary).  A tiled load of a box that
// reaches past the image (negative coordinates, x >= W, y >= H) reads zeros
// there, which is what the staging kernels need at image borders.  The
// innermost start coordinate times 4 bytes must be a multiple of 16: the
// kernels start boxes at multiples of 4 columns.
#pragma once

#include <cuda.h>  // CUtensorMap and its enums (types only)

#include <map>
#include <tuple>
#include <vector>

#include "dtsgb_internal.cuh"

namespace dtsgb {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// Makes the initialised mbarrier visible to the async proxy (the TMA unit).
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of the mbarrier at most `limit` polls (each
// try_wait itself suspends for a bounded, hardware-chosen time); false when
// the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned limit) {
  for (unsigned i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 2D tiled load of the box at (x, y) of tensor map `tmap` (global memory)
// into shared memory at dst (128-byte aligned), completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tmap, int x, int y,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// 3D tiled load of the box at (x, y, z) of tensor map `tmap` into shared
// memory at dst (128-byte aligned), completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tmap, int x, int y,
                                            int z, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(x), "r"(y), "r"(z),
      "r"(smem_u32(bar))
      : "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later async-proxy (TMA) accesses: issued by the thread that reuses
// a buffer for a TMA load after a barrier with the threads that read it.
__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Polls of a staging wait before a kernel gives up (about a second at the
// hardware's try_wait suspend time); a CTA that gives up counts the event
// in its translation unit's wait-timeout counter (dtsgb_wait_timeouts) and
// returns without writing its tile.
constexpr unsigned kTmaWaitPolls = 1u << 22;

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

// Encodes a tensor map of one 4-byte-element plane (W x H, row pitch in
// elements) with a box of box_w x box_h elements; a DTSGB_* status.
int tma_encode_plane(CUtensorMap* out, const void* base, int w, int h, int pitch, int box_w,
                     int box_h);

// One instance's 3D grid inside a grid plane: gx x gy x gl 4-byte voxels at
// element offset off, rows of px voxels (px a multiple of 4).
struct TmaGrid {
  long long off;
  int gx, gy, gl, px;
};

// Encodes a tensor map of one grid (dims gx, gy, gl; row pitch px voxels,
// level pitch px * gy) with a box of bx x by x bl voxels.
int tma_encode_grid(CUtensorMap* out, const void* base, const TmaGrid& g, int bx, int by,
                    int bl);

// Device tables of tensor maps, one entry per instance, for a source plane
// (the arena base of a per-pixel plane or of a grid plane) and a box shape;
// built on first use (never while the stream is being captured) and kept
// until clear() or destruction.  The owner clears the cache when the
// instances' geometry changes.
class TmaCache {
 public:
  TmaCache() = default;
  TmaCache(const TmaCache&) = delete;
  TmaCache& operator=(const TmaCache&) = delete;
  ~TmaCache();
  // the table for `plane` (instances h_inst[0..n)), or nullptr when it is
  // not built and cannot be built now (capture in progress, failure)
  const CUtensorMap* get(const Inst* h_inst, int n, const float* plane, int box_w, int box_h,
                         cudaStream_t s);
  // the same for grids (3D boxes of bx x by x bl voxels)
  const CUtensorMap* get_grid(const TmaGrid* grids, int n, const float* plane, int bx, int by,
                              int bl, cudaStream_t s);
  void clear();

 private:
  const CUtensorMap* upload(const std::vector<CUtensorMap>& maps,
                            const std::tuple<const float*, int, int, int>& key);
  std::map<std::tuple<const float*, int, int, int>, CUtensorMap*> tables_;
};

}  // namespace dtsgb
