// Stand-in for the CUB block collectives the reference's row scan uses
// (cub::BlockLoad, cub::BlockStore, cub::BlockScan) -- TEST INFRASTRUCTURE
// ONLY.  CUB (the reference's ext/cub submodule) is not in the checkout.
// Restated from CUB's published algorithms, executed by refemu's
// cooperative launches (every thread of the block calls each collective):
//   * BlockLoad / BlockStore with a *_WARP_TRANSPOSE algorithm leave the
//     items in a blocked arrangement -- thread t holds items
//     t*ITEMS .. t*ITEMS+ITEMS-1 -- and touch only the first valid_items;
//   * BlockScan<..., BLOCK_SCAN_RAKING[_MEMOIZE]>::InclusiveSum with a
//     block aggregate and a prefix callback: each thread reduces its items
//     left to right; the thread partials are reduced in segments of
//     ceil(threads / 32) by up to 32 raking threads; those raking partials
//     get an exclusive warp scan (Kogge-Stone: at distance 1, 2, 4, 8, 16
//     lane i adds lane i-d's value in front of its own); every thread of
//     warp 0 calls the callback with the block aggregate and lane 0's answer
//     is the block prefix, which is added in front of the raking lanes'
//     exclusive prefixes (lane 0 takes it as its prefix); the raking
//     threads scan their segments exclusively from those prefixes, and each
//     thread scans its own items inclusively from its prefix.
// The association order follows that description; bit-for-bit equality
// with a particular CUB release is not claimed.
#pragma once

#include "refemu.h"

namespace cub {

enum BlockLoadAlgorithm {
  BLOCK_LOAD_DIRECT,
  BLOCK_LOAD_VECTORIZE,
  BLOCK_LOAD_TRANSPOSE,
  BLOCK_LOAD_WARP_TRANSPOSE
};
enum BlockStoreAlgorithm {
  BLOCK_STORE_DIRECT,
  BLOCK_STORE_VECTORIZE,
  BLOCK_STORE_TRANSPOSE,
  BLOCK_STORE_WARP_TRANSPOSE
};
enum BlockScanAlgorithm { BLOCK_SCAN_RAKING, BLOCK_SCAN_RAKING_MEMOIZE, BLOCK_SCAN_WARP_SCANS };

template <class Ptr, int BLOCK_THREADS, int ITEMS, BlockLoadAlgorithm ALG = BLOCK_LOAD_DIRECT>
class BlockLoad {
 public:
  struct TempStorage {
    char unused;
  };
  explicit BlockLoad(TempStorage&) {}
  template <class T>
  void Load(Ptr in, T (&items)[ITEMS], int valid_items) {
    const int base = (int)refemu::linear_tid() * ITEMS;
    for (int i = 0; i < ITEMS; ++i)
      if (base + i < valid_items) items[i] = in[base + i];
  }
};

template <class Ptr, int BLOCK_THREADS, int ITEMS, BlockStoreAlgorithm ALG = BLOCK_STORE_DIRECT>
class BlockStore {
 public:
  struct TempStorage {
    char unused;
  };
  explicit BlockStore(TempStorage&) {}
  template <class T>
  void Store(Ptr out, T (&items)[ITEMS], int valid_items) {
    const int base = (int)refemu::linear_tid() * ITEMS;
    for (int i = 0; i < ITEMS; ++i)
      if (base + i < valid_items) out[base + i] = items[i];
  }
};

template <class T, int BLOCK_THREADS, BlockScanAlgorithm ALG = BLOCK_SCAN_RAKING>
class BlockScan {
  static constexpr int kWarp = 32;
  static constexpr int kMaxRaking = BLOCK_THREADS < kWarp ? BLOCK_THREADS : kWarp;
  static constexpr int kSegment = (BLOCK_THREADS + kMaxRaking - 1) / kMaxRaking;
  static constexpr int kRaking = (BLOCK_THREADS + kSegment - 1) / kSegment;

 public:
  struct TempStorage {
    T partial[BLOCK_THREADS];   // thread partials, then their exclusive prefixes
    T raking_excl[kRaking];     // raking lanes' exclusive prefixes (no block prefix)
    T aggregate;
    T block_prefix;
  };
  explicit BlockScan(TempStorage& s) : s_(s) {}

  template <int ITEMS, class PrefixOp>
  void InclusiveSum(T (&in)[ITEMS], T (&out)[ITEMS], T& block_aggregate, PrefixOp& prefix_op) {
    const int t = (int)refemu::linear_tid();
    T partial = in[0];
    for (int i = 1; i < ITEMS; ++i) partial = partial + in[i];
    s_.partial[t] = partial;
    __syncthreads();
    if (t == 0) {
      // Upsweep: each raking lane reduces its segment.
      T lane[kWarp];
      for (int r = 0; r < kRaking; ++r) {
        T acc = s_.partial[r * kSegment];
        for (int k = 1; k < kSegment && r * kSegment + k < BLOCK_THREADS; ++k)
          acc = acc + s_.partial[r * kSegment + k];
        lane[r] = acc;
      }
      // Kogge-Stone inclusive warp scan over the raking partials.
      for (int d = 1; d < kRaking; d *= 2) {
        T next[kWarp];
        for (int r = 0; r < kRaking; ++r) next[r] = r >= d ? lane[r - d] + lane[r] : lane[r];
        for (int r = 0; r < kRaking; ++r) lane[r] = next[r];
      }
      s_.aggregate = lane[kRaking - 1];
      for (int r = 0; r < kRaking; ++r) s_.raking_excl[r] = r == 0 ? T() : lane[r - 1];
    }
    __syncthreads();
    // Warp 0 calls the callback; lane 0's answer is the block prefix.
    if (t < kWarp) {
      const T bp = prefix_op(s_.aggregate);
      if (t == 0) s_.block_prefix = bp;
    }
    __syncthreads();
    if (t == 0) {
      // Downsweep: raking lanes scan their segments from their prefixes.
      for (int r = 0; r < kRaking; ++r) {
        T run = r == 0 ? s_.block_prefix : s_.block_prefix + s_.raking_excl[r];
        for (int k = 0; k < kSegment && r * kSegment + k < BLOCK_THREADS; ++k) {
          const T p = s_.partial[r * kSegment + k];
          s_.partial[r * kSegment + k] = run;
          run = run + p;
        }
      }
    }
    __syncthreads();
    T run = s_.partial[t];
    for (int i = 0; i < ITEMS; ++i) {
      run = run + in[i];
      out[i] = run;
    }
    block_aggregate = s_.aggregate;
    __syncthreads();
  }

 private:
  TempStorage& s_;
};

}  // namespace cub
