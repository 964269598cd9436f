// Internal HFBS declarations (not part of the C ABI).
#pragma once

#include "dtsgb_internal.cuh"

namespace dtsgb {

// One HFBS instance: its image plane (shared layout with the DTS planes)
// and its bilateral grid.
struct HInst {
  int w, h, pitch;
  int gx, gy, gl;
  // pad faces written by the reference's FillGrid (g % 8 != 0 and inside
  // the max-size allocation); they read the last fill value of the buffer
  int cov_x, cov_y, cov_l;
  // luma bin == gl is stored (and read back by the slice) only when the
  // z = gl plane lies inside the allocation
  int ovf_stored;
  long long pix_off;    // element offset of pixel (0,0)
  long long grid_off;   // element offset of voxel (0,0,0)
  long long plane_off;  // element offset of the overflow count plane
  // float2 offset of the slice grid: (count * z, count) over (gx + 1) x
  // (gy + 1) x (gl + 2) voxels, zero past the grid and the overflow counts
  // in plane gl (see k_slice_pack)
  long long slice_off;
};

// First pixel index p >= 0 with floorf(p * 1.0f / sigma) >= cell (the
// reference's bin of pixel p, src/hfbs.cu:82-83); n if none.
__device__ __forceinline__ int cell_start(int cell, float sigma, int n) {
  int p = (int)ceilf((float)cell * sigma) - 2;
  if (p < 0) p = 0;
  if (p > n) p = n;
  while (p < n && (int)floorf((float)p * 1.0f / sigma) < cell) ++p;
  while (p > 0 && (int)floorf((float)(p - 1) * 1.0f / sigma) >= cell) --p;
  return p;
}

// Solver parameters shared by a batch (HFBSGridParams minus the grid dims).
struct HParams {
  float sigma_x, sigma_y, sigma_l, lambda, alpha, beta;
  int bistoch_iter_max, optim_iter_max;
  float neg_exp_beta;
};

// Forward iterates kept for the HFBS adjoint, and its scratch grids (all
// total_voxels floats per plane).  segment 1: z_0 stays in the z0 buffer and
// z_k (1 <= k < K) is written to hist + (k - 1) planes, nothing is recomputed.
// segment S > 1: z and h at the start of every S-step segment go to slot j of
// ckz / ckh (step j*S), and the backward recomputes a segment's iterates into
// seg (S - 1 planes) with h in hrec.
struct HfbsGradState {
  int segment = 1;
  float* hist = nullptr;
  float *ckz = nullptr, *ckh = nullptr, *seg = nullptr, *hrec = nullptr;
  float *gz = nullptr, *gh = nullptr, *gg = nullptr, *gw = nullptr, *gb = nullptr,
        *ginv = nullptr;
};

// Device buffers and sizes of a batch of HFBS instances.
struct HfbsBatch {
  const HInst* d_inst;
  int n_inst;
  // host copy of the instance table and the voxel budget of an L2-resident
  // group (0: all instances together); see hfbs_enqueue_solve
  const HInst* h_inst = nullptr;
  long long group_voxels = 0;
  // the bistochastized normalisation in n0 / n1 (by the parity of
  // bistoch_iter_max) is that of the same guide and grid: skip recomputing it
  bool reuse_norm = false;
  long long max_voxels, max_pixels, max_cells, max_lines;
  // voxels of the whole grid arena (instances and the gaps that round each
  // instance's grid to 32 voxels): the span of the elementwise kernels
  long long total_voxels;
  long long max_rows;  // max over instances of gy * gl (grid rows along x)
  int max_gl;
  const uchar4* guide;
  const void* target;  // storage type st
  const void* conf;
  Storage st;
  float* out;
  float *count, *csum, *b, *n0, *n1, *invA, *z0, *z1, *h, *t0, *t1, *t2, *ovf;
  float2* sgrid;  // the instances' slice grids (HInst::slice_off)
  // optional debug copies (single-instance class API)
  bool keep_debug;
  size_t grid_bytes;
  float *dbg_norm, *dbg_blur_c, *dbg_z_init, *dbg_z_final;
  // non-null: record the forward iterates for hfbs_enqueue_backward (the
  // one-step heavy-ball kernel, all instances as one group)
  const HfbsGradState* grad = nullptr;
};

// Enqueue the whole HFBS::Optimize sequence (splat .. slice) on a stream.
int hfbs_enqueue_solve(const HfbsBatch& B, const HParams& p, cudaStream_t s);

// One heavy-ball step of every instance: zs -> zd, h in place.
void hfbs_launch_step(const HfbsBatch& B, const HParams& p, const float* zs, float* zd,
                      float* h, const float* norm, cudaStream_t s);

// X -> Y -> Z Laplace blur of two grids s0, s1 into x0, x1 (y0, y1 scratch).
void hfbs_launch_blur_pair(const HfbsBatch& B, const HParams& p, const float* s0,
                           const float* s1, float* x0, float* x1, float* y0, float* y1,
                           cudaStream_t s);

// Adjoint of the last hfbs_enqueue_solve of B (run with B.grad): upstream
// gradient gout (pixel layout of the instances) to dL/dtarget and
// dL/dconfidence (same layout; either may be null).
int hfbs_enqueue_backward(const HfbsBatch& B, const HParams& p, const float* gout,
                          float* grad_t, float* grad_c, cudaStream_t s);

}  // namespace dtsgb
