// Internal HFBS declarations (not part of the C ABI).
#pragma once

#include "dtsgb_internal.cuh"
#include "tma.cuh"

namespace dtsgb {

// One HFBS instance: its image plane (shared layout with the DTS planes)
// and its bilateral grid.
struct HInst {
  int w, h, pitch;
  int gx, gy, gl;
  // row pitch of the grids in voxels: gx rounded up to a multiple of 4, so
  // that every grid row starts on a 16-byte boundary (tensor-map tiles);
  // voxel (x, y, l) is at grid_off + (l * gy + y) * px + x, and the voxels
  // x >= gx of a row are padding that no stencil reads
  int px;
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
// total_voxels floats per plane).  segment 1: z_k (0 <= k < K) in hist plane
// k, nothing is recomputed.  segment S > 1: z and h at the start of every
// S-step segment go to slot j of ckz / ckh (step j*S), and the backward
// recomputes a segment's iterates into seg (S - 1 planes) with h ping-ponging
// through hrec / hrec2.  The adjoint's scratch: gz, gh, gb, ginv and two
// (gg, gw) pairs.
struct HfbsGradState {
  int segment = 1;
  float* hist = nullptr;
  float *ckz = nullptr, *ckh = nullptr, *seg = nullptr, *hrec = nullptr, *hrec2 = nullptr;
  float *gz = nullptr, *gh = nullptr, *gb = nullptr, *ginv = nullptr;
  float *gg = nullptr, *gw = nullptr, *gg2 = nullptr, *gw2 = nullptr;
};

// Grid planes of an HfbsGradState for K steps and segment S.
inline long long hfbs_grad_planes(int K, int S) {
  if (S == 1) return 8 + (K > 0 ? K : 0);
  const long long nck = (K + S - 1) / S;
  return 8 + 2 * nck + (S - 1) + 2;
}

// Point G's planes into an arena of hfbs_grad_planes(K, S) * tv floats.
inline void hfbs_carve_grad(HfbsGradState& G, float* arena, int K, int S, long long tv) {
  float* q = arena;
  auto take = [&](long long planes) {
    float* r = q;
    q += planes * tv;
    return r;
  };
  G = HfbsGradState{};
  G.segment = S;
  G.gz = take(1);
  G.gh = take(1);
  G.gb = take(1);
  G.ginv = take(1);
  G.gg = take(1);
  G.gw = take(1);
  G.gg2 = take(1);
  G.gw2 = take(1);
  if (S == 1) {
    G.hist = take(K > 0 ? K : 0);
  } else {
    const long long nck = (K + S - 1) / S;
    G.ckz = take(nck);
    G.ckh = take(nck);
    G.seg = take(S - 1);
    G.hrec = take(1);
    G.hrec2 = take(1);
  }
}

// Device buffers and sizes of a batch of HFBS instances.
struct HfbsBatch {
  const HInst* d_inst;
  int n_inst;
  // host copy of the instance table and the voxel budget of an L2-resident
  // group (0: all instances together); see hfbs_enqueue_solve
  const HInst* h_inst = nullptr;
  long long group_voxels = 0;
  // heavy-ball steps per launch: kHfbsTBSteps (the temporally blocked
  // kernel, where every grid has at most 16 levels) or 1 (the one-step
  // kernel for every grid)
  int solve_steps = 4;
  // tensor maps of the grid planes for the temporally blocked kernels' TMA
  // staging (null: they stage by 4-byte copies); owned by the caller, which
  // clears it when the instances' grids change
  TmaCache* tma = nullptr;
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

// Heavy-ball steps per launch of the temporally blocked kernel.
constexpr int kHfbsTBSteps = 4;

// Builds the grid tensor maps the solve of B will stage from (grid planes
// b, invA, both z and h buffers, both normalisation buffers, the counts),
// so that a graph capture of the solve finds them; a no-op without B.tma.
void hfbs_prepare_tma(const HfbsBatch& B, cudaStream_t s);

// CTAs of the temporally blocked kernels that gave up waiting for their TMA
// staging since the library was loaded (0 on a healthy run).
unsigned long long hfbs_wait_timeouts();

// Whether the batch's heavy-ball steps run temporally blocked (every grid
// at most 16 levels, host instance table given, solve_steps not 1).  Its neighbour sums add
// rounded z * n products; the one-step kernel's fuse them (FMA).
bool hfbs_uses_tb(const HfbsBatch& B);

// `steps` heavy-ball steps of every instance from (zs, hs) to (zd, hd): one
// temporally blocked launch (steps <= kHfbsTBSteps), else one one-step launch
// (steps == 1, h updated in place in hd: the caller passes hs == hd).  rec:
// z after each of the first rec_steps steps, plane stride total_voxels
// (temporally blocked launches only).
void hfbs_launch_steps(const HfbsBatch& B, const HParams& p, const float* norm,
                       const float* zs, float* zd, const float* hs, float* hd, int steps,
                       float* rec, int rec_steps, cudaStream_t s);

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
