// Internal declarations shared by the CUDA translation units of libdtsgb.
// Nothing here is part of the public C ABI (include/dtsgb.h).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace dtsgb {

// ---------------------------------------------------------------------------
// Layout of one image instance in HBM.  Every per-pixel plane of a solver
// (guide, target, confidence, window bounds, iterates) uses the same
// element offset and row pitch, so one descriptor addresses all of them.
// The pitch is the width rounded up to 32 elements so that every row starts
// on a 128-byte boundary for 4-byte planes.
// ---------------------------------------------------------------------------
struct Inst {
  int w, h, pitch, pad;
  long long off;  // element offset of pixel (0,0)
};

// One 2D tile of an instance for the tiled DTS kernels.
struct Tile {
  int inst, x0, y0, pad;
};

// Packed per-pixel window bounds: the window along an axis is the half-open
// index range (p - dl, p + du], i.e. pixels p-dl+1 .. p+du, n = dl + du.
//   bits  0- 7 dl_x, 8-15 du_x, 16-23 dl_y, 24-31 du_y
__host__ __device__ inline uint32_t pack_bounds(int dlx, int dux, int dly,
                                                int duy) {
  return (uint32_t)dlx | ((uint32_t)dux << 8) | ((uint32_t)dly << 16) |
         ((uint32_t)duy << 24);
}

// dH / dV integrand of src/domain_transform_common_kernels.cuh:71-116
// (Uchar4SumOfSquaredDiffNormalize inside Compute_dHdx / Compute_dVdy):
// sqrt(SSD4(a - b) * kINV255Sq * r * r + 1) with r = sigma_{x|y} / sigma_r
// and kINV255Sq the float constant 0.0000153787 (:10), evaluated in the
// order nvcc compiles the reference expression.  >= 1 for every input.
// The sum of squared channel differences is exact integer arithmetic: the
// four |a - b| bytes (one SIMD byte instruction) dotted with themselves.
__device__ __forceinline__ float edge_weight(uchar4 a, uchar4 b, float ratio) {
  const unsigned d = __vabsdiffu4(*reinterpret_cast<const unsigned*>(&a),
                                  *reinterpret_cast<const unsigned*>(&b));
  const float ssd = (float)__dp4a(d, d, 0u);
  float t = __fmul_rn(ssd, (float)0.0000153787);
  t = __fmul_rn(t, ratio);
  return __fsqrt_rn(__fmaf_rn(t, ratio, 1.0f));
}

// Storage types for target / confidence.
enum class Storage : int { F32 = 0, BF16 = 1 };

template <typename T>
__device__ __forceinline__ float load_f(const T* p);
template <>
__device__ __forceinline__ float load_f<float>(const float* p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ float load_f<__nv_bfloat16>(const __nv_bfloat16* p) {
  return __bfloat162float(__ldg(p));
}

template <typename T>
__device__ __forceinline__ T store_cast(float v);
template <>
__device__ __forceinline__ float store_cast<float>(float v) {
  return v;
}
template <>
__device__ __forceinline__ __nv_bfloat16 store_cast<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}

// ---------------------------------------------------------------------------
// Status handling.
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define DTSGB_CUDA(call)                                  \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return ::dtsgb::cuda_fail(e_, #call); \
  } while (0)

// ---------------------------------------------------------------------------
// Programmatic dependent launch: a chain of kernels on one stream (solver
// iterations, heavy-ball and bistochastization passes) launches each kernel
// as a dependent of the one before it, so that its launch overlaps the
// predecessor's last blocks.  Every such kernel starts with
// pdl_wait_then_release(): it waits for the predecessor's grid to complete
// (its writes visible) before touching memory, then lets its own dependent
// launch.  In a plain launch both instructions are no-ops.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait_then_release() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block,
                                    size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchAttribute a[1];
  a[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  a[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t c = {};
  c.gridDim = grid;
  c.blockDim = block;
  c.dynamicSmemBytes = smem;
  c.stream = s;
  c.attrs = a;
  c.numAttrs = 1;
  return cudaLaunchKernelEx(&c, kernel, static_cast<KArgs>(args)...);
}

// ---------------------------------------------------------------------------
// Host helpers shared by the API translation units.
// ---------------------------------------------------------------------------
inline int round_up(int v, int m) { return (v + m - 1) / m * m; }
inline long long round_up_ll(long long v, long long m) { return (v + m - 1) / m * m; }
inline bool finite_pos(float v) { return v == v && v > 0.f && v < 3.4e38f; }

// Zero-initialised device allocation; returns a DTSGB_* status.  The fill
// runs on the legacy default stream, which the handles' non-blocking streams
// do not wait for, so it is finished here before the buffer is handed out.
template <typename T>
int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    (void)cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? (set_error("cudaMalloc: out of memory"), 5)
                                          : cuda_fail(e, "cudaMalloc");
  }
  e = cudaMemset(*p, 0, count * sizeof(T));
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemset");
  return 0;
}
template <typename T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

// sigma multiplier of DomainTransformFilter::Filter
// (src/domain_transform_filter.cu:142-152): 1 at iteration 0, else
// 3*2^(N-i-1)/sqrt(4^N-1) evaluated in double and stored as float.
float filter_sigma_multiplier(int it, int n);

// ---------------------------------------------------------------------------
// Kernel timing (profile.cu): no-ops unless enabled through the C ABI.
// ---------------------------------------------------------------------------
void prof_begin(cudaStream_t s, int kernel_id);
void prof_end(cudaStream_t s, int kernel_id);
bool prof_enabled();
void prof_set_capture_tag(const void* tag);
void prof_drop_captured(const void* tag);

struct ProfScope {
  cudaStream_t s;
  int id;
  ProfScope(cudaStream_t s_, int id_) : s(s_), id(id_) { prof_begin(s, id); }
  ~ProfScope() { prof_end(s, id); }
};

// ---------------------------------------------------------------------------
// DTS launchers (dts_kernels.cu).  All take device pointers and a stream and
// return a DTSGB_* status.
// ---------------------------------------------------------------------------
class TmaCache;

struct DtsLaunch {
  const Inst* d_inst;   // device instance table
  const Tile* d_tiles;  // device tile table for the tile shape in use
  int n_tiles;
  int n_inst;
  bool small = false;   // iteration tiles of kIterSmallTW x kIterSmallTH
  // kIterSmallTW x kIterSmallTH tiles, used when a halo is too large for the
  // shared memory of the big tiles (null: none)
  const Tile* d_tiles_small = nullptr;
  int n_tiles_small = 0;
  // tensor maps of the iterate planes for TMA staging, and the host copy of
  // the instance table they describe (null: the kernels stage by loads)
  TmaCache* tma = nullptr;
  const Inst* h_inst = nullptr;
  // pixels per thread and axis of the window-bound walks (4, 8 or 16)
  int bounds_seg = 8;
  // the same launch on the small tiles
  DtsLaunch as_small() const {
    DtsLaunch s = *this;
    s.d_tiles = d_tiles_small;
    s.n_tiles = n_tiles_small;
    s.small = true;
    return s;
  }
};

// Tile shapes (compile-time in the kernels).
constexpr int kBoundsTW = 32, kBoundsTH = 32;
constexpr int kIterTW = 64, kIterTH = 128;
// Work too small to give every SM a few 64x64-pixel blocks (under about
// 2.5 Mpx in all) uses 32x32 tiles.  tiles_big counts kIterTW x kIterTH tiles.
constexpr int kIterSmallTW = 32, kIterSmallTH = 32;
inline bool use_small_iter_tiles(long long tiles_big) {
  return tiles_big * kIterTW * kIterTH < 4LL * 152 * 64 * 64;
}

int launch_color_convert(const Inst* h_inst, const Inst* d_inst, int n_inst,
                         uchar4* guide, int color_space, cudaStream_t s);
// in-place conversion over a flat run of n pixels (ignores pitch padding)
int launch_color_convert_flat(uchar4* guide, long long n, int color_space,
                              cudaStream_t s);

int launch_bounds(const DtsLaunch& L, const uchar4* guide, uint32_t* bounds,
                  float ratio_x, float ratio_y, float sigma_x, float sigma_y,
                  int ref_y_limit, cudaStream_t s);

enum class IterMode : int { L2 = 0, CHARB = 1 };

// DomainTransformStereo's photometric term (src/domain_transform_loss_term.cuh):
// converted left / right guides (same layout as the iterate), centre
// offset, photo_consis_lambda, alpha = (sigma_r/sigma_x)^2 and the sigma
// ratio of the right image's dHdx (negative: dHdx never computed, reads 0).
struct StereoArgs {
  const uchar4* left;
  const uchar4* right;
  float offset, lam_p, alpha, ratio;
};

int launch_dts_iter(const DtsLaunch& L, Storage st, IterMode mode,
                    const float* vin, float* vout, const void* target,
                    const void* conf, const uint32_t* bounds, float lambda,
                    float step, float overwrite, int halo_x, int halo_y,
                    cudaStream_t s, const StereoArgs* stereo = nullptr);
// v = target (as float), optionally overwritten nowhere: the initial iterate.
int launch_init_var(const DtsLaunch& L, Storage st, const void* target,
                    float* v, cudaStream_t s);

// Box pass of the domain-transform filter over nch channels sharing bounds.
// When conf_out is non-null (confidence epilogue), nch must be 2 and the
// result written is exp(-(ch1 - ch0^2) * scale) (0 for x <= left_clear or a
// negative / non-finite variance) into conf_out (storage st).
int launch_filter_pass(const DtsLaunch& L, int nch, const float* in0,
                       const float* in1, float* out0, float* out1,
                       const uint32_t* bounds, int halo_x, int halo_y,
                       Storage st, void* conf_out, float scale,
                       int left_clear, cudaStream_t s);

// Helpers for the filter / confidence paths.
int launch_target_to_float(const DtsLaunch& L, Storage st, const void* src,
                           float* dst, float* dst_sq, cudaStream_t s);
int launch_storage_from_float(const Inst* h_inst, int n_inst, Storage st,
                              const float* src, void* dst, long long n,
                              cudaStream_t s);
int launch_fill_storage(Storage st, void* dst, long long n, float value,
                        cudaStream_t s);

// Debug / download helpers.
int launch_differential(const DtsLaunch& L, const uchar4* guide, float ratio,
                        int axis, float* out, cudaStream_t s);
int launch_row_prefix(const Inst* h_inst, const Inst* d_inst, int n_inst,
                      const float* in, float* out, cudaStream_t s);
int launch_unpack_bounds(const DtsLaunch& L, const uint32_t* bounds, int axis,
                         int32_t* l, int32_t* u, cudaStream_t s);
// CTAs of the iteration kernels that gave up waiting for their TMA staging
// since the library was loaded (0 on a healthy run).
unsigned long long dts_wait_timeouts();
// The box (columns x rows) of the iteration kernel's TMA staging for halos
// hx, hy on L's tile shape; 0 x 0 when it stages by loads.  An owner builds
// its tensor maps for that box before a graph capture.
void dts_iter_tma_box(const DtsLaunch& L, int hx, int hy, int* box_w, int* box_h);

// ---------------------------------------------------------------------------
// Adjoint of the fixed-window solve (dts_adjoint.cu).
// ---------------------------------------------------------------------------
struct DtsGrad {
  int seg;               // iterations per checkpoint segment (>= 1)
  float* const* cp;      // checkpoints v_seg, v_2seg, ...: ceil(N/seg) - 1 planes
  float* const* segbuf;  // seg planes for the recomputed iterates of a segment
  float* g[2];           // adjoint ping-pong; g[0] holds dL/dv_N on entry
};
// The segment length that minimises the planes held, ceil(N/seg) - 1 + seg
// (near sqrt(N)), taking the smallest such length, which recomputes the
// fewest iterations.
int dts_checkpoint_segment(int num_iterations);
// The forward solve (init + num_iterations fused iterations, no overwrite),
// writing v_seg, v_2seg, ... into G.cp; the result ends in v0 or v1
// (*result_idx).
int dts_forward_checkpointed(const DtsLaunch& L, Storage st, IterMode mode,
                             const DtsGrad& G, const void* target, const void* conf,
                             const uint32_t* bounds, float lambda, float step, int halo,
                             int num_iterations, float* v0, float* v1, int* result_idx,
                             cudaStream_t s);
// Which of v0 / v1 holds the result of dts_forward_checkpointed.
int dts_checkpointed_result_index(int num_iterations, int seg);
// dL/dt and dL/dc (planes of the instance layout, overwritten) for the
// upstream gradient in G.g[0]; G.g[0] and G.g[1] are clobbered.
int dts_backward(const DtsLaunch& L, const Inst* d_inst, int n_inst, long long plane,
                 Storage st, IterMode mode, const DtsGrad& G, const void* target,
                 const void* conf, const uint32_t* bounds, float lambda, float step,
                 int halo, int num_iterations, float* grad_t, float* grad_c,
                 cudaStream_t s);

}  // namespace dtsgb
