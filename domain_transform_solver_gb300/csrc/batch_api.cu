// Batched DTS / HFBS over many images of uneven size (C ABI in
// include/dtsgb.h).  All instances live in one arena: plane k of instance i
// starts at element offset off_i (rows pitched to 32 elements), and every
// kernel launch covers every instance through the instance and tile tables,
// so a solve costs the same number of launches for 1 or 1000 images.  The
// fixed launch sequence of each solve can be captured as a CUDA graph and
// replayed (the iteration counts are fixed and nothing depends on data).
//
// HFBS instances of a batch behave like HFBS objects whose max grid exceeds
// their grid on every axis (as in the reference's CLIs): pad faces of axes
// with g % 8 != 0 are covered, and the luma-overflow plane is stored.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <initializer_list>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/dtsgb.h"
#include "color.cuh"
#include "dtsgb_internal.cuh"
#include "hfbs_internal.cuh"
#include "tma.cuh"

using namespace dtsgb;

namespace {

struct Graph {
  cudaGraphExec_t exec = nullptr;
  std::vector<char> key;
};

template <typename T>
void key_append(std::vector<char>& k, const T& v) {
  const char* p = reinterpret_cast<const char*>(&v);
  k.insert(k.end(), p, p + sizeof(T));
}

enum { HG_COUNT = 0, HG_CSUM, HG_B, HG_N0, HG_N1, HG_INVA, HG_Z0, HG_Z1, HG_H,
       HG_T0, HG_T1, HG_T2, HG_NUM };

}  // namespace

struct dtsgb_batch_s {
  int n = 0;
  unsigned flags = 0;
  Storage st = Storage::F32;
  int ref_y = 1;
  std::vector<Inst> inst;
  long long total = 0;
  int max_w = 0, max_h = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  uchar4* guide = nullptr;
  void* target = nullptr;
  void* conf = nullptr;
  uint32_t* bounds = nullptr;
  float* v[2] = {nullptr, nullptr};
  float* hout = nullptr;
  float* scratch = nullptr;
  // host uploads: every image is copied whole (one contiguous copy per
  // plane) into a dense staging area, then one kernel writes the pitched
  // planes; soff[i] = pixels of the instances before i
  std::vector<long long> soff;
  long long dense = 0;
  long long* d_soff = nullptr;
  // device copies of caller pointer arrays (3 x n), for the _device calls,
  // and the host copy of what each slot holds (a slot is re-sent only when
  // the caller's pointers change)
  float** d_uptr = nullptr;
  std::vector<const void*> uptr_host;
  bool uptr_valid[3] = {false, false, false};
  unsigned char* stage = nullptr;  // dense x (rgba 4 B, target 4 B, conf 4 B)
  Inst* d_inst = nullptr;
  Tile* d_tb = nullptr;
  Tile* d_ti = nullptr;     // iteration tiles of the shape in use
  Tile* d_ti_big = nullptr;  // kIterTW x kIterTH tiles
  Tile* d_ti_small = nullptr;  // kIterSmallTW x kIterSmallTH tiles
  int ntb = 0, nti = 0, nti_big = 0, nti_small = 0;
  bool small = false;
  long long hfbs_group_voxels = 0;  // L2-resident HFBS group budget (0: off)
  int hfbs_solve_steps = 4;         // heavy-ball steps per launch (4 or 1)
  int bounds_seg = 8;               // pixels per window-bound walk (4, 8, 16)
  // Guide-derived state kept across solves while the guide is unchanged
  // (video frames that change only the target): the DTS window bounds and
  // the HFBS bistochastized normalisation.
  unsigned long long guide_gen = 0;  // bumped by every guide upload
  bool reuse = true;
  struct BoundsKey {
    unsigned long long gen;
    float rx, ry, sz;
    int ref_y;
  } bkey{~0ull, 0.f, 0.f, 0.f, 0};
  struct NormKey {
    unsigned long long gen;
    float sx, sy, sl;
    int bistoch;
  } nkey{~0ull, 0.f, 0.f, 0.f, 0};
  int dts_res = -1;
  bool hfbs_done = false;
  bool use_graphs = true;
  Graph g_dts, g_hfbs;
  std::vector<HInst> hinst;
  HInst* d_hinst = nullptr;
  float* hg[HG_NUM] = {};
  long long gcap = 0;
  float* ovf = nullptr;
  long long ocap = 0;
  float2* sgrid = nullptr;
  long long scap = 0;
  // gradients of the DTS solve
  bool grad = false;
  int grad_seg_req = 0;          // 0: dts_checkpoint_segment(N)
  int grad_seg = 1;              // segment length of the planes below
  int grad_n = -1;               // iterations the adjoint replays (-1: none kept)
  std::vector<float*> gplanes;   // checkpoints, segment planes, 2 adjoint, dt, dc
  dtsgb_optimize_params gopt{};  // parameters of the solve the planes belong to
  float ghalo = 0.f;
  Graph g_bwd;
  // gradients of the HFBS solve (the same enable_grad switch): the kept
  // iterates and adjoint grids (hfbs_grad_planes) in hgbuf; three pixel
  // planes (dL/dout, dL/dtarget, dL/dconfidence) in hpix
  float* hgbuf = nullptr;
  size_t hgcap = 0;  // floats
  float* hpix = nullptr;
  HfbsGradState hgs{};
  int hgrad_seg = 0, hgrad_planes = 0;
  bool hgrad_ready = false;  // the last HFBS solve kept its iterates
  HfbsBatch hB{};            // that solve's batch description and parameters
  HParams hhp{};
  Graph g_hbwd;

  // tensor maps of the iterate planes (TMA staging of the iteration) and of
  // the HFBS grid planes (cleared when the grids change)
  TmaCache tma;
  TmaCache htma;

  size_t tsize() const { return st == Storage::F32 ? 4 : 2; }
};

namespace {

void drop_graph(dtsgb_batch_t b, Graph& g) {
  if (g.exec) {
    cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
  }
  prof_drop_captured(&g);
  g.key.clear();
}

void free_grad_planes(dtsgb_batch_t b) {
  for (auto& p : b->gplanes) dfree(p);
  b->gplanes.clear();
}

void select_tiles(dtsgb_batch_t b, bool small) {
  b->small = small;
  b->d_ti = small ? b->d_ti_small : b->d_ti_big;
  b->nti = small ? b->nti_small : b->nti_big;
}

void batch_free(dtsgb_batch_t b) {
  drop_graph(b, b->g_dts);
  drop_graph(b, b->g_hfbs);
  drop_graph(b, b->g_bwd);
  drop_graph(b, b->g_hbwd);
  free_grad_planes(b);
  dfree(b->hgbuf);
  dfree(b->hpix);
  dfree(b->guide);
  dfree(b->target);
  dfree(b->conf);
  dfree(b->bounds);
  dfree(b->v[0]);
  dfree(b->v[1]);
  dfree(b->hout);
  dfree(b->scratch);
  dfree(b->d_inst);
  dfree(b->d_tb);
  dfree(b->d_ti_big);
  dfree(b->d_ti_small);
  b->d_ti = nullptr;
  dfree(b->d_hinst);
  for (auto& p : b->hg) dfree(p);
  dfree(b->ovf);
  dfree(b->sgrid);
  dfree(b->d_soff);
  dfree(b->d_uptr);
  dfree(b->stage);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  b->stream = nullptr;
}

// Planes for the adjoint of an N-iteration solve with segment length seg:
// ceil(N/seg) - 1 checkpoints, seg recompute planes, two adjoint planes and
// the two gradient planes.  Reallocation drops the graphs that captured the
// old pointers.
int ensure_grad_planes(dtsgb_batch_t b, int n_iter, int seg) {
  const int nseg = (n_iter + seg - 1) / seg;
  const size_t need = (size_t)std::max(nseg - 1, 0) + seg + 4;
  if (b->gplanes.size() == need && b->grad_seg == seg) return DTSGB_OK;
  DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  drop_graph(b, b->g_dts);
  drop_graph(b, b->g_bwd);
  free_grad_planes(b);
  b->grad_seg = seg;
  for (size_t k = 0; k < need; ++k) {
    float* p = nullptr;
    int st = dalloc(&p, (size_t)b->total);
    if (st) {
      free_grad_planes(b);
      return st;
    }
    b->gplanes.push_back(p);
  }
  return DTSGB_OK;
}

DtsGrad grad_view(dtsgb_batch_t b, int n_iter) {
  const int seg = b->grad_seg;
  const int ncp = std::max((n_iter + seg - 1) / seg - 1, 0);
  float* const* P = b->gplanes.data();
  DtsGrad G;
  G.seg = seg;
  G.cp = P;
  G.segbuf = P + ncp;
  G.g[0] = P[ncp + seg];
  G.g[1] = P[ncp + seg + 1];
  return G;
}
float* grad_plane_t(dtsgb_batch_t b) { return b->gplanes[b->gplanes.size() - 2]; }
float* grad_plane_c(dtsgb_batch_t b) { return b->gplanes[b->gplanes.size() - 1]; }

// Run `enqueue` directly, or through the solve's CUDA graph (captured on the
// first call with this key, replayed afterwards).
template <typename F>
int run_graph(dtsgb_batch_t b, Graph& g, std::vector<char> key, F enqueue) {
  if (!b->use_graphs) return enqueue();
  key_append(key, prof_enabled());
  if (g.exec && g.key == key) {
    DTSGB_CUDA(cudaGraphLaunch(g.exec, b->stream));
    return DTSGB_OK;
  }
  drop_graph(b, g);
  prof_set_capture_tag(&g);
  cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    prof_set_capture_tag(nullptr);
    return cuda_fail(e, "cudaStreamBeginCapture");
  }
  int st = enqueue();
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(b->stream, &graph);
  prof_set_capture_tag(nullptr);
  if (st) {
    if (graph) cudaGraphDestroy(graph);
    prof_drop_captured(&g);
    return st;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    g.exec = nullptr;
    prof_drop_captured(&g);
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  g.key = key;
  DTSGB_CUDA(cudaGraphLaunch(g.exec, b->stream));
  return DTSGB_OK;
}

int upload_plane(dtsgb_batch_t b, int i, const float* src, void* dst,
                 cudaMemcpyKind kind) {
  const Inst& I = b->inst[i];
  const size_t wb = (size_t)I.w * 4;
  if (b->st == Storage::F32) {
    DTSGB_CUDA(cudaMemcpy2DAsync((float*)dst + I.off, (size_t)I.pitch * 4, src, wb,
                                 wb, I.h, kind, b->stream));
  } else {
    DTSGB_CUDA(cudaMemcpy2DAsync(b->scratch + I.off, (size_t)I.pitch * 4, src, wb,
                                 wb, I.h, kind, b->stream));
  }
  return DTSGB_OK;
}

// Dense staged images -> pitched planes: the guide (color-converted; not
// written when guide is null), target and confidence in the storage type.
template <typename TS>
__global__ void k_ingest(const Inst* __restrict__ insts, const long long* __restrict__ soff,
                         const uchar4* __restrict__ s_rgba, const float* __restrict__ s_t,
                         const float* __restrict__ s_c, uchar4* __restrict__ guide,
                         TS* __restrict__ target, TS* __restrict__ conf, int cs) {
  const Inst I = insts[blockIdx.y];
  const long long so = soff[blockIdx.y];
  for (int y = blockIdx.x; y < I.h; y += gridDim.x) {
    const long long srow = so + (long long)y * I.w, drow = I.off + (long long)y * I.pitch;
    for (int x = threadIdx.x; x < I.w; x += blockDim.x) {
      if (guide) {
        const uchar4 p = s_rgba[srow + x];
        guide[drow + x] = cs == DTSGB_RGB ? p : convert_pixel(p, cs);
      }
      target[drow + x] = store_cast<TS>(s_t[srow + x]);
      conf[drow + x] = store_cast<TS>(s_c[srow + x]);
    }
  }
}

// Dense staged plane -> pitched plane (gradient uploads).  Downloads stay
// row-by-row DMA copies: those need no SM, so in a pipeline they do not wait
// behind another chunk's solve.
__global__ void k_unstage(const Inst* __restrict__ insts, const long long* __restrict__ soff,
                          const float* __restrict__ src, float* __restrict__ dst) {
  const Inst I = insts[blockIdx.y];
  const long long so = soff[blockIdx.y];
  for (int y = blockIdx.x; y < I.h; y += gridDim.x) {
    const long long drow = so + (long long)y * I.w, prow = I.off + (long long)y * I.pitch;
    for (int x = threadIdx.x; x < I.w; x += blockDim.x) dst[prow + x] = src[drow + x];
  }
}

int ensure_stage(dtsgb_batch_t b) {
  if (b->stage) return DTSGB_OK;
  return dalloc(&b->stage, (size_t)b->dense * 12);
}

// Float region k (0..2) of the staging area.
float* stage_plane(dtsgb_batch_t b, int k) {
  return reinterpret_cast<float*>(b->stage + (size_t)b->dense * 4 * k);
}

// n host images -> pitched device plane, through staging region `region`.
int host_upload_plane(dtsgb_batch_t b, const float* const* src, float* dst, int region) {
  int st = ensure_stage(b);
  if (st) return st;
  float* d = stage_plane(b, region);
  for (int i = 0; i < b->n; ++i) {
    const Inst& I = b->inst[i];
    DTSGB_CUDA(cudaMemcpyAsync(d + b->soff[i], src[i], (size_t)I.w * I.h * 4,
                               cudaMemcpyHostToDevice, b->stream));
  }
  const dim3 grid((unsigned)std::min(b->max_h, 512), (unsigned)b->n);
  k_unstage<<<grid, 256, 0, b->stream>>>(b->d_inst, b->d_soff, d, dst);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

// Caller device images (dense W x H, one pointer each; null: skipped) <->
// pitched arena plane: one kernel instead of a row-by-row copy per image.
template <bool TO_ARENA>
__global__ void k_user_copy(const Inst* __restrict__ insts, float* const* __restrict__ user,
                            float* __restrict__ arena) {
  const Inst I = insts[blockIdx.y];
  float* u = user[blockIdx.y];
  if (!u) return;
  for (int y = blockIdx.x; y < I.h; y += gridDim.x) {
    float* urow = u + (long long)y * I.w;
    float* arow = arena + I.off + (long long)y * I.pitch;
    for (int x = threadIdx.x; x < I.w; x += blockDim.x) {
      if (TO_ARENA)
        arow[x] = urow[x];
      else
        urow[x] = arow[x];
    }
  }
}

// Copies between n caller device images and an arena plane (slot 0..2 of the
// pointer table, so that up to three such copies can be in flight in order).
// Send n caller pointers to device slot `slot` unless it already holds them.
// The copy comes from pageable host memory, so the call may wait for the
// stream's earlier work; repeated calls with the same buffers skip it.
int upload_slot(dtsgb_batch_t b, int slot, const void* const* ptrs) {
  const size_t n = (size_t)b->n;
  if (b->uptr_host.size() != 3 * n) b->uptr_host.assign(3 * n, nullptr);
  const void** h = b->uptr_host.data() + slot * n;
  if (b->uptr_valid[slot] && std::memcmp(h, ptrs, sizeof(void*) * n) == 0) return DTSGB_OK;
  DTSGB_CUDA(cudaMemcpyAsync(b->d_uptr + slot * n, ptrs, sizeof(void*) * n,
                             cudaMemcpyHostToDevice, b->stream));
  std::memcpy(h, ptrs, sizeof(void*) * n);
  b->uptr_valid[slot] = true;
  return DTSGB_OK;
}

int user_plane_copy(dtsgb_batch_t b, float* const* user, float* arena, bool to_arena,
                    int slot) {
  float** d = b->d_uptr + (size_t)slot * b->n;
  if (int st = upload_slot(b, slot, reinterpret_cast<const void* const*>(user))) return st;
  const dim3 grid((unsigned)std::min(b->max_h, 512), (unsigned)b->n);
  if (to_arena)
    k_user_copy<true><<<grid, 256, 0, b->stream>>>(b->d_inst, d, arena);
  else
    k_user_copy<false><<<grid, 256, 0, b->stream>>>(b->d_inst, d, arena);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

// Caller device images -> pitched planes (the _device uploads): the guide
// (color-converted; not written when rgba is null), target and confidence in
// the storage type; a null confidence image stands for ones.
template <typename TS>
__global__ void k_ingest_ptr(const Inst* __restrict__ insts, uchar4* const* __restrict__ rgba,
                             float* const* __restrict__ tgt, float* const* __restrict__ cnf,
                             uchar4* __restrict__ guide, TS* __restrict__ target,
                             TS* __restrict__ conf, int cs) {
  const Inst I = insts[blockIdx.y];
  const uchar4* g = rgba ? rgba[blockIdx.y] : nullptr;
  const float* t = tgt[blockIdx.y];
  const float* c = cnf ? cnf[blockIdx.y] : nullptr;
  for (int y = blockIdx.x; y < I.h; y += gridDim.x) {
    const long long srow = (long long)y * I.w, drow = I.off + (long long)y * I.pitch;
    for (int x = threadIdx.x; x < I.w; x += blockDim.x) {
      if (g) {
        const uchar4 p = g[srow + x];
        guide[drow + x] = cs == DTSGB_RGB ? p : convert_pixel(p, cs);
      }
      target[drow + x] = store_cast<TS>(t[srow + x]);
      conf[drow + x] = store_cast<TS>(c ? c[srow + x] : 1.f);
    }
  }
}

int device_ingest(dtsgb_batch_t b, int cs, const void* const* rgba,
                  const float* const* target, const float* const* conf) {
  const size_t n = (size_t)b->n;
  float** slots = b->d_uptr;  // [rgba | target | confidence]
  std::vector<const void*> cf(n, nullptr);
  if (conf)
    for (size_t i = 0; i < n; ++i) cf[i] = conf[i];
  int st = DTSGB_OK;
  if (rgba) st = upload_slot(b, 0, rgba);
  if (!st) st = upload_slot(b, 1, reinterpret_cast<const void* const*>(target));
  if (!st) st = upload_slot(b, 2, cf.data());
  if (st) return st;
  // the pointer copies come from pageable host memory: the calls return
  // once the arrays are copied out, so cf may go out of scope
  const dim3 grid((unsigned)std::min(b->max_h, 512), (unsigned)b->n);
  uchar4* const* rp = rgba ? reinterpret_cast<uchar4* const*>(slots) : nullptr;
  uchar4* g = rgba ? b->guide : nullptr;
  if (b->st == Storage::F32)
    k_ingest_ptr<float><<<grid, 256, 0, b->stream>>>(b->d_inst, rp, slots + n, slots + 2 * n,
                                                     g, (float*)b->target, (float*)b->conf,
                                                     cs);
  else
    k_ingest_ptr<__nv_bfloat16><<<grid, 256, 0, b->stream>>>(
        b->d_inst, rp, slots + n, slots + 2 * n, g, (__nv_bfloat16*)b->target,
        (__nv_bfloat16*)b->conf, cs);
  DTSGB_CUDA(cudaGetLastError());
  if (rgba) ++b->guide_gen;
  b->dts_res = -1;
  b->grad_n = -1;
  b->hfbs_done = false;
  b->hgrad_ready = false;
  return DTSGB_OK;
}

// Host upload: one contiguous copy per image and plane into the staging
// area (pinned host memory makes them asynchronous), ones for missing
// confidences, then k_ingest.  rgba null: targets only (guides kept).
int host_ingest(dtsgb_batch_t b, int cs, const void* const* rgba,
                const float* const* target, const float* const* conf, bool sync_host) {
  if (int st = ensure_stage(b)) return st;
  uchar4* s_rgba = reinterpret_cast<uchar4*>(b->stage);
  float* s_t = reinterpret_cast<float*>(b->stage + (size_t)b->dense * 4);
  float* s_c = reinterpret_cast<float*>(b->stage + (size_t)b->dense * 8);
  for (int i = 0; i < b->n; ++i) {
    const Inst& I = b->inst[i];
    const size_t px = (size_t)I.w * I.h;
    const long long o = b->soff[i];
    if (rgba)
      DTSGB_CUDA(cudaMemcpyAsync(s_rgba + o, rgba[i], px * 4, cudaMemcpyHostToDevice,
                                 b->stream));
    DTSGB_CUDA(cudaMemcpyAsync(s_t + o, target[i], px * 4, cudaMemcpyHostToDevice,
                               b->stream));
    if (conf && conf[i]) {
      DTSGB_CUDA(cudaMemcpyAsync(s_c + o, conf[i], px * 4, cudaMemcpyHostToDevice,
                                 b->stream));
    } else {
      int st = launch_fill_storage(Storage::F32, s_c + o, (long long)px, 1.f, b->stream);
      if (st) return st;
    }
  }
  const dim3 grid((unsigned)std::min(b->max_h, 512), (unsigned)b->n);
  uchar4* g = rgba ? b->guide : nullptr;
  if (b->st == Storage::F32)
    k_ingest<float><<<grid, 256, 0, b->stream>>>(b->d_inst, b->d_soff, s_rgba, s_t, s_c, g,
                                                 (float*)b->target, (float*)b->conf, cs);
  else
    k_ingest<__nv_bfloat16><<<grid, 256, 0, b->stream>>>(
        b->d_inst, b->d_soff, s_rgba, s_t, s_c, g, (__nv_bfloat16*)b->target,
        (__nv_bfloat16*)b->conf, cs);
  DTSGB_CUDA(cudaGetLastError());
  if (rgba) ++b->guide_gen;
  b->dts_res = -1;
  b->grad_n = -1;
  b->hfbs_done = false;
  b->hgrad_ready = false;
  if (sync_host) DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  return DTSGB_OK;
}

// sync_host: a host upload returns only when the copies are done (the
// reference's CopyTo semantics; the host buffers may be reused at once).
int batch_upload_targets(dtsgb_batch_t b, const float* const* target,
                         const float* const* conf, cudaMemcpyKind kind,
                         bool sync_host = true) {
  if (kind == cudaMemcpyHostToDevice)
    return host_ingest(b, DTSGB_RGB, nullptr, target, conf, sync_host);
  if (kind == cudaMemcpyDeviceToDevice) return device_ingest(b, DTSGB_RGB, nullptr, target, conf);
  int st;
  for (int i = 0; i < b->n; ++i)
    if ((st = upload_plane(b, i, target[i], b->target, kind))) return st;
  if (b->st == Storage::BF16 &&
      (st = launch_storage_from_float(nullptr, 0, b->st, b->scratch, b->target,
                                      b->total, b->stream)))
    return st;
  // confidence (missing -> ones)
  for (int i = 0; i < b->n; ++i) {
    const Inst& I = b->inst[i];
    if (conf && conf[i]) {
      if ((st = upload_plane(b, i, conf[i], b->conf, kind))) return st;
    } else if (b->st == Storage::F32) {
      if ((st = launch_fill_storage(Storage::F32, (float*)b->conf + I.off,
                                    (long long)I.pitch * I.h, 1.f, b->stream)))
        return st;
    } else {
      if ((st = launch_fill_storage(Storage::F32, b->scratch + I.off,
                                    (long long)I.pitch * I.h, 1.f, b->stream)))
        return st;
    }
  }
  if (b->st == Storage::BF16 &&
      (st = launch_storage_from_float(nullptr, 0, b->st, b->scratch, b->conf,
                                      b->total, b->stream)))
    return st;
  b->dts_res = -1;
  b->grad_n = -1;
  b->hfbs_done = false;
  b->hgrad_ready = false;
  if (kind == cudaMemcpyHostToDevice && sync_host)
    DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  return DTSGB_OK;
}

int batch_upload(dtsgb_batch_t b, int cs, const void* const* rgba,
                 const float* const* target, const float* const* conf,
                 cudaMemcpyKind kind, bool sync_host = true) {
  if (!b || !rgba || !target) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (cs < DTSGB_RGB || cs > DTSGB_YYY)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid color space");
  for (int i = 0; i < b->n; ++i)
    if (!rgba[i] || !target[i])
      return fail(DTSGB_ERR_INVALID_ARGUMENT, "null image pointer");
  if (kind == cudaMemcpyHostToDevice)
    return host_ingest(b, cs, rgba, target, conf, sync_host);
  if (kind == cudaMemcpyDeviceToDevice) return device_ingest(b, cs, rgba, target, conf);
  for (int i = 0; i < b->n; ++i) {
    const Inst& I = b->inst[i];
    const size_t wb = (size_t)I.w * 4;
    DTSGB_CUDA(cudaMemcpy2DAsync(b->guide + I.off, (size_t)I.pitch * 4, rgba[i], wb,
                                 wb, I.h, kind, b->stream));
  }
  int st = launch_color_convert_flat(b->guide, b->total, cs, b->stream);
  if (st) return st;
  ++b->guide_gen;
  return batch_upload_targets(b, target, conf, kind, sync_host);
}

// The HFBS gradient arena for K heavy-ball steps over tv voxels (the choice
// of segment as for the DTS checkpoints: every iterate when that fits in a
// quarter of the free device memory, else about sqrt(K) steps), and the
// three pixel planes of the backward.
int hfbs_prepare_grad(dtsgb_batch_t b, int K, long long tv) {
  int S = b->grad_seg_req;
  if (K <= 1) S = 1;
  if (S <= 0 && b->hgrad_seg == 1 && b->hgcap >= (size_t)(hfbs_grad_planes(K, 1) * tv))
    S = 1;  // every iterate already held: no memory query
  if (S <= 0) {
    size_t fr = 0, tot = 0;
    DTSGB_CUDA(cudaMemGetInfo(&fr, &tot));
    const double avail = (double)fr + (double)b->hgcap * 4.0;
    S = (double)hfbs_grad_planes(K, 1) * tv * 4.0 <= avail / 4
            ? 1
            : std::max(2, (int)std::ceil(std::sqrt((double)K)));
  }
  S = std::min(S, std::max(K, 1));
  const long long need = hfbs_grad_planes(K, S) * tv;
  if ((size_t)need > b->hgcap) {
    DTSGB_CUDA(cudaStreamSynchronize(b->stream));  // a backward may still read it
    dfree(b->hgbuf);
    b->hgcap = 0;
    if (int st = dalloc(&b->hgbuf, (size_t)need)) return st;
    b->hgcap = (size_t)need;
    drop_graph(b, b->g_hbwd);
  }
  if (!b->hpix) {
    if (int st = dalloc(&b->hpix, (size_t)(3 * b->total))) return st;
  }
  hfbs_carve_grad(b->hgs, b->hgbuf, K, S, tv);
  b->hgrad_seg = S;
  b->hgrad_planes = (int)hfbs_grad_planes(K, S);
  return DTSGB_OK;
}

int ensure_hfbs_buffers(dtsgb_batch_t b, long long voxels, long long planes,
                        long long slice_voxels) {
  if (voxels > b->gcap) {
    for (auto& p : b->hg) dfree(p);
    b->gcap = 0;
    b->nkey.gen = ~0ull;  // the normalisation is gone with the old planes
    for (int k = 0; k < HG_NUM; ++k) {
      int st = dalloc(&b->hg[k], (size_t)voxels);
      if (st) return st;
    }
    b->gcap = voxels;
    drop_graph(b, b->g_hfbs);
  }
  if (planes > b->ocap) {
    dfree(b->ovf);
    int st = dalloc(&b->ovf, (size_t)planes);
    if (st) return st;
    b->ocap = planes;
    drop_graph(b, b->g_hfbs);
  }
  if (slice_voxels > b->scap) {
    dfree(b->sgrid);
    int st = dalloc(&b->sgrid, (size_t)slice_voxels);
    if (st) return st;
    b->scap = slice_voxels;
    drop_graph(b, b->g_hfbs);
  }
  return DTSGB_OK;
}

}  // namespace

namespace {
// Mean device time of `reps` runs of `run` on the batch stream (after one
// untimed run, which also captures the graph).
template <typename F>
int time_runs(dtsgb_batch_t b, int reps, F run, float* ms) {
  int st = run();
  if (st) return st;
  cudaEvent_t e0, e1;
  DTSGB_CUDA(cudaEventCreate(&e0));
  cudaError_t e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_fail(e, "cudaEventCreate");
  }
  e = cudaEventRecord(e0, b->stream);
  for (int r = 0; r < reps && !st && e == cudaSuccess; ++r) st = run();
  if (!st && e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
  if (!st && e == cudaSuccess) e = cudaEventSynchronize(e1);
  float t = 0.f;
  if (!st && e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if (e != cudaSuccess) return cuda_fail(e, "autotune timing");
  *ms = t / reps;
  return DTSGB_OK;
}
}  // namespace

extern "C" {

DTSGB_API int dtsgb_batch_create(int n, const int* widths, const int* heights,
                                 unsigned flags, dtsgb_batch_t* out) {
  if (!out || !widths || !heights || n <= 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "bad batch description");
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (widths[i] <= 0 || heights[i] <= 0)
      return fail(DTSGB_ERR_INVALID_DIMS, "instance dims must be positive");
  dtsgb_batch_t b = new dtsgb_batch_s();
  b->n = n;
  b->flags = flags;
  b->st = (flags & DTSGB_FLAG_BF16_STORAGE) ? Storage::BF16 : Storage::F32;
  b->ref_y = (flags & DTSGB_FLAG_FIX_Y_LIMIT) ? 0 : 1;
  std::vector<Tile> tb, ti, ts;
  long long off = 0, tiles64 = 0;
  for (int i = 0; i < n; ++i)
    tiles64 += (long long)((widths[i] + kIterTW - 1) / kIterTW) *
               ((heights[i] + kIterTH - 1) / kIterTH);
  b->small = use_small_iter_tiles(tiles64);
  for (int i = 0; i < n; ++i) {
    Inst I{widths[i], heights[i], round_up(widths[i], 32), 0, off};
    b->inst.push_back(I);
    b->soff.push_back(b->dense);
    b->dense += (long long)widths[i] * heights[i];
    off += (long long)I.pitch * I.h;
    b->max_w = std::max(b->max_w, I.w);
    b->max_h = std::max(b->max_h, I.h);
    for (int y = 0; y < I.h; y += kBoundsTH)
      for (int x = 0; x < I.w; x += kBoundsTW) tb.push_back(Tile{i, x, y, 0});
    for (int y = 0; y < I.h; y += kIterTH)
      for (int x = 0; x < I.w; x += kIterTW) ti.push_back(Tile{i, x, y, 0});
    for (int y = 0; y < I.h; y += kIterSmallTH)
      for (int x = 0; x < I.w; x += kIterSmallTW) ts.push_back(Tile{i, x, y, 0});
  }
  b->total = off;
  b->ntb = (int)tb.size();
  b->nti_big = (int)ti.size();
  b->nti_small = (int)ts.size();
  int st = DTSGB_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "cudaStreamCreate");
  }
  b->own_stream = true;
  const size_t T = (size_t)b->total;
  if (!st) st = dalloc(&b->guide, T);
  if (!st) st = dalloc((char**)&b->target, T * b->tsize());
  if (!st) st = dalloc((char**)&b->conf, T * b->tsize());
  if (!st) st = dalloc(&b->bounds, T);
  if (!st) st = dalloc(&b->v[0], T);
  if (!st) st = dalloc(&b->v[1], T);
  if (!st) st = dalloc(&b->hout, T);
  if (!st && b->st == Storage::BF16) st = dalloc(&b->scratch, T);
  if (!st) st = dalloc(&b->d_inst, (size_t)n);
  if (!st) st = dalloc(&b->d_tb, tb.size());
  if (!st) st = dalloc(&b->d_ti_big, ti.size());
  if (!st) st = dalloc(&b->d_ti_small, ts.size());
  if (!st) st = dalloc(&b->d_hinst, (size_t)n);
  if (!st) st = dalloc(&b->d_soff, (size_t)n);
  if (!st) st = dalloc(&b->d_uptr, (size_t)3 * n);
  if (!st) {
    e = cudaMemcpy(b->d_inst, b->inst.data(), n * sizeof(Inst), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_soff, b->soff.data(), n * sizeof(long long), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_tb, tb.data(), tb.size() * sizeof(Tile), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_ti_big, ti.data(), ti.size() * sizeof(Tile),
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_ti_small, ts.data(), ts.size() * sizeof(Tile),
                     cudaMemcpyHostToDevice);
    if (e != cudaSuccess) st = cuda_fail(e, "batch tables");
  }
  select_tiles(b, b->small);
  if (st) {
    batch_free(b);
    delete b;
    return st;
  }
  *out = b;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_destroy(dtsgb_batch_t b) {
  if (!b) return DTSGB_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_free(b);
  delete b;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_set_stream(dtsgb_batch_t b, void* stream) {
  if (!b) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  if (b->own_stream) cudaStreamDestroy(b->stream);
  b->own_stream = false;
  b->stream = (cudaStream_t)stream;
  if (!stream) {
    DTSGB_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->own_stream = true;
  }
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_use_graphs(dtsgb_batch_t b, int enable) {
  if (!b) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  b->use_graphs = enable != 0;
  if (!b->use_graphs) {
    drop_graph(b, b->g_dts);
    drop_graph(b, b->g_hfbs);
  }
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_upload(dtsgb_batch_t b, int cs, const void* const* rgba,
                                 const float* const* target,
                                 const float* const* conf) {
  return batch_upload(b, cs, rgba, target, conf, cudaMemcpyHostToDevice);
}

DTSGB_API int dtsgb_batch_upload_targets(dtsgb_batch_t b, const float* const* target,
                                         const float* const* conf) {
  if (!b || !target) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  for (int i = 0; i < b->n; ++i)
    if (!target[i]) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null image pointer");
  return batch_upload_targets(b, target, conf, cudaMemcpyHostToDevice);
}

DTSGB_API int dtsgb_batch_upload_targets_device(dtsgb_batch_t b,
                                                const float* const* target,
                                                const float* const* conf) {
  if (!b || !target) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  for (int i = 0; i < b->n; ++i)
    if (!target[i]) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null image pointer");
  return batch_upload_targets(b, target, conf, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_batch_upload_device(dtsgb_batch_t b, int cs,
                                        const void* const* rgba,
                                        const float* const* target,
                                        const float* const* conf) {
  return batch_upload(b, cs, rgba, target, conf, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_batch_solve_dts(dtsgb_batch_t b, const dtsgb_filter_params* f,
                                    const dtsgb_optimize_params* p,
                                    float overwrite) {
  if (!b || !f || !p) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (!finite_pos(f->sigma_x) || !finite_pos(f->sigma_y) || !finite_pos(f->sigma_r))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "filter sigmas must be finite, positive");
  if (p->loss < DTSGB_L1 || p->loss > DTSGB_CHARBONNIER)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "invalid loss");
  if (p->num_iterations < 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "num_iterations < 0");
  if (!finite_pos(p->sigma_z) || p->sigma_z >= 254.f)
    return fail(DTSGB_ERR_UNSUPPORTED, "sigma_z must be in (0, 254)");
  const float rx = f->sigma_x / f->sigma_r, ry = f->sigma_y / f->sigma_r;
  const int halo = (int)std::floor(p->sigma_z);
  const bool iterate = p->loss != DTSGB_L1 && p->num_iterations > 0;
  DtsLaunch Lb{b->d_inst, b->d_tb, b->ntb, b->n};
  Lb.bounds_seg = b->bounds_seg;
  const DtsLaunch Li{b->d_inst, b->d_ti, b->nti, b->n, b->small, b->d_ti_small,
                     b->nti_small, &b->tma, b->inst.data()};
  // the iterate planes' tensor maps exist before any capture (a capture
  // cannot build them: the kernels would stage by loads)
  {
    int bw = 0, bh = 0;
    dts_iter_tma_box(Li, halo, halo, &bw, &bh);
    if (bw > 0)
      for (float* v : b->v) (void)b->tma.get(b->inst.data(), b->n, v, bw, bh, b->stream);
  }
  const bool over = overwrite > 0.f && overwrite < 1.f;
  const int n_kept = iterate ? p->num_iterations : 0;
  b->grad_n = -1;
  if (b->grad) {
    if (iterate && over)
      return fail(DTSGB_ERR_UNSUPPORTED,
                  "gradients are not available with the confidence overwrite");
    int seg = b->grad_seg_req;
    if (seg <= 0) {
      // automatic: every iterate kept (nothing recomputed by the backward)
      // when its N + 4 planes fit in a quarter of the free device memory (or
      // are held already), else the fewest planes
      const int n = std::max(n_kept, 1);
      const size_t need = (size_t)(n + 4) * (size_t)b->total * sizeof(float);
      size_t free_b = 0, total_b = 0;
      const bool held = b->grad_seg == 1 && b->gplanes.size() == (size_t)n + 4;
      if (!held) DTSGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
      seg = held || need <= free_b / 4 ? 1 : dts_checkpoint_segment(n);
    }
    int st = ensure_grad_planes(b, n_kept, seg);
    if (st) return st;
  }
  int res = 0;
  const dtsgb_batch_s::BoundsKey bk{b->guide_gen, rx, ry, p->sigma_z, b->ref_y};
  const bool keep_bounds = b->reuse && std::memcmp(&bk, &b->bkey, sizeof bk) == 0;
  auto bounds = [&]() -> int {
    if (keep_bounds) return DTSGB_OK;  // same guide and sigmas: windows unchanged
    return launch_bounds(Lb, b->guide, b->bounds, rx, ry, p->sigma_z, p->sigma_z,
                         b->ref_y, b->stream);
  };
  auto enqueue = [&]() -> int {
    if (b->grad && iterate) {
      const IterMode mode = p->loss == DTSGB_L2 ? IterMode::L2 : IterMode::CHARB;
      int st = bounds();
      if (st) return st;
      return dts_forward_checkpointed(Li, b->st, mode, grad_view(b, n_kept), b->target,
                                      b->conf, b->bounds, p->lambda, p->step_size, halo,
                                      p->num_iterations, b->v[0], b->v[1], &res,
                                      b->stream);
    }
    int st = launch_init_var(Li, b->st, b->target, b->v[0], b->stream);
    if (st || !iterate) return st;
    st = bounds();
    if (st) return st;
    const IterMode mode = p->loss == DTSGB_L2 ? IterMode::L2 : IterMode::CHARB;
    int a = 0;
    for (int it = 0; it < p->num_iterations; ++it) {
      st = launch_dts_iter(Li, b->st, mode, b->v[a], b->v[1 - a], b->target,
                           b->conf, b->bounds, p->lambda, p->step_size, overwrite,
                           halo, halo, b->stream);
      if (st) return st;
      a = 1 - a;
    }
    return DTSGB_OK;
  };
  res = iterate ? (b->grad ? dts_checkpointed_result_index(p->num_iterations, b->grad_seg)
                           : p->num_iterations % 2)
                : 0;
  std::vector<char> key;
  key_append(key, *f);
  key_append(key, *p);
  key_append(key, overwrite);
  key_append(key, b->grad);
  key_append(key, b->grad_seg);
  key_append(key, b->small);
  key_append(key, keep_bounds);
  key_append(key, b->bounds_seg);
  int st = run_graph(b, b->g_dts, key, enqueue);
  if (st) {
    b->bkey.gen = ~0ull;
    return st;
  }
  if (iterate) b->bkey = bk;
  b->dts_res = res;
  if (b->grad) {
    b->grad_n = n_kept;
    b->gopt = *p;
    b->ghalo = (float)halo;
  }
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_enable_grad(dtsgb_batch_t b, int enable, int segment) {
  if (!b) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if (segment < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "segment < 0");
  if (b->grad != (enable != 0) || b->grad_seg_req != segment) {
    DTSGB_CUDA(cudaStreamSynchronize(b->stream));
    drop_graph(b, b->g_dts);
    drop_graph(b, b->g_bwd);
    drop_graph(b, b->g_hfbs);
    drop_graph(b, b->g_hbwd);
  }
  b->grad = enable != 0;
  b->grad_seg_req = segment;
  b->grad_n = -1;
  b->hgrad_ready = false;
  if (!b->grad) {
    free_grad_planes(b);
    dfree(b->hgbuf);
    dfree(b->hpix);
    b->hgcap = 0;
    b->hgrad_seg = b->hgrad_planes = 0;
  }
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_grad_info(dtsgb_batch_t b, int* segment, int* planes) {
  if (!b || !segment || !planes) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  *segment = b->grad_n >= 0 ? b->grad_seg : 0;
  *planes = (int)b->gplanes.size();
  return DTSGB_OK;
}

static int batch_backward(dtsgb_batch_t b, const float* const* grad_out,
                          float* const* grad_t, float* const* grad_c,
                          cudaMemcpyKind up, cudaMemcpyKind down, bool sync_host = true) {
  if (!b || !grad_out) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (b->grad_n < 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT,
                "no DTS solve with gradients enabled since the last upload");
  for (int i = 0; i < b->n; ++i)
    if (!grad_out[i]) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null gradient pointer");
  const int n_iter = b->grad_n;
  DtsGrad G = grad_view(b, n_iter);
  if (up == cudaMemcpyHostToDevice) {
    if (int st = host_upload_plane(b, grad_out, G.g[0], 0)) return st;
  } else {
    if (int st = user_plane_copy(b, const_cast<float* const*>(grad_out), G.g[0], true, 0))
      return st;
  }
  const DtsLaunch Li{b->d_inst, b->d_ti, b->nti, b->n, b->small, b->d_ti_small,
                     b->nti_small};
  const dtsgb_optimize_params p = b->gopt;
  const int halo = (int)b->ghalo;
  auto enqueue = [&]() -> int {
    const IterMode mode = p.loss == DTSGB_L2 ? IterMode::L2 : IterMode::CHARB;
    return dts_backward(Li, b->d_inst, b->n, b->total, b->st, mode, G, b->target, b->conf,
                        b->bounds, p.lambda, p.step_size, halo, n_iter, grad_plane_t(b),
                        grad_plane_c(b), b->stream);
  };
  std::vector<char> key;
  key_append(key, p);
  key_append(key, n_iter);
  key_append(key, b->grad_seg);
  key_append(key, b->small);
  int st = run_graph(b, b->g_bwd, key, enqueue);
  if (st) return st;
  for (int k = 0; k < 2; ++k) {
    float* const* dst = k == 0 ? grad_t : grad_c;
    const float* src = k == 0 ? grad_plane_t(b) : grad_plane_c(b);
    if (!dst) continue;
    if (down == cudaMemcpyDeviceToDevice) {
      if (int st = user_plane_copy(b, dst, const_cast<float*>(src), false, 1 + k)) return st;
      continue;
    }
    for (int i = 0; i < b->n; ++i) {
      if (!dst[i]) continue;
      const Inst& I = b->inst[i];
      const size_t wb = (size_t)I.w * 4;
      DTSGB_CUDA(cudaMemcpy2DAsync(dst[i], wb, src + I.off, (size_t)I.pitch * 4, wb, I.h,
                                   down, b->stream));
    }
  }
  if (down == cudaMemcpyDeviceToHost && sync_host)
    DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_dts_backward(dtsgb_batch_t b, const float* const* grad_out,
                                       float* const* grad_target,
                                       float* const* grad_confidence) {
  return batch_backward(b, grad_out, grad_target, grad_confidence, cudaMemcpyHostToDevice,
                        cudaMemcpyDeviceToHost);
}

DTSGB_API int dtsgb_batch_dts_backward_device(dtsgb_batch_t b,
                                              const float* const* grad_out,
                                              float* const* grad_target,
                                              float* const* grad_confidence) {
  return batch_backward(b, grad_out, grad_target, grad_confidence,
                        cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_batch_solve_hfbs(dtsgb_batch_t b, const dtsgb_hfbs_params* p) {
  if (!b || !p) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (!finite_pos(p->sigma_x) || !finite_pos(p->sigma_y) || !finite_pos(p->sigma_l))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "grid sigmas must be finite, positive");
  if (p->bistoch_iter_max < 0 || p->optim_iter_max < 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "iteration counts must be >= 0");
  const int gl = (int)std::ceil(255.0 / (double)p->sigma_l);
  if (gl > 256) return fail(DTSGB_ERR_UNSUPPORTED, "more than 256 luma bins");
  std::vector<HInst> hi(b->n);
  long long goff = 0, poff = 0, soff = 0, max_vox = 0, max_px = 0, max_cells = 0,
            max_lines = 0;
  for (int i = 0; i < b->n; ++i) {
    const Inst& I = b->inst[i];
    HInst& H = hi[i];
    H.w = I.w;
    H.h = I.h;
    H.pitch = I.pitch;
    H.gx = (int)std::ceil((float)I.w / p->sigma_x);
    H.gy = (int)std::ceil((float)I.h / p->sigma_y);
    H.gl = gl;
    H.px = round_up(H.gx, 4);
    H.cov_x = H.gx % 8 != 0;
    H.cov_y = H.gy % 8 != 0;
    H.cov_l = H.gl % 8 != 0;
    H.ovf_stored = 1;
    H.pix_off = I.off;
    H.grid_off = goff;
    H.plane_off = poff;
    H.slice_off = soff;
    soff += round_up_ll((long long)(H.gx + 1) * (H.gy + 1) * (H.gl + 2), 32);
    const long long vox = (long long)H.gx * H.gy * H.gl;
    goff += round_up_ll((long long)H.px * H.gy * H.gl, 32);
    poff += round_up_ll((long long)H.gx * H.gy, 32);
    max_vox = std::max(max_vox, vox);
    max_px = std::max(max_px, (long long)I.w * I.h);
    max_cells = std::max(max_cells, (long long)H.gx * H.gy);
    max_lines = std::max({max_lines, (long long)H.gy * H.gl, (long long)H.gx * H.gl,
                          (long long)H.gx * H.gy});
  }
  int st = ensure_hfbs_buffers(b, goff, poff, soff);
  if (st) return st;
  const bool same_tables =
      b->hinst.size() == hi.size() &&
      std::memcmp(b->hinst.data(), hi.data(), hi.size() * sizeof(HInst)) == 0;
  if (!same_tables) {
    b->htma.clear();
    b->hinst = hi;
    DTSGB_CUDA(cudaMemcpyAsync(b->d_hinst, b->hinst.data(), hi.size() * sizeof(HInst),
                               cudaMemcpyHostToDevice, b->stream));
    DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  }
  HfbsBatch B{};
  B.d_inst = b->d_hinst;
  B.n_inst = b->n;
  B.max_voxels = max_vox;
  B.total_voxels = goff;
  B.max_pixels = max_px;
  B.max_cells = max_cells;
  B.max_lines = max_lines;
  B.max_rows = 0;
  for (const HInst& H : hi) B.max_rows = std::max(B.max_rows, (long long)H.gy * H.gl);
  B.max_gl = gl;
  B.guide = b->guide;
  B.target = b->target;
  B.conf = b->conf;
  B.st = b->st;
  B.out = b->hout;
  B.count = b->hg[HG_COUNT];
  B.csum = b->hg[HG_CSUM];
  B.b = b->hg[HG_B];
  B.n0 = b->hg[HG_N0];
  B.n1 = b->hg[HG_N1];
  B.invA = b->hg[HG_INVA];
  B.z0 = b->hg[HG_Z0];
  B.z1 = b->hg[HG_Z1];
  B.h = b->hg[HG_H];
  B.t0 = b->hg[HG_T0];
  B.t1 = b->hg[HG_T1];
  B.t2 = b->hg[HG_T2];
  B.sgrid = b->sgrid;
  B.ovf = b->ovf;
  B.keep_debug = false;
  B.h_inst = b->hinst.data();
  B.group_voxels = b->hfbs_group_voxels;
  B.solve_steps = b->hfbs_solve_steps;
  B.tma = &b->htma;
  // the bistochastized normalisation depends only on the guide's bins
  const dtsgb_batch_s::NormKey nk{b->guide_gen, p->sigma_x, p->sigma_y, p->sigma_l,
                                  p->bistoch_iter_max};
  B.reuse_norm = b->reuse && same_tables && std::memcmp(&nk, &b->nkey, sizeof nk) == 0;
  HParams hp{p->sigma_x, p->sigma_y, p->sigma_l, p->lambda, p->alpha, p->beta,
             p->bistoch_iter_max, p->optim_iter_max, p->neg_exp_beta};
  b->hgrad_ready = false;
  if (b->grad) {
    if ((st = hfbs_prepare_grad(b, p->optim_iter_max, goff))) return st;
    B.grad = &b->hgs;
  }
  hfbs_prepare_tma(B, b->stream);  // before any capture of the solve
  std::vector<char> key;
  key_append(key, hp);
  key_append(key, b->hfbs_group_voxels);
  key_append(key, b->hfbs_solve_steps);
  key_append(key, B.reuse_norm);
  key_append(key, b->grad ? b->hgbuf : nullptr);  // the kept iterates' arena
  key_append(key, b->grad ? b->hgrad_seg : 0);
  st = run_graph(b, b->g_hfbs, key, [&]() { return hfbs_enqueue_solve(B, hp, b->stream); });
  if (st) {
    b->nkey.gen = ~0ull;
    return st;
  }
  b->nkey = nk;
  b->hfbs_done = true;
  if (b->grad) {
    b->hB = B;
    b->hhp = hp;
    b->hgrad_ready = true;
  }
  return DTSGB_OK;
}

// Adjoint of the last differentiable dtsgb_batch_solve_hfbs (the HFBS
// counterpart of batch_backward): upstream gradients in, dL/dtarget and
// dL/dconfidence out, the launch sequence replayed from a CUDA graph.
static int batch_hfbs_backward(dtsgb_batch_t b, const float* const* grad_out,
                               float* const* grad_t, float* const* grad_c,
                               cudaMemcpyKind up, cudaMemcpyKind down) {
  if (!b || !grad_out) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (!b->hgrad_ready)
    return fail(DTSGB_ERR_INVALID_ARGUMENT,
                "no HFBS solve with gradients enabled since the last upload");
  for (int i = 0; i < b->n; ++i)
    if (!grad_out[i]) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null gradient pointer");
  float* gout = b->hpix;
  float* gt = b->hpix + b->total;
  float* gc = b->hpix + 2 * b->total;
  if (up == cudaMemcpyHostToDevice) {
    if (int st = host_upload_plane(b, grad_out, gout, 0)) return st;
  } else {
    if (int st = user_plane_copy(b, const_cast<float* const*>(grad_out), gout, true, 0))
      return st;
  }
  std::vector<char> key;
  key_append(key, b->hhp);
  key_append(key, b->hgbuf);
  key_append(key, b->hgrad_seg);
  key_append(key, b->hB.total_voxels);
  int st = run_graph(b, b->g_hbwd, key,
                     [&]() { return hfbs_enqueue_backward(b->hB, b->hhp, gout, gt, gc, b->stream); });
  if (st) return st;
  for (int k = 0; k < 2; ++k) {
    float* const* dst = k == 0 ? grad_t : grad_c;
    const float* src = k == 0 ? gt : gc;
    if (!dst) continue;
    if (down == cudaMemcpyDeviceToDevice) {
      if (int st = user_plane_copy(b, dst, const_cast<float*>(src), false, 1 + k)) return st;
      continue;
    }
    for (int i = 0; i < b->n; ++i) {
      if (!dst[i]) continue;
      const Inst& I = b->inst[i];
      const size_t wb = (size_t)I.w * 4;
      DTSGB_CUDA(cudaMemcpy2DAsync(dst[i], wb, src + I.off, (size_t)I.pitch * 4, wb, I.h,
                                   down, b->stream));
    }
  }
  if (down == cudaMemcpyDeviceToHost) DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_hfbs_backward(dtsgb_batch_t b, const float* const* grad_out,
                                        float* const* grad_target,
                                        float* const* grad_confidence) {
  return batch_hfbs_backward(b, grad_out, grad_target, grad_confidence,
                             cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost);
}

DTSGB_API int dtsgb_batch_hfbs_backward_device(dtsgb_batch_t b, const float* const* grad_out,
                                               float* const* grad_target,
                                               float* const* grad_confidence) {
  return batch_hfbs_backward(b, grad_out, grad_target, grad_confidence,
                             cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_batch_hfbs_grad_info(dtsgb_batch_t b, int* segment, int* planes) {
  if (!b || !segment || !planes) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  *segment = b->hgrad_ready ? b->hgrad_seg : 0;
  *planes = b->hgrad_ready ? b->hgrad_planes : 0;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_set_tuning(dtsgb_batch_t b, int knob, long long value) {
  if (!b) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if (knob == DTSGB_TUNE_DTS_TILE) {
    if (value != kIterTW && value != kIterSmallTW)
      return fail(DTSGB_ERR_INVALID_ARGUMENT, "DTS tile must be 64 or 32");
    const bool small = value == kIterSmallTW;
    if (small != b->small) {
      select_tiles(b, small);
      b->grad_n = -1;  // checkpoints were computed with the other tile shape
    }
    return DTSGB_OK;
  }
  if (knob == DTSGB_TUNE_HFBS_GROUP_VOXELS) {
    if (value < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "group budget < 0");
    b->hfbs_group_voxels = value;
    return DTSGB_OK;
  }
  if (knob == DTSGB_TUNE_REUSE_GUIDE_STATE) {
    b->reuse = value != 0;
    return DTSGB_OK;
  }
  if (knob == DTSGB_TUNE_BOUNDS_SEGMENT) {
    if (value != 4 && value != 8 && value != 16)
      return fail(DTSGB_ERR_INVALID_ARGUMENT, "bounds segment must be 4, 8 or 16");
    b->bounds_seg = (int)value;
    return DTSGB_OK;
  }
  if (knob == DTSGB_TUNE_HFBS_SOLVE_STEPS) {
    if (value != 1 && value != kHfbsTBSteps)
      return fail(DTSGB_ERR_INVALID_ARGUMENT, "HFBS steps per launch must be 1 or 4");
    if (value != b->hfbs_solve_steps) b->hgrad_ready = false;  // kept iterates' arithmetic
    b->hfbs_solve_steps = (int)value;
    return DTSGB_OK;
  }
  return fail(DTSGB_ERR_INVALID_ARGUMENT, "unknown tuning knob");
}

DTSGB_API int dtsgb_batch_get_tuning(dtsgb_batch_t b, int knob, long long* value) {
  if (!b || !value) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (knob == DTSGB_TUNE_DTS_TILE) {
    *value = b->small ? kIterSmallTW : kIterTW;
    return DTSGB_OK;
  }
  if (knob == DTSGB_TUNE_HFBS_GROUP_VOXELS) {
    *value = b->hfbs_group_voxels;
    return DTSGB_OK;
  }
  if (knob == DTSGB_TUNE_REUSE_GUIDE_STATE) {
    *value = b->reuse ? 1 : 0;
    return DTSGB_OK;
  }
  if (knob == DTSGB_TUNE_HFBS_SOLVE_STEPS) {
    *value = b->hfbs_solve_steps;
    return DTSGB_OK;
  }
  if (knob == DTSGB_TUNE_BOUNDS_SEGMENT) {
    *value = b->bounds_seg;
    return DTSGB_OK;
  }
  return fail(DTSGB_ERR_INVALID_ARGUMENT, "unknown tuning knob");
}


}  // extern "C"

// The knob value of `choices` that gives the shortest run, each run timed
// reps times after one untimed run; choices the kernels cannot take
// (DTSGB_ERR_UNSUPPORTED) are skipped.  Leaves the knob at the best value.
template <typename F>
static int tune_knob(dtsgb_batch_t b, int knob, std::initializer_list<long long> choices,
                     int reps, F run) {
  float best = 3.4e38f;
  long long best_v = -1;
  for (long long v : choices) {
    int st = dtsgb_batch_set_tuning(b, knob, v);
    if (st) return st;
    float ms = 0.f;
    st = time_runs(b, reps, run, &ms);
    if (st == DTSGB_ERR_UNSUPPORTED) continue;  // e.g. a halo too large for this shape
    if (st) return st;
    if (ms < best) {
      best = ms;
      best_v = v;
    }
  }
  if (best_v < 0) return fail(DTSGB_ERR_UNSUPPORTED, "no tuning choice runs");
  return dtsgb_batch_set_tuning(b, knob, best_v);
}

extern "C" {

DTSGB_API int dtsgb_batch_autotune(dtsgb_batch_t b, const dtsgb_filter_params* f,
                                   const dtsgb_optimize_params* p, float overwrite,
                                   const dtsgb_hfbs_params* hp, int reps) {
  if (!b) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null handle");
  if ((f == nullptr) != (p == nullptr))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "filter and optimize params go together");
  if (reps < 1) reps = 3;
  // every timed solve does all of its work (no guide state kept across runs)
  const bool reuse = b->reuse;
  b->reuse = false;
  int st = DTSGB_OK;
  if (f) {
    auto dts = [&]() { return dtsgb_batch_solve_dts(b, f, p, overwrite); };
    st = tune_knob(b, DTSGB_TUNE_DTS_TILE, {(long long)kIterTW, (long long)kIterSmallTW}, reps,
                   dts);
    if (!st) st = tune_knob(b, DTSGB_TUNE_BOUNDS_SEGMENT, {8, 4, 16}, reps, dts);
  }
  if (hp && !st) {
    auto hfbs = [&]() { return dtsgb_batch_solve_hfbs(b, hp); };
    float best = 3.4e38f;
    long long best_s = kHfbsTBSteps, best_g = 0;
    for (long long steps : {(long long)kHfbsTBSteps, 1LL}) {
      if ((st = dtsgb_batch_set_tuning(b, DTSGB_TUNE_HFBS_SOLVE_STEPS, steps))) break;
      for (long long g : {0LL, 1000000LL, 2000000LL, 4000000LL, 8000000LL}) {
        if ((st = dtsgb_batch_set_tuning(b, DTSGB_TUNE_HFBS_GROUP_VOXELS, g))) break;
        float ms = 0.f;
        if ((st = time_runs(b, reps, hfbs, &ms))) break;
        if (ms < best) {
          best = ms;
          best_s = steps;
          best_g = g;
        }
      }
      if (st) break;
    }
    if (!st) st = dtsgb_batch_set_tuning(b, DTSGB_TUNE_HFBS_SOLVE_STEPS, best_s);
    if (!st) st = dtsgb_batch_set_tuning(b, DTSGB_TUNE_HFBS_GROUP_VOXELS, best_g);
  }
  b->reuse = reuse;
  if (st) return st;
  // leave the results of one solve with the chosen setting
  if (f && (st = dtsgb_batch_solve_dts(b, f, p, overwrite))) return st;
  if (hp && (st = dtsgb_batch_solve_hfbs(b, hp))) return st;
  return DTSGB_OK;
}

}  // extern "C"

namespace {

// FNV-1a over bytes: the autotune cache key.
struct Fnv {
  unsigned long long h = 1469598103934665603ull;
  template <typename T>
  void add(const T& v) {
    const unsigned char* q = reinterpret_cast<const unsigned char*>(&v);
    for (size_t i = 0; i < sizeof(T); ++i) h = (h ^ q[i]) * 1099511628211ull;
  }
};

const int kCachedKnobs[4] = {DTSGB_TUNE_DTS_TILE, DTSGB_TUNE_BOUNDS_SEGMENT,
                             DTSGB_TUNE_HFBS_SOLVE_STEPS, DTSGB_TUNE_HFBS_GROUP_VOXELS};

}  // namespace

extern "C" {

DTSGB_API int dtsgb_batch_autotune_cached(dtsgb_batch_t b, const dtsgb_filter_params* f,
                                          const dtsgb_optimize_params* p, float overwrite,
                                          const dtsgb_hfbs_params* hp, int reps,
                                          const char* cache_path, int* from_cache) {
  if (!b || !cache_path) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if ((f == nullptr) != (p == nullptr))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "filter and optimize params go together");
  int dev = 0;
  DTSGB_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop{};
  DTSGB_CUDA(cudaGetDeviceProperties(&prop, dev));
  // key: the device, the batch's shapes and storage, and the parameters
  Fnv k;
  for (const char* c = prop.name; *c; ++c) k.add(*c);
  k.add(prop.multiProcessorCount);
  k.add(b->n);
  k.add(b->flags);
  for (const Inst& I : b->inst) {
    k.add(I.w);
    k.add(I.h);
  }
  k.add(f != nullptr);
  if (f) {
    k.add(*f);
    k.add(*p);
    k.add(overwrite);
  }
  k.add(hp != nullptr);
  if (hp) k.add(*hp);
  char key[32];
  std::snprintf(key, sizeof key, "%016llx", k.h);
  if (from_cache) *from_cache = 0;
  {
    std::ifstream in(cache_path);
    std::string line;
    while (in && std::getline(in, line)) {
      std::istringstream ls(line);
      std::string lk;
      long long v[4];
      if (!(ls >> lk >> v[0] >> v[1] >> v[2] >> v[3]) || lk != key) continue;
      int st = DTSGB_OK;
      for (int i = 0; i < 4 && !st; ++i) st = dtsgb_batch_set_tuning(b, kCachedKnobs[i], v[i]);
      if (st) break;  // a stale line: tune again
      if (f && (st = dtsgb_batch_solve_dts(b, f, p, overwrite))) return st;
      if (hp && (st = dtsgb_batch_solve_hfbs(b, hp))) return st;
      if (from_cache) *from_cache = 1;
      return DTSGB_OK;
    }
  }
  int st = dtsgb_batch_autotune(b, f, p, overwrite, hp, reps);
  if (st) return st;
  std::ofstream out(cache_path, std::ios::app);
  if (out) {
    out << key;
    for (int kn : kCachedKnobs) {
      long long v = 0;
      dtsgb_batch_get_tuning(b, kn, &v);
      out << ' ' << v;
    }
    out << ' ' << prop.name << '\n';
  }
  return DTSGB_OK;  // a cache that cannot be written only costs the next caller a tuning
}

static int batch_download(dtsgb_batch_t b, int which, float* const* dst,
                          cudaMemcpyKind kind, bool sync_host = true) {
  if (!b || !dst) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  const float* src = nullptr;
  if (which == 0) {
    if (b->dts_res < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "no DTS solve yet");
    src = b->v[b->dts_res];
  } else if (which == 1) {
    if (!b->hfbs_done) return fail(DTSGB_ERR_INVALID_ARGUMENT, "no HFBS solve yet");
    src = b->hout;
  } else {
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "which must be 0 (DTS) or 1 (HFBS)");
  }
  for (int i = 0; i < b->n; ++i)
    if (!dst[i]) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null output pointer");
  if (kind == cudaMemcpyDeviceToDevice)
    return user_plane_copy(b, dst, const_cast<float*>(src), false, 0);
  for (int i = 0; i < b->n; ++i) {
    const Inst& I = b->inst[i];
    const size_t wb = (size_t)I.w * 4;
    DTSGB_CUDA(cudaMemcpy2DAsync(dst[i], wb, src + I.off, (size_t)I.pitch * 4, wb, I.h,
                                 kind, b->stream));
  }
  if (kind == cudaMemcpyDeviceToHost && sync_host)
    DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  return DTSGB_OK;
}

DTSGB_API int dtsgb_batch_download(dtsgb_batch_t b, int which, float* const* dst) {
  return batch_download(b, which, dst, cudaMemcpyDeviceToHost);
}

DTSGB_API int dtsgb_batch_download_device(dtsgb_batch_t b, int which,
                                          float* const* dst) {
  return batch_download(b, which, dst, cudaMemcpyDeviceToDevice);
}

DTSGB_API int dtsgb_batch_debug_plane(dtsgb_batch_t b, int i, int which, void* dst,
                                      long long dst_bytes) {
  if (!b || !dst) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  if (i < 0 || i >= b->n) return fail(DTSGB_ERR_INVALID_ARGUMENT, "instance index");
  if (which == DTSGB_BATCH_PLANE_BOUNDS) {
    if (b->dts_res < 0) return fail(DTSGB_ERR_INVALID_ARGUMENT, "no DTS solve yet");
    const Inst& I = b->inst[i];
    const size_t wb = (size_t)I.w * 4;
    if (dst_bytes < (long long)wb * I.h)
      return fail(DTSGB_ERR_INVALID_ARGUMENT, "dst_bytes smaller than W*H*4");
    DTSGB_CUDA(cudaMemcpy2DAsync(dst, wb, b->bounds + I.off, (size_t)I.pitch * 4, wb, I.h,
                                 cudaMemcpyDeviceToHost, b->stream));
  } else if (which >= DTSGB_BATCH_PLANE_COUNT && which <= DTSGB_BATCH_PLANE_B) {
    if (!b->hfbs_done || (int)b->hinst.size() != b->n)
      return fail(DTSGB_ERR_INVALID_ARGUMENT, "no HFBS solve yet");
    const HInst& H = b->hinst[i];
    const long long n = (long long)H.gx * H.gy * H.gl;
    if (dst_bytes < n * 4)
      return fail(DTSGB_ERR_INVALID_ARGUMENT, "dst_bytes smaller than gx*gy*gl*4");
    const int g = which == DTSGB_BATCH_PLANE_COUNT ? HG_COUNT
                  : which == DTSGB_BATCH_PLANE_CSUM ? HG_CSUM : HG_B;
    // rows of px voxels on the device, of gx in dst
    DTSGB_CUDA(cudaMemcpy2DAsync(dst, (size_t)H.gx * 4, b->hg[g] + H.grid_off,
                                 (size_t)H.px * 4, (size_t)H.gx * 4, (size_t)H.gy * H.gl,
                                 cudaMemcpyDeviceToHost, b->stream));
  } else {
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "which must be a DTSGB_BATCH_PLANE_* value");
  }
  DTSGB_CUDA(cudaStreamSynchronize(b->stream));
  return DTSGB_OK;
}


// ---------------------------------------------------------------------------
// Overlapped host-to-host solves: chunks of the instances, each a batch on
// its own stream; every chunk's upload, solves and downloads are enqueued
// without waiting, so copies of one chunk overlap the solves of another.
// ---------------------------------------------------------------------------
struct dtsgb_pipeline_s {
  std::vector<dtsgb_batch_t> chunk;
  std::vector<int> first;  // index of each chunk's first instance
  int n = 0;
};

DTSGB_API int dtsgb_pipeline_destroy(dtsgb_pipeline_t p) {
  if (!p) return DTSGB_OK;
  for (dtsgb_batch_t b : p->chunk) dtsgb_batch_destroy(b);
  delete p;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_pipeline_create(int n, const int* widths, const int* heights,
                                    unsigned flags, int n_chunks, dtsgb_pipeline_t* out) {
  if (!out || !widths || !heights || n <= 0 || n_chunks <= 0)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "bad pipeline description");
  *out = nullptr;
  long long total = 0;
  for (int i = 0; i < n; ++i) {
    if (widths[i] <= 0 || heights[i] <= 0)
      return fail(DTSGB_ERR_INVALID_DIMS, "instance dims must be positive");
    total += (long long)widths[i] * heights[i];
  }
  n_chunks = std::min(n_chunks, n);
  dtsgb_pipeline_t p = new dtsgb_pipeline_s();
  p->n = n;
  // contiguous runs of instances, cut where the running pixel count passes
  // k / n_chunks of the total
  long long acc = 0;
  int start = 0;
  for (int i = 0; i < n; ++i) {
    acc += (long long)widths[i] * heights[i];
    const int k = (int)p->first.size() + 1;  // chunk being filled, 1-based
    const bool last = i == n - 1;
    const bool cut = acc * n_chunks >= total * k && n - (i + 1) >= n_chunks - k;
    const bool must = n - (i + 1) == n_chunks - k;  // one instance per chunk left
    if (last || ((cut || must) && k < n_chunks)) {
      dtsgb_batch_t b = nullptr;
      int st = dtsgb_batch_create(i + 1 - start, widths + start, heights + start, flags, &b);
      if (st) {
        dtsgb_pipeline_destroy(p);
        return st;
      }
      p->chunk.push_back(b);
      p->first.push_back(start);
      start = i + 1;
    }
  }
  *out = p;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_pipeline_run_grad(dtsgb_pipeline_t p, int color_space,
                                      const void* const* rgba, const float* const* target,
                                      const float* const* conf,
                                      const dtsgb_filter_params* filter,
                                      const dtsgb_optimize_params* optimize,
                                      const float* const* grad_out, float* const* out_v,
                                      float* const* grad_target,
                                      float* const* grad_confidence) {
  if (!p || !rgba || !target || !filter || !optimize || !grad_out || !out_v)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  int st = DTSGB_OK;
  size_t k = 0;
  for (; k < p->chunk.size() && !st; ++k) {
    dtsgb_batch_t b = p->chunk[k];
    const int f = p->first[k];
    if (!b->grad) st = dtsgb_batch_enable_grad(b, 1, 0);
    if (!st)
      st = batch_upload(b, color_space, rgba + f, target + f, conf ? conf + f : nullptr,
                        cudaMemcpyHostToDevice, false);
    if (!st) st = dtsgb_batch_solve_dts(b, filter, optimize, -1.f);
    if (!st) st = batch_download(b, 0, out_v + f, cudaMemcpyDeviceToHost, false);
    if (!st)
      st = batch_backward(b, grad_out + f, grad_target ? grad_target + f : nullptr,
                          grad_confidence ? grad_confidence + f : nullptr,
                          cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, false);
  }
  for (size_t j = 0; j < k; ++j) {
    const cudaError_t e = cudaStreamSynchronize(p->chunk[j]->stream);
    if (e != cudaSuccess && !st) st = cuda_fail(e, "cudaStreamSynchronize");
  }
  return st;
}

DTSGB_API int dtsgb_pipeline_chunks(dtsgb_pipeline_t p) {
  return p ? (int)p->chunk.size() : 0;
}

DTSGB_API int dtsgb_pipeline_batch(dtsgb_pipeline_t p, int k, dtsgb_batch_t* out) {
  if (!p || !out || k < 0 || k >= (int)p->chunk.size())
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "no such chunk");
  *out = p->chunk[k];
  return DTSGB_OK;
}

DTSGB_API int dtsgb_pipeline_run(dtsgb_pipeline_t p, int color_space,
                                 const void* const* rgba, const float* const* target,
                                 const float* const* conf,
                                 const dtsgb_filter_params* filter,
                                 const dtsgb_optimize_params* optimize,
                                 float overwrite_target_above_conf,
                                 const dtsgb_hfbs_params* hfbs, float* const* out_dts,
                                 float* const* out_hfbs) {
  if (!p || !rgba || !target) return fail(DTSGB_ERR_INVALID_ARGUMENT, "null argument");
  const bool dts = filter && optimize;
  if ((dts && !out_dts) || (hfbs && !out_hfbs))
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "null output array");
  int st = DTSGB_OK;
  size_t k = 0;
  for (; k < p->chunk.size() && !st; ++k) {
    dtsgb_batch_t b = p->chunk[k];
    const int f = p->first[k];
    st = batch_upload(b, color_space, rgba + f, target + f, conf ? conf + f : nullptr,
                      cudaMemcpyHostToDevice, false);
    if (!st && dts)
      st = dtsgb_batch_solve_dts(b, filter, optimize, overwrite_target_above_conf);
    if (!st && hfbs) st = dtsgb_batch_solve_hfbs(b, hfbs);
    if (!st && dts) st = batch_download(b, 0, out_dts + f, cudaMemcpyDeviceToHost, false);
    if (!st && hfbs) st = batch_download(b, 1, out_hfbs + f, cudaMemcpyDeviceToHost, false);
  }
  // wait for every chunk enqueued so far, also after a failure (the host
  // buffers must not be in use when this returns)
  for (size_t j = 0; j < k; ++j) {
    const cudaError_t e = cudaStreamSynchronize(p->chunk[j]->stream);
    if (e != cudaSuccess && !st) st = cuda_fail(e, "cudaStreamSynchronize");
  }
  return st;
}

}  // extern "C"
