// Per-kernel launch timing with CUDA events recorded on the launching
// stream.  Disabled by default; enabled by dtsgb_profile_enable().  Events
// are pooled and reused across resets.
#include <mutex>
#include <vector>

#include "../../include/dtsgb.h"
#include "dtsgb_internal.cuh"

namespace dtsgb {
namespace {

// A record captured into a CUDA graph holds events that the graph's event
// nodes record on every replay (the read returns the latest replay); those
// events belong to the graph from then on and are never recycled.
struct Rec {
  int id;
  cudaEvent_t a, b;
  bool captured;
  const void* tag;  // owner of the graph a captured record belongs to
};

struct Profiler {
  std::mutex mu;
  bool enabled = false;
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  std::vector<int> open;  // index into recs of the open record per kernel id
  const void* capture_tag = nullptr;
  Profiler() : open(DTSGB_K_COUNT, -1) {}

  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
  }
};

Profiler& prof() {
  static Profiler p;
  return p;
}

}  // namespace

bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return false;
  return st == cudaStreamCaptureStatusActive;
}

void record(cudaEvent_t e, cudaStream_t s, bool cap) {
  if (cap)
    cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
  else
    cudaEventRecord(e, s);
}

void prof_begin(cudaStream_t s, int id) {
  Profiler& p = prof();
  if (!p.enabled) return;
  std::lock_guard<std::mutex> g(p.mu);
  const bool cap = capturing(s);
  Rec r{id, nullptr, nullptr, cap, cap ? p.capture_tag : nullptr};
  if (cap) {
    if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess)
      return;
  } else {
    r.a = p.get();
    r.b = p.get();
  }
  if (!r.a || !r.b) return;
  record(r.a, s, cap);
  p.recs.push_back(r);
  p.open[id] = (int)p.recs.size() - 1;
}

void prof_end(cudaStream_t s, int id) {
  Profiler& p = prof();
  if (!p.enabled) return;
  std::lock_guard<std::mutex> g(p.mu);
  const int k = p.open[id];
  if (k < 0) return;
  record(p.recs[k].b, s, p.recs[k].captured);
  p.open[id] = -1;
}

bool prof_enabled() { return prof().enabled; }

void prof_set_capture_tag(const void* tag) {
  Profiler& p = prof();
  std::lock_guard<std::mutex> g(p.mu);
  p.capture_tag = tag;
}

// Forget the records captured into the graphs of `tag` (call after the graph
// executable is destroyed).
void prof_drop_captured(const void* tag) {
  Profiler& p = prof();
  std::lock_guard<std::mutex> g(p.mu);
  std::vector<Rec> keep;
  for (Rec& r : p.recs) {
    if (r.captured && r.tag == tag) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
      continue;
    }
    keep.push_back(r);
  }
  p.recs.swap(keep);
  for (int& o : p.open) o = -1;
}

}  // namespace dtsgb

using namespace dtsgb;

extern "C" {

DTSGB_API int dtsgb_profile_enable(int enable) {
  prof().enabled = enable != 0;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_profile_reset(void) {
  Profiler& p = prof();
  std::lock_guard<std::mutex> g(p.mu);
  std::vector<Rec> keep;
  for (Rec& r : p.recs) {
    if (r.captured) {
      keep.push_back(r);  // still referenced by a graph
      continue;
    }
    cudaEventSynchronize(r.b);
    p.pool.push_back(r.a);
    p.pool.push_back(r.b);
  }
  p.recs.swap(keep);
  for (int& o : p.open) o = -1;
  return DTSGB_OK;
}

DTSGB_API int dtsgb_profile_read(int id, int* launches, double* total_ms) {
  if (id < 0 || id >= DTSGB_K_COUNT || !launches || !total_ms)
    return fail(DTSGB_ERR_INVALID_ARGUMENT, "bad profile query");
  Profiler& p = prof();
  std::lock_guard<std::mutex> g(p.mu);
  int n = 0;
  double t = 0.0;
  for (const Rec& r : p.recs) {
    if (r.id != id) continue;
    DTSGB_CUDA(cudaEventSynchronize(r.b));
    float ms = 0.f;
    // a captured record whose graph has not been replayed has no time yet
    if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) {
      (void)cudaGetLastError();
      continue;
    }
    ++n;
    t += ms;
  }
  *launches = n;
  *total_ms = t;
  return DTSGB_OK;
}

}  // extern "C"
