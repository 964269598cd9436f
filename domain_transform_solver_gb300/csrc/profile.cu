// Per-kernel launch timing with CUDA events recorded on the launching
// stream.  Disabled by default; enabled by dtsgb_profile_enable().  Events
// are pooled and reused across resets.
#include <mutex>
#include <vector>

#include "../../include/dtsgb.h"
#include "dtsgb_internal.cuh"

namespace dtsgb {
namespace {

struct Rec {
  int id;
  cudaEvent_t a, b;
};

struct Profiler {
  std::mutex mu;
  bool enabled = false;
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  std::vector<int> open;  // index into recs of the open record per kernel id
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

void prof_begin(cudaStream_t s, int id) {
  Profiler& p = prof();
  if (!p.enabled) return;
  std::lock_guard<std::mutex> g(p.mu);
  Rec r{id, p.get(), p.get()};
  if (!r.a || !r.b) return;
  cudaEventRecord(r.a, s);
  p.recs.push_back(r);
  p.open[id] = (int)p.recs.size() - 1;
}

void prof_end(cudaStream_t s, int id) {
  Profiler& p = prof();
  if (!p.enabled) return;
  std::lock_guard<std::mutex> g(p.mu);
  const int k = p.open[id];
  if (k < 0) return;
  cudaEventRecord(p.recs[k].b, s);
  p.open[id] = -1;
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
  for (Rec& r : p.recs) {
    cudaEventSynchronize(r.b);
    p.pool.push_back(r.a);
    p.pool.push_back(r.b);
  }
  p.recs.clear();
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
    DTSGB_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    ++n;
    t += ms;
  }
  *launches = n;
  *total_ms = t;
  return DTSGB_OK;
}

}  // extern "C"
