// CPU execution of CUDA C++ kernels, for compiling the reference's own DTS /
// HFBS sources with g++ -- TEST INFRASTRUCTURE ONLY (it produces golden
// vectors; no product code includes it).
//
// What it provides, in place of the CUDA toolkit's headers:
//   * the execution-space keywords (__global__, __device__, __host__,
//     __forceinline__) as plain C++, __shared__ as `static` (blocks run one
//     after another, so a function-local static is the block's shared memory);
//   * the builtin variables threadIdx / blockIdx / blockDim / gridDim as
//     globals that the launcher sets before it runs each thread;
//   * refemu::launch: a kernel launch as a loop over blocks and threads
//     (x fastest), and refemu::launch_coop for kernels that call
//     __syncthreads(): each thread of a block is a ucontext fiber and a
//     barrier switches to the next fiber until all have reached it;
//   * the vector types, atomicAdd (sequential: one thread at a time), the
//     mixed-type min/max overloads of CUDA's math headers (the wider type
//     wins), and the error-query calls (nothing fails on the host).
// Floating-point arithmetic is the host's: g++ contracts a*b+c to fma like
// nvcc does (-ffp-contract=fast), sqrt is correctly rounded as on the GPU,
// and expf is glibc's (within an ulp of CUDA's).
#pragma once

#include <math.h>
#include <ucontext.h>

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static

struct uint3 {
  unsigned int x, y, z;
};

struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};

struct uchar4 {
  unsigned char x, y, z, w;
};

inline uchar4 make_uchar4(unsigned char x, unsigned char y, unsigned char z, unsigned char w) {
  uchar4 v;
  v.x = x;
  v.y = y;
  v.z = z;
  v.w = w;
  return v;
}

inline uint3 threadIdx;
inline uint3 blockIdx;
inline dim3 blockDim;
inline dim3 gridDim;

enum cudaError_t { cudaSuccess = 0 };
typedef cudaError_t cudaError;
inline const char* cudaGetErrorString(cudaError_t) { return "no error"; }
inline cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }

template <class T, class U>
inline T atomicAdd(T* address, U value) {
  const T old = *address;
  *address = old + value;
  return old;
}

// CUDA's math headers overload min/max for every pair of int, float and
// double; the result has the wider operand type.
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, float b) { return fminf(a, b); }
inline double max(double a, double b) { return fmax(a, b); }
inline double min(double a, double b) { return fmin(a, b); }
inline double max(double a, float b) { return fmax(a, (double)b); }
inline double max(float a, double b) { return fmax((double)a, b); }
inline double min(double a, float b) { return fmin(a, (double)b); }
inline double min(float a, double b) { return fmin((double)a, b); }
inline float max(int a, float b) { return fmaxf((float)a, b); }
inline float max(float a, int b) { return fmaxf(a, (float)b); }

namespace refemu {

// ---- plain launches: one thread after another ----------------------------
template <class Body>
void launch(dim3 grid, dim3 block, Body&& body) {
  gridDim = grid;
  blockDim = block;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = uint3{bx, by, bz};
        for (unsigned tz = 0; tz < block.z; ++tz)
          for (unsigned ty = 0; ty < block.y; ++ty)
            for (unsigned tx = 0; tx < block.x; ++tx) {
              threadIdx = uint3{tx, ty, tz};
              body();
            }
      }
}

// ---- cooperative launches: threads of a block as fibers -------------------
struct Fiber {
  ucontext_t ctx;
  std::vector<char> stack;
  uint3 tid;
  bool done;
};

struct CoopState {
  ucontext_t scheduler;
  Fiber* current = nullptr;
  void (*entry)(void*) = nullptr;
  void* arg = nullptr;
  bool active = false;
};
inline CoopState coop;

inline void fiber_main() {
  coop.entry(coop.arg);
  coop.current->done = true;  // uc_link returns to the scheduler
}

template <class Body>
void launch_coop(dim3 grid, dim3 block, Body&& body) {
  constexpr size_t kStack = 256 * 1024;
  const size_t n = (size_t)block.x * block.y * block.z;
  std::vector<Fiber> fibers(n);
  for (auto& f : fibers) f.stack.resize(kStack);
  coop.entry = [](void* p) { (*static_cast<Body*>(p))(); };
  coop.arg = &body;
  coop.active = true;
  gridDim = grid;
  blockDim = block;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = uint3{bx, by, bz};
        size_t k = 0;
        for (unsigned tz = 0; tz < block.z; ++tz)
          for (unsigned ty = 0; ty < block.y; ++ty)
            for (unsigned tx = 0; tx < block.x; ++tx, ++k) {
              Fiber& f = fibers[k];
              f.tid = uint3{tx, ty, tz};
              f.done = false;
              getcontext(&f.ctx);
              f.ctx.uc_stack.ss_sp = f.stack.data();
              f.ctx.uc_stack.ss_size = f.stack.size();
              f.ctx.uc_link = &coop.scheduler;
              makecontext(&f.ctx, fiber_main, 0);
            }
        // Run every unfinished thread up to its next barrier (or its end),
        // until all have finished.
        for (bool any = true; any;) {
          any = false;
          for (auto& f : fibers) {
            if (f.done) continue;
            threadIdx = f.tid;
            coop.current = &f;
            swapcontext(&coop.scheduler, &f.ctx);
            any = any || !f.done;
          }
        }
      }
  coop.active = false;
}

inline unsigned linear_tid() {
  return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
}

}  // namespace refemu

inline void __syncthreads() {
  if (!refemu::coop.active) {
    std::fprintf(stderr, "refemu: __syncthreads() outside a cooperative launch\n");
    std::abort();
  }
  swapcontext(&refemu::coop.current->ctx, &refemu::coop.scheduler);
}
