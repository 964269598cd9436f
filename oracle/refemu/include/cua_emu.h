// Host-memory stand-ins for the libcua container types the reference's
// DTS / HFBS sources use (cua::CudaArray2D/3D, cua::CudaSurface2D/3D) --
// TEST INFRASTRUCTURE ONLY.  libcua (the reference's ext/cudaArray
// submodule) is not in the checkout; this restates the behaviour the
// reference's call sites rely on:
//   * copies of a container share its memory (kernels take them by value,
//     and the solvers swap buffers by assignment);
//   * arrays are pitched linear memory, rows padded to 512 bytes as
//     cudaMallocPitch pads them; get/set/ptr index it without a bounds
//     check, so a read just outside the image lands in the row padding or
//     the neighbouring row, as on the GPU.  Every allocation is zeroed and
//     sits between zeroed guard regions, so reads the reference makes
//     before or after an allocation return 0 instead of faulting;
//   * surfaces are bounds-checked: a read outside returns zero and a write
//     outside is dropped (CUDA's cudaBoundaryModeZero);
//   * `container = host_ptr` and `container.View(x, y, w, h) = host_ptr`
//     upload a dense host image, `View(...).CopyTo(host_ptr)` downloads one,
//     Fill sets every element of the width x height (x depth) extent.
#pragma once

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "refemu.h"

namespace cua {
namespace emu {

constexpr size_t kPitchAlign = 512;

template <class T>
struct Storage {
  std::vector<T> mem;
  size_t guard = 0;
  T* base() { return mem.data() + guard; }
};

template <class T>
std::shared_ptr<Storage<T>> make_storage(size_t elems, size_t guard_before, size_t guard_after) {
  auto s = std::make_shared<Storage<T>>();
  s->mem.assign(guard_before + elems + guard_after, T());
  s->guard = guard_before;
  return s;
}

// A rectangle of a 2-D container: upload from / download to a dense host
// image of w x h elements.
template <class C>
struct View2D {
  C c;
  int x0, y0, w, h;
  View2D& operator=(const typename C::Scalar* host) {
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) c.set(x0 + x, y0 + y, host[(size_t)y * w + x]);
    return *this;
  }
  void CopyTo(typename C::Scalar* host) const {
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) host[(size_t)y * w + x] = c.get(x0 + x, y0 + y);
  }
};

}  // namespace emu

template <class T>
class CudaArray2D {
 public:
  typedef T Scalar;
  CudaArray2D(size_t width, size_t height) : w_(width), h_(height) {
    pitch_ = (width * sizeof(T) + emu::kPitchAlign - 1) / emu::kPitchAlign * emu::kPitchAlign /
             sizeof(T);
    const size_t n = pitch_ * height;
    s_ = emu::make_storage<T>(n, pitch_ + 4096, n + 4096);
    base_ = s_->base();
  }
  CudaArray2D& operator=(const T* host) {
    View(0, 0, (int)w_, (int)h_) = host;
    return *this;
  }
  T get(int x, int y) const { return base_[(ptrdiff_t)y * (ptrdiff_t)pitch_ + x]; }
  void set(int x, int y, T v) const { base_[(ptrdiff_t)y * (ptrdiff_t)pitch_ + x] = v; }
  T* ptr() const { return base_; }
  T* ptr(int x, int y) const { return base_ + (ptrdiff_t)y * (ptrdiff_t)pitch_ + x; }
  size_t Pitch() const { return pitch_ * sizeof(T); }
  size_t Width() const { return w_; }
  size_t Height() const { return h_; }
  void Fill(T v) const {
    for (size_t y = 0; y < h_; ++y) std::fill(base_ + y * pitch_, base_ + y * pitch_ + w_, v);
  }
  emu::View2D<CudaArray2D> View(int x, int y, int w, int h) const {
    return emu::View2D<CudaArray2D>{*this, x, y, w, h};
  }

 private:
  size_t w_, h_, pitch_;
  std::shared_ptr<emu::Storage<T>> s_;
  T* base_;
};

template <class T>
class CudaArray3D {
 public:
  typedef T Scalar;
  CudaArray3D(size_t width, size_t height, size_t depth) : w_(width), h_(height), d_(depth) {
    pitch_ = (width * sizeof(T) + emu::kPitchAlign - 1) / emu::kPitchAlign * emu::kPitchAlign /
             sizeof(T);
    const size_t n = pitch_ * height * depth;
    s_ = emu::make_storage<T>(n, pitch_ * height + 4096, n + 4096);
    base_ = s_->base();
  }
  ptrdiff_t index(int x, int y, int z) const {
    return ((ptrdiff_t)z * (ptrdiff_t)h_ + y) * (ptrdiff_t)pitch_ + x;
  }
  T get(int x, int y, int z) const { return base_[index(x, y, z)]; }
  void set(int x, int y, int z, T v) const { base_[index(x, y, z)] = v; }
  T* ptr() const { return base_; }
  T* ptr(int x, int y, int z) const { return base_ + index(x, y, z); }
  size_t Pitch() const { return pitch_ * sizeof(T); }
  size_t Width() const { return w_; }
  size_t Height() const { return h_; }
  size_t Depth() const { return d_; }
  void Fill(T v) const {
    for (size_t z = 0; z < d_; ++z)
      for (size_t y = 0; y < h_; ++y) {
        T* row = base_ + index(0, (int)y, (int)z);
        std::fill(row, row + w_, v);
      }
  }

 private:
  size_t w_, h_, d_, pitch_;
  std::shared_ptr<emu::Storage<T>> s_;
  T* base_;
};

template <class T>
class CudaSurface2D {
 public:
  typedef T Scalar;
  CudaSurface2D(size_t width, size_t height) : w_(width), h_(height) {
    s_ = emu::make_storage<T>(width * height, 0, 0);
    base_ = s_->base();
  }
  CudaSurface2D& operator=(const T* host) {
    View(0, 0, (int)w_, (int)h_) = host;
    return *this;
  }
  bool inside(int x, int y) const {
    return x >= 0 && y >= 0 && (size_t)x < w_ && (size_t)y < h_;
  }
  T get(int x, int y) const { return inside(x, y) ? base_[(size_t)y * w_ + x] : T(); }
  void set(int x, int y, T v) const {
    if (inside(x, y)) base_[(size_t)y * w_ + x] = v;
  }
  size_t Width() const { return w_; }
  size_t Height() const { return h_; }
  void Fill(T v) const { std::fill(base_, base_ + w_ * h_, v); }
  emu::View2D<CudaSurface2D> View(int x, int y, int w, int h) const {
    return emu::View2D<CudaSurface2D>{*this, x, y, w, h};
  }

 private:
  size_t w_, h_;
  std::shared_ptr<emu::Storage<T>> s_;
  T* base_;
};

template <class T>
class CudaSurface3D {
 public:
  typedef T Scalar;
  CudaSurface3D(size_t width, size_t height, size_t depth) : w_(width), h_(height), d_(depth) {
    s_ = emu::make_storage<T>(width * height * depth, 0, 0);
    base_ = s_->base();
  }
  bool inside(int x, int y, int z) const {
    return x >= 0 && y >= 0 && z >= 0 && (size_t)x < w_ && (size_t)y < h_ && (size_t)z < d_;
  }
  size_t index(int x, int y, int z) const { return ((size_t)z * h_ + y) * w_ + x; }
  T get(int x, int y, int z) const { return inside(x, y, z) ? base_[index(x, y, z)] : T(); }
  void set(int x, int y, int z, T v) const {
    if (inside(x, y, z)) base_[index(x, y, z)] = v;
  }
  size_t Width() const { return w_; }
  size_t Height() const { return h_; }
  size_t Depth() const { return d_; }
  void Fill(T v) const { std::fill(base_, base_ + w_ * h_ * d_, v); }

 private:
  size_t w_, h_, d_;
  std::shared_ptr<emu::Storage<T>> s_;
  T* base_;
};

}  // namespace cua
