// RAII device buffer shared by the translation units of libcbx.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>
#include "cbx_common.cuh"

namespace cbx {

// RAII device buffer (cudaMalloc / cudaFree, no pooling; the handle owns them).
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void resize(size_t count) {
    if (count == n && p) return;
    release();
    if (count) CBX_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void zero(cudaStream_t s) {
    if (n) CBX_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
};

}  // namespace cbx
