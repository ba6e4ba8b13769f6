// Internal handle shared by the translation units of libcbx.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
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

struct cbx_handle {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int64_t launches = 0;
  cbx::DevBuf<int> status;  // device-side error word(s)

  // Genomic relationship matrix kept on the device after cbx_grm_bed.
  cbx::DevBuf<double> G;
  int64_t G_n = 0;

  // count a kernel launch and check the launch error
  void launched(const char* what) {
    ++launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
      throw cbx::Error(CBX_ERR_CUDA, std::string("launch ") + what + ": " + cudaGetErrorString(e));
  }
  // read the device status word, reset it, and throw on a device-side failure
  void check_status(const char* what);
};

// Run fn, translating exceptions to status codes stored in h->last_error.
template <typename F>
int cbx_guard(cbx_handle* h, F&& fn) {
  if (!h) return CBX_ERR_ARG;
  try {
    fn();
    h->last_error.clear();
    return CBX_OK;
  } catch (const cbx::Error& e) {
    h->last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    h->last_error = e.what();
    return CBX_ERR_ARG;
  }
}
