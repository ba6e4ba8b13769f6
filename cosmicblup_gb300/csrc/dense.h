// Shared host helpers of the dense FP64 paths: cuSOLVER / cuBLAS handles
// owned by a cbx_handle, status-checking macros and small wrappers.
#pragma once
#include <algorithm>
#include <memory>
#include <string>
#include <vector>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include "handle.h"

namespace cbx {

#define CBX_SOLVER(call)                                                          \
  do {                                                                            \
    cusolverStatus_t st_ = (call);                                                \
    if (st_ != CUSOLVER_STATUS_SUCCESS)                                           \
      throw Error(CBX_ERR_CUDA, std::string(#call) + " failed: " + std::to_string((int)st_)); \
  } while (0)
#define CBX_BLAS(call)                                                            \
  do {                                                                            \
    cublasStatus_t st_ = (call);                                                  \
    if (st_ != CUBLAS_STATUS_SUCCESS)                                             \
      throw Error(CBX_ERR_CUDA, std::string(#call) + " failed: " + std::to_string((int)st_)); \
  } while (0)

inline unsigned gridn(int64_t n, int threads, int cap) {
  int64_t g = (n + threads - 1) / threads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

// Library handles owned by a cbx_handle (created on first use).
struct Libs {
  cusolverDnHandle_t sol = nullptr;
  cublasHandle_t blas = nullptr;
  ~Libs() {
    if (sol) cusolverDnDestroy(sol);
    if (blas) cublasDestroy(blas);
  }
};
inline Libs& libs(cbx_handle* h) {
  if (!h->libs_slot) {
    auto l = std::make_shared<Libs>();
    CBX_SOLVER(cusolverDnCreate(&l->sol));
    CBX_SOLVER(cusolverDnSetStream(l->sol, h->stream));
    CBX_BLAS(cublasCreate(&l->blas));
    CBX_BLAS(cublasSetStream(l->blas, h->stream));
    h->libs_slot = l;
  }
  return *static_cast<Libs*>(h->libs_slot.get());
}

template <typename T>
inline std::vector<T> d2h(cbx_handle* h, const T* d, size_t n) {
  std::vector<T> v(n);
  CBX_CUDA(cudaMemcpyAsync(v.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
  CBX_CUDA(cudaStreamSynchronize(h->stream));
  return v;
}

// Cholesky of a column-major SPD matrix in place; returns false if not PD.
inline bool potrf(cbx_handle* h, double* A, int64_t n) {
  Libs& L = libs(h);
  int lw = 0;
  CBX_SOLVER(cusolverDnDpotrf_bufferSize(L.sol, CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n, &lw));
  DevBuf<double> work;
  work.resize(std::max(lw, 1));
  DevBuf<int> info;
  info.resize(1);
  CBX_SOLVER(cusolverDnDpotrf(L.sol, CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n, work.p, lw, info.p));
  int hi = 0;
  CBX_CUDA(cudaMemcpyAsync(&hi, info.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CBX_CUDA(cudaStreamSynchronize(h->stream));
  return hi == 0;
}
inline void potrs(cbx_handle* h, const double* Lf, int64_t n, double* B, int64_t nrhs) {
  Libs& L = libs(h);
  DevBuf<int> info;
  info.resize(1);
  CBX_SOLVER(cusolverDnDpotrs(L.sol, CUBLAS_FILL_MODE_LOWER, (int)n, (int)nrhs, Lf, (int)n, B, (int)n, info.p));
}
// Eigen-bending inverse (invert_psd_matrix) and Cholesky inverse on the device.
void invert_psd_device(cbx_handle* h, const double* M_dev, int64_t n, double ridge, double* out_dev);
bool chol_inverse_device(cbx_handle* h, double* A_dev, int64_t n);

}  // namespace cbx
