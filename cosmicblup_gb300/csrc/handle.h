// Internal handle shared by the translation units of libcbx.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "cbx_common.cuh"
#include "devbuf.h"
#include "mme.h"
#include <memory>
#include <mutex>
#include <set>
#include <tuple>


struct cbx_handle {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  // second stream of the PCG operator: the sparse part runs on it beside the
  // dense block product on `stream` (fork / join events, captured into graphs)
  cudaStream_t stream2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::string last_error;
  int64_t launches = 0;
  cbx::DevBuf<int> status;  // device-side error word(s)

  // Genomic relationship matrix kept on the device after cbx_grm_bed, and its
  // eigen-bent inverse after cbx_invert_psd.
  cbx::DevBuf<double> G;
  int64_t G_n = 0;
  cbx::DevBuf<double> Ginv;
  int64_t Ginv_n = 0;
  int64_t Ginv_gen = 0;  // counts the writes of Ginv
  // dense block of the single-step H^-1 (G_blend^-1 - A22^-1, ng x ng) left on
  // the device by cbx_ssgblup_qinv
  cbx::DevBuf<double> Hd;
  int64_t Hd_n = 0;
  int64_t Hd_gen = 0;    // counts the writes of Hd
  // Rademacher probe vectors of the trace estimator's stream (q x count,
  // column-major) for seed probe_z_seed and order probe_z_q: deterministic, so
  // each 16-probe batch is drawn on the host once and later MMEs of the handle
  // copy it on the device
  cbx::DevBuf<double> probe_z;
  std::vector<char> probe_z_have;
  int probe_z_seed = -1;
  int64_t probe_z_q = -1;
  // mixed-model equations and REML state
  std::unique_ptr<cbx::Mme> mme;
  // cbx_mme_keep_warm: an MME rebuilt with the same shape starts its solves from
  // the previous MME's last data and probe solutions (a REML run whose records
  // are uploaded again at every iteration)
  bool keep_warm = false;
  // library handles (cuSOLVER / cuBLAS) and dense exact AI state, owned here
  std::shared_ptr<void> libs_slot;
  std::shared_ptr<void> dense_slot;
  // scratch of the device W'W assembly (wtw.cu), kept between MMEs
  std::shared_ptr<void> wtw_slot;
  // genotypes kept on the device by cbx_geno_attach (matrix-free Z / Z^T products)
  std::shared_ptr<void> geno_slot;
  // device address of the static scratch array of cbx_dense_apply_noalloc,
  // resolved by this handle's first call (with the handle's device current)
  void* noalloc_scratch = nullptr;

  // optional per-launch timing of the dense block product (bench roofline):
  // bucket 0 = FP32 launches, bucket 1 = FP64 launches
  bool prof_on = false;
  struct ProfRec {
    cudaEvent_t a, b;
    int bucket;
    double bytes;
  };
  std::vector<ProfRec> prof;
  cudaEvent_t timer_a = nullptr, timer_b = nullptr;

  // optional launch trace (diagnostics): an event after every launch, so the
  // time between consecutive events is charged to the later launch (its own
  // run time plus any idle gap before it, host syncs included)
  bool trace_on = false;
  std::vector<std::pair<const char*, cudaEvent_t>> trace;
  std::vector<cudaEvent_t> trace_pool;
  cudaEvent_t trace_start = nullptr;

  // count a kernel launch and check the launch error
  void launched(const char* what) {
    ++launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
      throw cbx::Error(CBX_ERR_CUDA, std::string("launch ") + what + ": " + cudaGetErrorString(e));
    if (trace_on) trace_mark(what);
  }
  void trace_mark(const char* what) {
    cudaEvent_t ev;
    if (trace_pool.empty()) {
      if (cudaEventCreate(&ev) != cudaSuccess) return;
    } else {
      ev = trace_pool.back();
      trace_pool.pop_back();
    }
    cudaEventRecord(ev, stream);
    trace.emplace_back(what, ev);
  }
  // read the device status word, reset it, and throw on a device-side failure
  void check_status(const char* what);
};

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per (kernel, device,
// size): later calls make no API call, so launch sequences that may be
// captured into a CUDA graph contain only stream work.
inline void ensure_smem(const void* fn, int bytes, int device) {
  static std::mutex mu;
  static std::set<std::tuple<const void*, int, int>> done;
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_tuple(fn, device, bytes);
  if (done.count(key)) return;
  CBX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done.insert(key);
}

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
