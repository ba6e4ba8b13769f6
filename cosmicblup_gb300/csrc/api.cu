// Handle lifetime and bookkeeping entry points of the C ABI.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include "handle.h"
#include "tune.h"
#include <nvtx3/nvToolsExt.h>

void cbx_handle::check_status(const char* what) {
  int st = 0;
  CBX_CUDA(cudaMemcpyAsync(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  CBX_CUDA(cudaStreamSynchronize(stream));
  if (st != cbx::DEV_OK) {
    CBX_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), stream));
    CBX_CUDA(cudaStreamSynchronize(stream));
    if (st == cbx::DEV_TIMEOUT)
      throw cbx::Error(CBX_ERR_TIMEOUT, std::string(what) + ": device-side wait timed out");
    if (st == cbx::DEV_BREAKDOWN)
      throw cbx::Error(CBX_ERR_BREAKDOWN, std::string(what) + ": breakdown");
    if (st == cbx::DEV_NONFINITE)
      throw cbx::Error(CBX_ERR_NONFINITE, std::string(what) + ": non-finite values");
    throw cbx::Error(CBX_ERR_CUDA, std::string(what) + ": device status " + std::to_string(st));
  }
}

extern "C" {

int cbx_version(void) { return 100; }  // 0.1.0

int cbx_create(int device, cbx_handle** out) {
  if (!out) return CBX_ERR_ARG;
  *out = nullptr;
  auto* h = new cbx_handle();
  int rc = cbx_guard(h, [&] {
    int ndev = 0;
    CBX_CUDA(cudaGetDeviceCount(&ndev));
    CBX_REQUIRE(device >= 0 && device < ndev, CBX_ERR_ARG, "device index out of range");
    cudaDeviceProp prop{};
    CBX_CUDA(cudaGetDeviceProperties(&prop, device));
    CBX_REQUIRE(prop.major == 10 && prop.minor == 3, CBX_ERR_CUDA,
                "libcbx is built for sm_103a (GB300); found sm_" + std::to_string(prop.major) +
                    std::to_string(prop.minor));
    CBX_CUDA(cudaSetDevice(device));
    h->device = device;
    h->num_sms = prop.multiProcessorCount;
    CBX_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CBX_CUDA(cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking));
    CBX_CUDA(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    CBX_CUDA(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
    h->status.resize(4);
    h->status.zero(h->stream);
    CBX_CUDA(cudaStreamSynchronize(h->stream));
  });
  if (rc != CBX_OK) {
    // keep the handle so the caller can read cbx_last_error, then destroy it
    *out = h;
    return rc;
  }
  *out = h;
  return CBX_OK;
}

int cbx_destroy(cbx_handle* h) {
  if (!h) return CBX_ERR_ARG;
  if (h->stream) {
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
  }
  {
    cbx_handle* tmp = h;
    tmp->G.release();
    tmp->Ginv.release();
    tmp->mme.reset();
    tmp->dense_slot.reset();
    tmp->wtw_slot.reset();
    tmp->libs_slot.reset();
    tmp->status.release();
    for (auto& r : tmp->prof) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto& t : tmp->trace) cudaEventDestroy(t.second);
    for (auto& e : tmp->trace_pool) cudaEventDestroy(e);
    if (tmp->trace_start) cudaEventDestroy(tmp->trace_start);
    if (tmp->timer_a) cudaEventDestroy(tmp->timer_a);
    if (tmp->timer_b) cudaEventDestroy(tmp->timer_b);
    if (tmp->ev_fork) cudaEventDestroy(tmp->ev_fork);
    if (tmp->ev_join) cudaEventDestroy(tmp->ev_join);
    if (tmp->stream2) cudaStreamDestroy(tmp->stream2);
    if (tmp->stream) cudaStreamDestroy(tmp->stream);
  }
  delete h;
  return CBX_OK;
}

const char* cbx_last_error(const cbx_handle* h) {
  return h ? h->last_error.c_str() : "null handle";
}

int64_t cbx_launch_count(const cbx_handle* h) { return h ? h->launches : -1; }

int cbx_sync(cbx_handle* h) {
  return cbx_guard(h, [&] {
    CBX_CUDA(cudaSetDevice(h->device));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int cbx_timer_start(cbx_handle* h) {
  return cbx_guard(h, [&] {
    CBX_CUDA(cudaSetDevice(h->device));
    if (!h->timer_a) CBX_CUDA(cudaEventCreate(&h->timer_a));
    if (!h->timer_b) CBX_CUDA(cudaEventCreate(&h->timer_b));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
    CBX_CUDA(cudaEventRecord(h->timer_a, h->stream));
  });
}

int cbx_timer_stop(cbx_handle* h, double* ms) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->timer_a && h->timer_b, CBX_ERR_STATE, "cbx_timer_start not called");
    CBX_CUDA(cudaSetDevice(h->device));
    CBX_CUDA(cudaEventRecord(h->timer_b, h->stream));
    CBX_CUDA(cudaEventSynchronize(h->timer_b));
    float t = 0;
    CBX_CUDA(cudaEventElapsedTime(&t, h->timer_a, h->timer_b));
    if (ms) *ms = t;
  });
}

// Named NVTX ranges on the calling thread (benchmark instrumentation): a
// profiler can keep only the kernels launched inside one (ncu --nvtx
// --nvtx-include "<name>/").  NVTX is header-only and does nothing unless a
// tool is attached.
int cbx_range_push(const char* name) {
  nvtxRangePushA(name ? name : "cbx");
  return CBX_OK;
}
int cbx_range_pop(void) {
  nvtxRangePop();
  return CBX_OK;
}

// Launch trace (diagnostics, not in the public header).  cbx_trace_enable(h, 1)
// starts a trace; cbx_trace_read writes "name<TAB>launches<TAB>ms" lines, most
// expensive first, into buf (NUL-terminated, truncated at cap) and clears it.
int cbx_trace_enable(cbx_handle* h, int32_t on) {
  return cbx_guard(h, [&] {
    CBX_CUDA(cudaSetDevice(h->device));
    for (auto& t : h->trace) h->trace_pool.push_back(t.second);
    h->trace.clear();
    h->trace_on = on != 0;
    if (h->trace_on) {
      if (!h->trace_start) CBX_CUDA(cudaEventCreate(&h->trace_start));
      CBX_CUDA(cudaEventRecord(h->trace_start, h->stream));
    }
  });
}

int cbx_trace_read(cbx_handle* h, char* buf, int64_t cap) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(buf && cap > 0, CBX_ERR_ARG, "no buffer");
    CBX_CUDA(cudaSetDevice(h->device));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
    std::map<std::string, std::pair<int64_t, double>> agg;
    cudaEvent_t prev = h->trace_start;
    for (auto& t : h->trace) {
      float ms = 0.f;
      if (prev) CBX_CUDA(cudaEventElapsedTime(&ms, prev, t.second));
      auto& a = agg[t.first];
      a.first += 1;
      a.second += ms;
      prev = t.second;
    }
    std::vector<std::pair<double, std::string>> rows;
    for (auto& kv : agg) {
      char line[256];
      snprintf(line, sizeof line, "%s\t%lld\t%.4f\n", kv.first.c_str(), (long long)kv.second.first,
               kv.second.second);
      rows.emplace_back(kv.second.second, line);
    }
    std::sort(rows.begin(), rows.end(), [](auto& a, auto& b) { return a.first > b.first; });
    std::string out;
    for (auto& r : rows) out += r.second;
    const size_t n = std::min<size_t>(out.size(), (size_t)cap - 1);
    memcpy(buf, out.data(), n);
    buf[n] = 0;
    for (auto& t : h->trace) h->trace_pool.push_back(t.second);
    h->trace.clear();
    if (h->trace_on) CBX_CUDA(cudaEventRecord(h->trace_start, h->stream));
  });
}

int cbx_tune_enable(int32_t on) {
  cbx::tune::enabled_flag().store(on ? 1 : 0);
  return CBX_OK;
}

int cbx_tune_reset(void) {
  cbx::tune::reset();
  return CBX_OK;
}

int cbx_tune_report(char* buf, int64_t cap) {
  if (!buf || cap <= 0) return CBX_ERR_ARG;
  const std::string out = cbx::tune::report();
  const size_t n = std::min<size_t>(out.size(), (size_t)cap - 1);
  memcpy(buf, out.data(), n);
  buf[n] = 0;
  return CBX_OK;
}

int cbx_host_register(void* p, int64_t bytes) {
  if (!p || bytes <= 0) return CBX_ERR_ARG;
  return cudaHostRegister(p, (size_t)bytes, cudaHostRegisterDefault) == cudaSuccess ? CBX_OK : CBX_ERR_CUDA;
}

int cbx_host_unregister(void* p) {
  if (!p) return CBX_ERR_ARG;
  return cudaHostUnregister(p) == cudaSuccess ? CBX_OK : CBX_ERR_CUDA;
}

}  // extern "C"
