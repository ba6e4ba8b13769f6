// Autotuner of launch shapes (tile heights, piece widths, chunk sizes).
//
// A kernel family offers a few candidate launch shapes that compute bit-identical
// results: they change how work is spread over warps and CTAs, never the order in
// which any single output is accumulated.  The first call of a (family, device,
// size class, width) key outside stream capture runs every candidate twice on the
// live operands, times the second run with CUDA events on the handle's stream and
// keeps the fastest; a candidate replaces the default only when it is at least 1.5 %
// faster, so timing noise does not move a key off its default for nothing.  Later calls (and
// calls during graph capture, which cannot time) use the stored choice, or the
// default when none is stored yet.  The environment variable CBX_TUNE=0 (or
// cbx_tune_enable(0)) pins every family to its default.  Because all candidates give
// the same bits, tuning never changes a result.
#pragma once
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>
#include "handle.h"

namespace cbx {
namespace tune {

enum Family : int { FF = 0, GEMV = 1, GENO_ZT = 2, GENO_Z = 3 };

inline const char* family_name(int f) {
  switch (f) {
    case FF: return "k_dense_ff";
    case GEMV: return "k_gemv";
    case GENO_ZT: return "k_geno_zt";
    case GENO_Z: return "k_geno_z";
    default: return "?";
  }
}

// Half-octave size class of a dimension.
inline int size_class(int64_t x) { return x > 0 ? (int)std::floor(2.0 * std::log2((double)x)) : 0; }

struct Decision {
  int choice = 0;
  std::vector<float> ms;  // measured time per candidate
};

using Key = std::tuple<int, int, int, int, int>;  // family, device, class a, class b, width

inline std::mutex& mu() {
  static std::mutex m;
  return m;
}
inline std::map<Key, Decision>& table() {
  static std::map<Key, Decision> t;
  return t;
}

// On unless the environment sets CBX_TUNE=0; cbx_tune_enable switches it at run time.
inline std::atomic<int>& enabled_flag() {
  static std::atomic<int> v{[] {
    const char* e = std::getenv("CBX_TUNE");
    return (e && e[0] == '0') ? 0 : 1;
  }()};
  return v;
}
inline bool enabled() { return enabled_flag().load() == 1; }

// Candidate index for the key; run(c) launches candidate c on the handle's stream.
// may_time = false only looks the key up (a call whose operands cannot tell the
// candidates apart).
template <typename F>
int choose(cbx_handle* h, int family, int class_a, int class_b, int width, int ncand, F&& run,
           bool may_time = true) {
  if (!enabled() || ncand <= 1) return 0;
  const Key key{family, h->device, class_a, class_b, width};
  {
    std::lock_guard<std::mutex> lk(mu());
    auto it = table().find(key);
    if (it != table().end()) return it->second.choice;
  }
  if (!may_time) return 0;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return 0;
  Decision d;
  d.ms.assign(ncand, 0.f);
  cudaEvent_t a = nullptr, b = nullptr;
  CBX_CUDA(cudaEventCreate(&a));
  CBX_CUDA(cudaEventCreate(&b));
  try {
    for (int c = 0; c < ncand; ++c) {
      run(c);
      CBX_CUDA(cudaEventRecord(a, h->stream));
      run(c);
      CBX_CUDA(cudaEventRecord(b, h->stream));
      CBX_CUDA(cudaEventSynchronize(b));
      CBX_CUDA(cudaEventElapsedTime(&d.ms[c], a, b));
    }
  } catch (...) {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  int best = 0;
  for (int c = 1; c < ncand; ++c)
    if (d.ms[c] < d.ms[best]) best = c;
  d.choice = (best != 0 && d.ms[best] <= 0.985f * d.ms[0]) ? best : 0;
  std::lock_guard<std::mutex> lk(mu());
  auto ins = table().emplace(key, d);
  return ins.first->second.choice;
}

// One line per decision: family, device, size classes, width, choice, times.
inline std::string report() {
  std::lock_guard<std::mutex> lk(mu());
  std::string s;
  for (const auto& [k, d] : table()) {
    s += std::string(family_name(std::get<0>(k))) + " dev " + std::to_string(std::get<1>(k)) + " class " +
         std::to_string(std::get<2>(k)) + "/" + std::to_string(std::get<3>(k)) + " width " +
         std::to_string(std::get<4>(k)) + " choice " + std::to_string(d.choice) + " ms";
    for (float t : d.ms) s += " " + std::to_string(t);
    s += "\n";
  }
  return s;
}

inline void reset() {
  std::lock_guard<std::mutex> lk(mu());
  table().clear();
}

}  // namespace tune
}  // namespace cbx
