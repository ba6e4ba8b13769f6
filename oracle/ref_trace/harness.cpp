// C entry points around the reference's own RNG and AdaptiveTraceEstimator
// (compiled from the reference tree, src/core/rng.h and
// src/core/adaptive_trace_estimator.cpp, single-threaded: no OpenMP).
#include <cstring>
#include "adaptive_trace_estimator.h"
#include "rng.h"

extern "C" {
typedef void (*ref_op_cb)(const double* z, double* out, int dim);

void ref_rademacher(unsigned long seed, int n, double* out) {
  cosmic::RNG rng(seed);
  Eigen::VectorXd v(n);
  rng.fill_rademacher(v);
  std::memcpy(out, v.data(), sizeof(double) * static_cast<size_t>(n));
}

double ref_trace_estimate(int dim, ref_op_cb cb, int min_samples, int max_samples, double tol,
                          int seed) {
  auto op = [&](const Eigen::VectorXd& z) {
    Eigen::VectorXd out(dim);
    cb(z.data(), out.data(), dim);
    return out;
  };
  return cosmic::AdaptiveTraceEstimator::estimate(dim, op, min_samples, max_samples, tol, seed);
}
}
