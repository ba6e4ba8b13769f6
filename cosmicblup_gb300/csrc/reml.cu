// AI-REML for one random component on the device, and the eigen-bending inverse.
//
// Replaces (reference src/core/vce.cpp unless noted):
//  * AI_REML::solve outer loop and stop rule sum|delta| < tol (:741-837);
//  * run_ai_iteration's EM branch with Hutchinson traces (:1490-1574),
//    estimate_trace_Qinv_Cuu (:1266-1315) and AdaptiveTraceEstimator::estimate
//    (src/core/adaptive_trace_estimator.cpp:11-81, one thread: batches of 16,
//    engine std::mt19937_64(seed + samples_done), Rademacher via
//    std::uniform_int_distribution<int>(0, 1) as in src/core/rng.h:48-53);
//    the probes of consecutive batches are solved together as one multi-RHS
//    block, then consumed in the reference's order with its stopping rule;
//  * stabilize_variance (:1379-1389);
//  * run_dense_exact_step (:2949-3195) with project_spd_2x2 (:267-283);
//  * invert_psd_matrix (src/core/matrix_io.cpp:488-501).
#include <algorithm>
#include <cmath>
#include <memory>
#include <random>
#include <thread>
#include <cstdlib>
#include <vector>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include "dense.h"
#include "handle.h"
#include "pcg.h"
#include "solver.cuh"

namespace cbx {

// ---------------------------------------------------------------------------
// kernels of the dense paths (column-major matrices)
__global__ void k_add_ridge_copy(const double* __restrict__ src, int64_t n, double ridge, double* __restrict__ dst) {
  const int64_t total = n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i % n, c = i / n;
    dst[i] = src[i] + (r == c ? ridge : 0.0);
  }
}
// V[:, j] = U[:, j] / w_j
__global__ void k_scale_cols(const double* __restrict__ U, const double* __restrict__ w, int64_t n,
                             double* __restrict__ V) {
  const int64_t total = n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    V[i] = U[i] / w[i / n];
}
// C = dense(D) + lam [0 0; 0 Qd]  (dim x dim, column-major; D CSR rows = columns by symmetry)
__global__ void k_build_lhs(int64_t dim, int64_t p, const int32_t* __restrict__ Dptr, const int32_t* __restrict__ Dcol,
                            const double* __restrict__ Dval, const double* __restrict__ Qd, int64_t ld, double lam,
                            double* __restrict__ C) {
  const int64_t total = dim * dim;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i % dim, c = i / dim;
    C[i] = (r >= p && c >= p) ? lam * Qd[(r - p) * ld + (c - p)] : 0.0;
  }
}
__global__ void k_scatter_csr(int64_t dim, const int32_t* __restrict__ Dptr, const int32_t* __restrict__ Dcol,
                              const double* __restrict__ Dval, double* __restrict__ C) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x)
    for (int32_t j = Dptr[r]; j < Dptr[r + 1]; ++j) C[(int64_t)Dcol[j] * dim + r] += Dval[j];
}
// P[i, j] = (delta_ij - (W C^-1 W^T)[i, j]) / ve from the explicit C^-1 (dim x
// dim, column-major, symmetric): a gather over the two records' design rows
// (their fixed-effect entries and their animal).
__global__ void k_build_P_ci(int64_t n_rec, int64_t p, int64_t q, int64_t dim, const int32_t* __restrict__ aid,
                             const int32_t* __restrict__ xp, const int32_t* __restrict__ xc,
                             const double* __restrict__ xv, const double* __restrict__ Ci, double ve,
                             double* __restrict__ P) {
  const int64_t total = n_rec * n_rec;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % n_rec, j = idx / n_rec;
    // column (W C^-1)[i, :] restricted to record j's entries: sum_b w_jb (sum_a w_ia Ci[b, a])
    auto row_i_dot = [&](int64_t b) {
      const double* cb = Ci + b * dim;
      double t = 0.0;
      for (int32_t k = xp[i]; k < xp[i + 1]; ++k)
        if (xc[k] < p) t += xv[k] * cb[xc[k]];
      const int32_t a = aid[i];
      if (a > 0 && a <= q) t += cb[p + a - 1];
      return t;
    };
    double hsum = 0.0;
    for (int32_t k = xp[j]; k < xp[j + 1]; ++k)
      if (xc[k] < p) hsum += xv[k] * row_i_dot(xc[k]);
    const int32_t bj = aid[j];
    if (bj > 0 && bj <= q) hsum += row_i_dot(p + bj - 1);
    P[idx] = ((i == j ? 1.0 : 0.0) - hsum) / ve;
  }
}
// C = A B for n x n column-major FP64 matrices: 64 x 64 output tiles per
// block, 4 x 4 per thread, K in steps of 16 staged in shared memory; every
// output sums its K terms in index order.  FP64 multiply-add issue bounds it
// (GB300 runs FP64 at 1/64 of the FP32 rate).
__global__ void __launch_bounds__(256) k_dgemm_nn(int64_t n, const double* __restrict__ A,
                                                  const double* __restrict__ B, double* __restrict__ C) {
  __shared__ double As[16][65];
  __shared__ double Bs[16][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t row0 = (int64_t)blockIdx.x * 64, col0 = (int64_t)blockIdx.y * 64;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int64_t k0 = 0; k0 < n; k0 += 16) {
    for (int t = threadIdx.x; t < 1024; t += 256) {
      const int r = t & 63, kk = t >> 6;
      As[kk][r] = (row0 + r < n && k0 + kk < n) ? A[(k0 + kk) * n + row0 + r] : 0.0;
      const int kb = t & 15, c = t >> 4;
      Bs[kb][c] = (col0 + c < n && k0 + kb < n) ? B[(col0 + c) * n + k0 + kb] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t r = row0 + ty * 4 + i, c = col0 + tx * 4 + j;
      if (r < n && c < n) C[c * n + r] = acc[i][j];
    }
}
// y = A x for an n x n column-major FP64 matrix (one thread per row, K in order)
__global__ void k_dgemv_n(int64_t n, const double* __restrict__ A, const double* __restrict__ x,
                          double* __restrict__ y) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int64_t k = 0; k < n; ++k) t = fma(A[k * n + r], x[k], t);
    y[r] = t;
  }
}
// ZAZt[i, j] = A[aid_i - 1, aid_j - 1] (0 for records without an animal)
__global__ void k_build_zazt(int64_t n_rec, int64_t q, const int32_t* __restrict__ aid, const double* __restrict__ A,
                             double* __restrict__ Z) {
  const int64_t total = n_rec * n_rec;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % n_rec, j = idx / n_rec;
    const int32_t a = aid[i], b = aid[j];
    Z[idx] = (a > 0 && a <= q && b > 0 && b <= q) ? A[(int64_t)(b - 1) * q + (a - 1)] : 0.0;
  }
}
// fill the strict upper triangle from the lower one (column-major)
__global__ void k_symmetrize_lower(double* __restrict__ A, int64_t n) {
  const int64_t total = n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx % n, c = idx / n;
    if (r < c) A[idx] = A[r * n + c];
  }
}
// partial sums of: sum M_ij M_ji, sum M_ij P_ij, sum P_ij^2, tr M, tr P
__global__ void k_ai_traces(const double* __restrict__ M, const double* __restrict__ P, int64_t n,
                            double* __restrict__ part) {
  __shared__ double red[256];
  double s[5] = {0, 0, 0, 0, 0};
  const int64_t total = n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % n, j = idx / n;
    const double m = M[idx], pv = P[idx];
    s[0] += m * M[i * n + j];
    s[1] += m * pv;
    s[2] += pv * pv;
    if (i == j) { s[3] += m; s[4] += pv; }
  }
  for (int k = 0; k < 5; ++k) {
    const double t = sv::block_sum_cols<1>(s[k], red);
    if (threadIdx.x == 0) part[blockIdx.x * 5 + k] = t;
  }
}
__global__ void k_log_diag_sum(const double* __restrict__ L, int64_t n, double* __restrict__ part, int* bad) {
  __shared__ double red[256];
  double s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = L[i * n + i];
    if (!(d > 0) || !isfinite(d)) atomicExch(bad, 1);
    s += log(d);
  }
  const double t = sv::block_sum_cols<1>(s, red);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// sum_i log L_ii of a Cholesky factor; NaN if a pivot is not positive
static double log_diag(cbx_handle* h, const double* Lf, int64_t n) {
  const unsigned g = gridn(n, 256, 256);
  DevBuf<double> part;
  part.resize(g);
  DevBuf<int> bad;
  bad.resize(1);
  bad.zero(h->stream);
  k_log_diag_sum<<<g, 256, 0, h->stream>>>(Lf, n, part.p, bad.p);
  h->launched("k_log_diag_sum");
  auto ph = d2h(h, part.p, g);
  if (d2h(h, bad.p, 1)[0]) return std::nan("");
  double s = 0;
  for (double v : ph) s += v;
  return s;
}

static double dot_h(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

// ---------------------------------------------------------------------------
struct RemlConfigI {
  int max_iter = 20;
  double tol = 1e-4;
  int mc_samples = 100;
  int pcg_max_iter = 10000;
  double pcg_tol = 1e-10;
  int precision = 0;
  int mode = 0;  // 0 auto, 1 EM + Hutchinson, 2 dense exact
  int seed = 42;
};

struct IterInfo {
  int kind = 0;
  double var_u = 0, var_e = 0, logL = std::nan(""), trace = std::nan("");
  int probes = 0;
  int64_t pcg_iters = 0, matvecs = 0;
  double e_sse = std::nan(""), uQu = std::nan("");
};

// variance bounds of stabilize_variance (vce.cpp:1375-1389)
static double stabilize(double proposed, double previous, double y_var) {
  const double floor_v = 1e-12, ceil_v = std::max(1.0, y_var * 1e6);
  if (!std::isfinite(proposed) || proposed <= 0.0) return std::max(previous, floor_v);
  double lo = floor_v, hi = ceil_v;
  if (std::isfinite(previous) && previous > 0.0) {
    lo = std::max(lo, previous * 0.1);
    hi = std::min(hi, previous * 10.0);
  }
  if (lo > hi) lo = floor_v;
  return std::min(std::max(proposed, lo), hi);
}

static double y_variance(const Mme& m) {
  const auto& y = m.y_host;
  const size_t n = y.size();
  if (n > 1) {
    double mean = 0;
    for (double v : y) mean += v;
    mean /= (double)n;
    double ss = 0;
    for (double v : y) ss += (v - mean) * (v - mean);
    return std::max(1e-12, ss / (double)(n - 1));
  }
  return std::max(1e-12, m.yty);
}

// out[c] = sum_i A[c * lda + i] * B[c * ldb + i] for i < n, one block per
// column, summed in a fixed order.
__global__ void __launch_bounds__(256) k_coldot(const double* __restrict__ A, int64_t lda,
                                                const double* __restrict__ B, int64_t ldb, int64_t n,
                                                double* __restrict__ out) {
  __shared__ double red[256];
  const int c = blockIdx.x, tid = threadIdx.x;
  const double* a = A + (int64_t)c * lda;
  const double* b = B + (int64_t)c * ldb;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  int64_t i = tid;
  for (; i + 3 * 256 < n; i += 4 * 256) {
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] += a[i + u * 256] * b[i + u * 256];
  }
  for (; i < n; i += 256) acc[0] += a[i] * b[i];
  red[tid] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (tid < o) red[tid] += red[tid + o];
    __syncthreads();
  }
  if (tid == 0) out[c] = red[0];
}

static std::vector<double> coldots(cbx_handle* h, const double* A, int64_t lda, const double* B, int64_t ldb,
                                   int64_t n, int ncols) {
  DevBuf<double> out;
  out.resize(ncols);
  k_coldot<<<ncols, 256, 0, h->stream>>>(A, lda, B, ldb, n, out.p);
  h->launched("k_coldot");
  return d2h(h, out.p, ncols);
}

// ---------------------------------------------------------------------------
// Probe stores shared by the EM iteration and the gradient.
//
// The reference's probe stream restarts at the same seed at every call
// (AdaptiveTraceEstimator: batches of 16, batch b drawn from
// mt19937_64(seed + first index of b)), so probe j is the same vector in every
// EM iteration and every gradient call.  Per probe column the handle keeps the
// right-hand side [0; z_j] (em_B column 1 + j), the latest solution with the
// lambda it belongs to and, in mixed precision, its true residual, and
// z_j' Qinv C^uu z_j of the last forward pass (probe_zv).

// Grow b to count elements, keeping its first keep elements and zeroing the rest.
template <typename T>
static void grow_keep(cbx_handle* h, DevBuf<T>& b, size_t keep, size_t count) {
  if (b.n >= count) return;
  DevBuf<T> nb;
  nb.resize(count);
  CBX_CUDA(cudaMemsetAsync(nb.p, 0, count * sizeof(T), h->stream));
  keep = std::min(keep, b.n);
  if (keep && b.p)
    CBX_CUDA(cudaMemcpyAsync(nb.p, b.p, keep * sizeof(T), cudaMemcpyDeviceToDevice, h->stream));
  b = std::move(nb);  // the old buffer's cudaFree waits for the copy
}

// Make room for cap probe columns of the stream `seed`; a new seed forgets
// every stored probe.
static void probe_store(cbx_handle* h, Mme& m, int seed, int cap) {
  if (m.em_B_seed != seed || m.probe_seed != seed) {
    m.probe_have.assign(m.probe_have.size(), 0);
    m.probe_lam.clear();
    m.probe_r_ok.clear();
    m.fwd.valid = false;
    m.em_B_seed = m.probe_seed = seed;
  }
  if (m.probe_cap >= cap) return;
  const size_t dim = (size_t)m.dim, old = (size_t)m.probe_cap;
  grow_keep(h, m.em_B, dim * (1 + old), dim * (1 + (size_t)cap));
  grow_keep(h, m.probe_x, dim * old, dim * (size_t)cap);
  grow_keep(h, m.probe_r, dim * old, dim * (size_t)cap);
  grow_keep(h, m.probe_zv, old, (size_t)cap);
  m.probe_have.resize(cap, 0);
  m.probe_cap = cap;
}

// Probes [start, start + size) of the stream: a batch of the reference's
// estimator, drawn from mt19937_64(seed + start) with uniform_int_distribution
// <int>(0, 1) (0 -> -1, 1 -> +1), probe by probe, q values each.
static void probe_draw(int seed, int start, int size, int64_t q, double* out) {
  std::mt19937_64 gen((unsigned long)(seed + start));
  std::uniform_int_distribution<int> dist(0, 1);
  for (int j = 0; j < size; ++j)
    for (int64_t i = 0; i < q; ++i) out[(size_t)j * q + i] = dist(gen) == 0 ? -1.0 : 1.0;
}

// Put the probe batches (start, size) into rows p.. of em_B columns 1 + start ..
// (the fixed rows stay zero).  Batches the handle has not drawn yet for this seed
// and q are drawn on host threads (one per batch: each batch is its own
// generator) and kept on the device; the others are copied there.
static void probe_batches(cbx_handle* h, Mme& m, int seed, const std::vector<std::pair<int, int>>& batches) {
  const int64_t q = m.q, dim = m.dim, p = m.p;
  cudaStream_t s = h->stream;
  if (h->probe_z_seed != seed || h->probe_z_q != q) {
    h->probe_z_have.clear();
    h->probe_z_seed = seed;
    h->probe_z_q = q;
  }
  int hi = 0;
  std::vector<std::pair<int, int>> need, draw;
  for (const auto& bt : batches) {
    bool have = true;
    for (int j = 0; j < bt.second; ++j) have = have && m.probe_have[bt.first + j];
    if (have) continue;
    need.push_back(bt);
    hi = std::max(hi, bt.first + bt.second);
    bool cached = (int)h->probe_z_have.size() >= bt.first + bt.second;
    for (int j = 0; cached && j < bt.second; ++j) cached = h->probe_z_have[bt.first + j] != 0;
    if (!cached) draw.push_back(bt);
  }
  if (need.empty()) return;
  if ((int)h->probe_z_have.size() < hi) {
    grow_keep(h, h->probe_z, (size_t)q * h->probe_z_have.size(), (size_t)q * hi);
    h->probe_z_have.resize(hi, 0);
  }
  if (!draw.empty()) {
    std::vector<std::vector<double>> buf(draw.size());
    std::vector<std::thread> pool;
    for (size_t t = 0; t < draw.size(); ++t) {
      buf[t].resize((size_t)q * draw[t].second);
      pool.emplace_back(probe_draw, seed, draw[t].first, draw[t].second, q, buf[t].data());
    }
    for (auto& th : pool) th.join();
    for (size_t t = 0; t < draw.size(); ++t) {
      CBX_CUDA(cudaMemcpyAsync(h->probe_z.p + (size_t)draw[t].first * q, buf[t].data(),
                               buf[t].size() * sizeof(double), cudaMemcpyHostToDevice, s));
      for (int j = 0; j < draw[t].second; ++j) h->probe_z_have[draw[t].first + j] = 1;
    }
    CBX_CUDA(cudaStreamSynchronize(s));  // the host buffers go out of scope
  }
  for (const auto& bt : need) {
    CBX_CUDA(cudaMemcpy2DAsync(m.em_B.p + (size_t)(1 + bt.first) * dim + p, dim * sizeof(double),
                               h->probe_z.p + (size_t)bt.first * q, q * sizeof(double), q * sizeof(double),
                               bt.second, cudaMemcpyDeviceToDevice, s));
    for (int j = 0; j < bt.second; ++j) m.probe_have[bt.first + j] = 1;
  }
}

// The stored solutions of probes [c0, c0 + k) are a warm start when every one
// exists, and (mixed precision) their residuals carry to a new lambda when
// all were solved at one lambda.
static bool probes_warm(const Mme& m, int c0, int k) { return (int)m.probe_lam.size() >= c0 + k; }
static bool probes_carry(const Mme& m, int c0, int k) {
  bool ok = probes_warm(m, c0, k);
  if (ok)
    for (int c = c0; c < c0 + k; ++c) ok = ok && m.probe_r_ok[c] && m.probe_lam[c] == m.probe_lam[c0];
  return ok;
}
static void probes_record(Mme& m, int c0, int k, double lam, bool mixed) {
  if ((int)m.probe_lam.size() < c0 + k) {
    m.probe_lam.resize(c0 + k);
    m.probe_r_ok.resize(c0 + k);
  }
  for (int c = c0; c < c0 + k; ++c) {
    m.probe_lam[c] = lam;
    m.probe_r_ok[c] = mixed;
  }
}

// Solve probes [c0, c0 + k) at lam in place in probe_x (residuals into probe_r).
static void probe_solve(cbx_handle* h, Mme& m, double lam, int c0, int k, int precision, double tol, int maxit,
                        PcgResult& pr) {
  const int64_t dim = m.dim;
  const bool warm = probes_warm(m, c0, k), carry = probes_carry(m, c0, k);
  ResidCarry pc;
  pc.r_prev = carry ? m.probe_r.p + (size_t)c0 * dim : nullptr;
  pc.dlam = carry ? lam - m.probe_lam[c0] : 0.0;
  pc.r_out = m.probe_r.p + (size_t)c0 * dim;
  pcg_solve(h, lam, k, m.em_B.p + (size_t)(1 + c0) * dim, m.probe_x.p + (size_t)c0 * dim, warm, tol, maxit, 0,
            precision, pr, &pc);
  probes_record(m, c0, k, lam, precision != 0);
  for (int c = 0; c < k; ++c)
    if (pr.status[c] == sv::COL_NONFINITE) throw Error(CBX_ERR_NONFINITE, "non-finite probe solve");
}

// z_j' Qinv C^uu z_j for probe columns [c0, c0 + k) into probe_zv[c0 ..]:
// Qinv C^uu z from the solutions and their true residuals in mixed precision
// (qinv_from_solution: one sparse product), else the product with the u rows.
static void probe_values(cbx_handle* h, Mme& m, double lam, int c0, int k, bool mixed) {
  cudaStream_t s = h->stream;
  const int64_t p = m.p, q = m.q, dim = m.dim;
  const double* B = m.em_B.p + (size_t)(1 + c0) * dim;
  const double* X = m.probe_x.p + (size_t)c0 * dim;
  DevBuf<double> QW;
  QW.resize((size_t)q * k);
  if (mixed) {
    qinv_from_solution(h, lam, k, B, X, m.probe_r.p + (size_t)c0 * dim, QW.p);
  } else {
    DevBuf<double> Wu;
    Wu.resize((size_t)q * k);
    CBX_CUDA(cudaMemcpy2DAsync(Wu.p, q * sizeof(double), X + p, dim * sizeof(double), q * sizeof(double), k,
                               cudaMemcpyDeviceToDevice, s));
    qinv_apply(h, k, Wu.p, QW.p);
  }
  // the u rows of the probe columns are z
  k_coldot<<<k, 256, 0, s>>>(B + p, dim, QW.p, q, q, m.probe_zv.p + c0);
  h->launched("k_coldot");
}

// One EM iteration (vce.cpp:1490-1574).
//
// The reference solves the data system, then the probe batches of the
// adaptive trace estimator, one right-hand side at a time.  Here the probe
// batches needed before the estimator's first check are one multi-RHS block,
// and in mixed precision the data right-hand side joins that block (the
// systems share the matrix, so one read of the dense block per PCG iteration
// serves them all).  Results per column are those of separate solves: every
// column runs its own CG recurrence and refinement.  The iteration leaves its
// forward state (m.fwd) for a gradient at its starting point.  `extra` > 0 (a
// gradient from that many probes follows at this point) widens the block to
// the first `extra` probes, up to 79 (16-probe batches; the block's tensor-core
// product takes 80 columns), so that the gradient reuses their solves; the
// estimator still uses exactly the probes its stopping rule selects.
static void em_iteration(cbx_handle* h, const RemlConfigI& cfg, double& vu, double& ve, IterInfo& info,
                         int extra = 0) {
  Mme& m = *h->mme;
  cudaStream_t s = h->stream;
  const int64_t p = m.p, q = m.q, dim = m.dim, n = m.n_rec;
  const double start_vu = vu, start_ve = ve;
  const double lam = ve / std::max(vu, 1e-9);
  const bool mixed = cfg.precision != 0;
  m.fwd.valid = false;
  m.last_solution.resize(dim);
  m.last_resid.resize(dim);

  // Hutchinson schedule of the reference (vce.cpp:1266-1315,
  // adaptive_trace_estimator.cpp:11-81): batches of 16 probes, batch b seeded
  // seed + (first probe index), at least min_s and at most max_s probes, stop
  // at SE / |mean| < 0.05 checked after each batch once min_s are done.
  const int n_samp = std::max(5, cfg.mc_samples / 2);
  int min_s = std::max(30, n_samp / 3), max_s = std::max(100, n_samp);
  if (min_s <= 0) min_s = 10;
  if (max_s < min_s) max_s = min_s;
  const int batch = 16;  // max(16, 4 * threads) with one thread
  probe_store(h, m, cfg.seed, std::max(max_s, extra));
  // column 0 of em_B: W'y
  CBX_CUDA(cudaMemcpyAsync(m.em_B.p, m.rhs.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, s));

  // the probe group starting at `done`: batches solved before the next check
  struct Group {
    std::vector<std::pair<int, int>> batches;  // (start, size)
    int k = 0;
  };
  auto make_group = [&](int done) {
    Group g;
    int next = done;
    do {
      const int sz = std::min(batch, max_s - next);
      g.batches.push_back({next, sz});
      next += sz;
    } while (next < min_s && next < max_s);
    g.k = next - done;
    probe_batches(h, m, cfg.seed, g.batches);
    return g;
  };
  auto count = [&](const PcgResult& pr, int c0, int k, const char* what) {
    for (int c = c0; c < c0 + k; ++c) {
      info.pcg_iters += pr.iters[c];
      if (pr.status[c] == sv::COL_NONFINITE) throw Error(CBX_ERR_NONFINITE, what);
    }
  };

  int done = 0;
  Group g0 = make_group(0);
  // probes solved in the data block: the first group, or the gradient's first
  // `extra` probes when they are more (whole batches, 79 at most)
  const int kx = std::max(g0.k, std::min(extra, 79) / batch * batch);
  {
    std::vector<std::pair<int, int>> bts;
    for (int b = g0.k; b < kx; b += batch) bts.push_back({b, std::min(batch, kx - b)});
    probe_batches(h, m, cfg.seed, bts);
  }
  // --- 1. the data solve (with the first probe group in mixed precision)
  const bool data_warm = m.has_last;
  const bool merge = mixed && data_warm == probes_warm(m, 0, kx);
  if (merge) {
    const int k = kx, nc = 1 + k;
    DevBuf<double> X, R;
    X.resize((size_t)dim * nc);
    R.resize((size_t)dim * nc);
    const bool carry = data_warm && m.has_last_resid && probes_carry(m, 0, k) && m.last_lam == m.probe_lam[0];
    if (data_warm) {
      CBX_CUDA(cudaMemcpyAsync(X.p, m.last_solution.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
      CBX_CUDA(cudaMemcpyAsync(X.p + dim, m.probe_x.p, (size_t)dim * k * sizeof(double), cudaMemcpyDeviceToDevice,
                               s));
      if (carry) {
        CBX_CUDA(cudaMemcpyAsync(R.p, m.last_resid.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
        CBX_CUDA(cudaMemcpyAsync(R.p + dim, m.probe_r.p, (size_t)dim * k * sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
      }
    }
    ResidCarry rc;
    rc.r_prev = carry ? R.p : nullptr;
    rc.dlam = carry ? lam - m.last_lam : 0.0;
    rc.r_out = R.p;
    PcgResult pr;
    pcg_solve(h, lam, nc, m.em_B.p, X.p, data_warm, cfg.pcg_tol, cfg.pcg_max_iter, 0, cfg.precision, pr, &rc);
    if (h->trace_on) h->trace_mark("#em: data + probe solve");
    info.matvecs += pr.matvecs;
    count(pr, 0, 1, "non-finite data solve");
    count(pr, 1, k, "non-finite probe solve");
    CBX_CUDA(cudaMemcpyAsync(m.last_solution.p, X.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(m.last_resid.p, R.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(m.probe_x.p, X.p + dim, (size_t)dim * k * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(m.probe_r.p, R.p + dim, (size_t)dim * k * sizeof(double), cudaMemcpyDeviceToDevice, s));
    probes_record(m, 0, k, lam, mixed);
  } else {
    // data solve alone, warm-started from the previous data solution (and, in
    // mixed precision, from its residual carried to the new lambda)
    PcgResult r;
    ResidCarry dc;
    dc.r_prev = (m.has_last && m.has_last_resid) ? m.last_resid.p : nullptr;
    dc.dlam = lam - m.last_lam;
    dc.r_out = m.last_resid.p;
    pcg_solve(h, lam, 1, m.rhs.p, m.last_solution.p, m.has_last, cfg.pcg_tol, cfg.pcg_max_iter, 0, cfg.precision,
              r, &dc);
    if (h->trace_on) h->trace_mark("#em: data solve");
    info.matvecs += r.matvecs;
    count(r, 0, 1, "non-finite data solve");
  }
  m.has_last = true;
  m.has_last_resid = mixed;
  m.last_lam = lam;
  // --- 2. residual sum of squares
  const double e_sse = record_residual(h, m.last_solution.p, nullptr);
  // --- 3. u' Qinv u
  DevBuf<double> Qu;
  Qu.resize(q);
  if (mixed)
    qinv_from_solution(h, lam, 1, m.rhs.p, m.last_solution.p, m.last_resid.p, Qu.p);
  else
    qinv_apply(h, 1, m.last_solution.p + p, Qu.p);
  const double uQu = coldots(h, m.last_solution.p + p, q, Qu.p, q, q, 1)[0];
  if (h->trace_on) h->trace_mark("#em: e'e and u'Qinv u");
  // --- 4. Hutchinson trace of Qinv C^uu
  double tsum = 0, tsq = 0;
  bool stop = false;
  bool first = true;
  int solved = 0;
  while (done < max_s && !stop) {
    Group g = first ? std::move(g0) : make_group(done);
    const int k = g.k;
    // groups inside the data block were solved there
    if (!(merge && done + k <= kx)) {
      PcgResult pr;
      probe_solve(h, m, lam, done, k, cfg.precision, cfg.pcg_tol, cfg.pcg_max_iter, pr);
      if (h->trace_on) h->trace_mark("#em: probe solve");
      count(pr, 0, k, "non-finite probe solve");
      info.matvecs += pr.matvecs;
    }
    first = false;
    probe_values(h, m, lam, done, k, mixed);
    solved = done + k;
    const std::vector<double> zv = d2h(h, m.probe_zv.p + done, k);
    int col = 0;
    for (auto& bt : g.batches) {
      double bs = 0, bq = 0;
      for (int j = 0; j < bt.second; ++j, ++col) {
        const double v = zv[col];
        bs += v;
        bq += v * v;
      }
      tsum += bs;
      tsq += bq;
      done += bt.second;
      if (done >= min_s) {
        const double mean = tsum / done;
        const double var = (tsq - (tsum * tsum) / done) / (done - 1.0);
        const double se = std::sqrt(std::max(0.0, var) / done);
        if (std::abs(mean) > 1e-12 && (se / std::abs(mean)) < 0.05) { stop = true; break; }
      }
    }
  }
  if (merge && kx > solved) {
    // the probes solved for a following gradient: their values too
    probe_values(h, m, lam, solved, kx - solved, mixed);
    solved = kx;
  }
  const double tr = tsum / done;
  // --- 5. updates (vce.cpp:1554-1569)
  const double y_var = y_variance(m);
  const double vu_new = (uQu + tr * start_ve) / (double)q;
  vu = stabilize(vu_new, start_vu, y_var);
  const double tr_c = (double)(p + q) - lam * tr;
  const double ve_new = (e_sse + start_ve * tr_c) / (double)n;
  ve = stabilize(ve_new, start_ve, y_var);
  info.kind = 0;
  info.trace = tr;
  info.probes = done;
  info.e_sse = e_sse;
  info.uQu = uQu;
  info.var_u = vu;
  info.var_e = ve;
  Mme::Forward& f = m.fwd;
  f.vu = start_vu;
  f.ve = start_ve;
  f.pcg_tol = cfg.pcg_tol;
  f.precision = cfg.precision;
  f.seed = cfg.seed;
  f.solved = solved;
  f.uQu = uQu;
  f.e_sse = e_sse;
  f.valid = true;
}

// ---------------------------------------------------------------------------
// The REML score from the forward terms, on the device.  tr = scale * (the sum
// of the per-probe values z' Qinv C^uu z, fixed order); scale = 1 / nprobe for
// Hutchinson probes, 1 for the q unit vectors.  Then (vce.cpp:2648-2675)
//   grad_u = (u'Qinv u + var_e tr - q var_u) / (2 var_u^2)
//   grad_e = (e'e - var_e (n - p - q + min(lambda tr, q - 1e-6))) / (2 var_e^2)
// out = {grad_u, grad_e, tr}.
__global__ void __launch_bounds__(256) k_reml_score(const double* __restrict__ zv, int64_t count, double scale,
                                                    double uQu, double e_sse, double vu, double ve, int64_t n,
                                                    int64_t p, int64_t q, double* __restrict__ out) {
  __shared__ double red[256];
  const int tid = threadIdx.x;
  double a = 0.0;
  for (int64_t i = tid; i < count; i += 256) a += zv[i];
  red[tid] = a;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (tid < o) red[tid] += red[tid + o];
    __syncthreads();
  }
  if (tid == 0) {
    const double tr = red[0] * scale;
    const double lam = ve / fmax(vu, 1e-9);
    double lambda_tr = lam * tr;
    if (lambda_tr > (double)q - 1e-6) lambda_tr = (double)q - 1e-6;  // as the reference (vce.cpp:2662)
    out[0] = 0.5 * (uQu + tr * ve - (double)q * vu) / (vu * vu);
    out[1] = 0.5 * (e_sse - ve * ((double)(n - p - q) + lambda_tr)) / (ve * ve);
    out[2] = tr;
  }
}

// ---------------------------------------------------------------------------
// REML score with respect to (var_u, var_e) -- the data-driven AI-REML score of
// run_aireml_step (vce.cpp:2648-2675), which is the exact REML derivative:
//   d logL / d var_u = (u'Qinv u + var_e tr - q var_u) / (2 var_u^2)
//   d logL / d var_e = (e'e - var_e (n - p - q + lambda tr)) / (2 var_e^2)
// with tr = tr(Qinv C^uu) estimated from `nprobe` Rademacher probes (the
// reference's probe stream, batches of 16 seeded seed + first index) solved as
// multi-RHS blocks, or exactly from the q unit vectors (exact != 0).
//
// Backward pass over the forward state: when the handle's last EM iteration
// (or gradient) ran at this very point with the same probe seed, precision and
// tolerance, its data-solve terms and the values of the probes it solved are
// reused, and only probes beyond those are solved.  Those start from their
// stored solutions of the previous call, with their true residuals carried to
// the new lambda in mixed precision.  A gradient right after an EM iteration
// with nprobe no larger than the iteration's probe count costs no solve.
static void reml_gradient(cbx_handle* h, double vu, double ve, int nprobe, int seed, int exact, int precision,
                          double pcg_tol, int pcg_maxit, double* grad, double* trace_out, int64_t* iters_out) {
  Mme& m = *h->mme;
  cudaStream_t s = h->stream;
  const int64_t p = m.p, q = m.q, dim = m.dim, n = m.n_rec;
  const double lam = ve / std::max(vu, 1e-9);
  const bool mixed = precision != 0;
  const int64_t total = exact ? q : nprobe;
  CBX_REQUIRE(total > 0, CBX_ERR_ARG, "nprobe must be positive");
  int64_t iters = 0;
  Mme::Forward& f = m.fwd;
  const bool reuse = f.valid && f.vu == vu && f.ve == ve && f.precision == precision && f.pcg_tol == pcg_tol;
  double uQu, e_sse;
  if (reuse) {
    uQu = f.uQu;
    e_sse = f.e_sse;
  } else {
    // the data solve, warm-started from the last data solution (its residual
    // carried to this lambda in mixed precision)
    f.valid = false;
    m.last_solution.resize(dim);
    m.last_resid.resize(dim);
    PcgResult r;
    ResidCarry dc;
    dc.r_prev = (m.has_last && m.has_last_resid) ? m.last_resid.p : nullptr;
    dc.dlam = lam - m.last_lam;
    dc.r_out = m.last_resid.p;
    pcg_solve(h, lam, 1, m.rhs.p, m.last_solution.p, m.has_last, pcg_tol, pcg_maxit, 0, precision, r, &dc);
    CBX_REQUIRE(r.status[0] != sv::COL_NONFINITE, CBX_ERR_NONFINITE, "non-finite data solve");
    iters += r.iters[0];
    m.has_last = true;
    m.has_last_resid = mixed;
    m.last_lam = lam;
    e_sse = record_residual(h, m.last_solution.p, nullptr);
    DevBuf<double> Qu;
    Qu.resize(q);
    if (mixed)
      qinv_from_solution(h, lam, 1, m.rhs.p, m.last_solution.p, m.last_resid.p, Qu.p);
    else
      qinv_apply(h, 1, m.last_solution.p + p, Qu.p);
    uQu = coldots(h, m.last_solution.p + p, q, Qu.p, q, q, 1)[0];
  }
  DevBuf<double> zv_exact, out;
  out.resize(3);
  const double* zv = nullptr;
  if (exact) {
    // the q unit vectors, cold, in blocks (64 columns in mixed precision, whose
    // PCG bulk reads the FP32 block once per iteration for all of them; the
    // FP64 product is FP64-bound, so 32 there)
    const int64_t blk = mixed ? 64 : 32;
    zv_exact.resize(q);
    for (int64_t c0 = 0; c0 < q; c0 += blk) {
      const int k = (int)std::min<int64_t>(blk, q - c0);
      std::vector<double> Bh((size_t)dim * k, 0.0);
      for (int j = 0; j < k; ++j) Bh[(size_t)j * dim + p + c0 + j] = 1.0;
      DevBuf<double> B, X, QW, R;
      B.resize((size_t)dim * k);
      X.resize((size_t)dim * k);
      QW.resize((size_t)q * k);
      CBX_CUDA(cudaMemcpyAsync(B.p, Bh.data(), Bh.size() * sizeof(double), cudaMemcpyHostToDevice, s));
      PcgResult pr;
      ResidCarry pc;
      if (mixed) {
        R.resize((size_t)dim * k);
        pc.r_out = R.p;
      }
      pcg_solve(h, lam, k, B.p, X.p, false, pcg_tol, pcg_maxit, 0, precision, pr, &pc);
      for (int c = 0; c < k; ++c) iters += pr.iters[c];
      if (mixed) {
        qinv_from_solution(h, lam, k, B.p, X.p, R.p, QW.p);
      } else {
        DevBuf<double> Wu;
        Wu.resize((size_t)q * k);
        CBX_CUDA(cudaMemcpy2DAsync(Wu.p, q * sizeof(double), X.p + p, dim * sizeof(double), q * sizeof(double), k,
                                   cudaMemcpyDeviceToDevice, s));
        qinv_apply(h, k, Wu.p, QW.p);
      }
      k_coldot<<<k, 256, 0, s>>>(B.p + p, dim, QW.p, q, q, zv_exact.p + c0);
      h->launched("k_coldot");
      CBX_CUDA(cudaStreamSynchronize(s));  // B and Bh are released at the end of this block
    }
    zv = zv_exact.p;
  } else {
    probe_store(h, m, seed, std::max(nprobe, m.probe_cap));
    const int prev = (reuse && f.seed == seed) ? f.solved : 0;
    const int have = std::min(prev, nprobe);
    // blocks of 64 columns in mixed precision, 32 in FP64 (as above), on
    // 16-probe batch boundaries
    const int blk = mixed ? 64 : 32;
    for (int c0 = have; c0 < nprobe;) {
      const int k = std::min(blk - (c0 % 16), nprobe - c0);
      std::vector<std::pair<int, int>> bts;
      for (int b = c0 - c0 % 16; b < c0 + k; b += 16) bts.push_back({b, std::min(16, m.probe_cap - b)});
      probe_batches(h, m, seed, bts);
      PcgResult pr;
      probe_solve(h, m, lam, c0, k, precision, pcg_tol, pcg_maxit, pr);
      for (int c = 0; c < k; ++c) iters += pr.iters[c];
      probe_values(h, m, lam, c0, k, mixed);
      c0 += k;
    }
    zv = m.probe_zv.p;
    // this call's solves are now the forward state at (vu, ve)
    f.vu = vu;
    f.ve = ve;
    f.pcg_tol = pcg_tol;
    f.precision = precision;
    f.seed = seed;
    f.solved = std::max(prev, nprobe);
    f.uQu = uQu;
    f.e_sse = e_sse;
    f.valid = true;
  }
  k_reml_score<<<1, 256, 0, s>>>(zv, total, exact ? 1.0 : 1.0 / (double)total, uQu, e_sse, vu, ve, n, p, q, out.p);
  h->launched("k_reml_score");
  const std::vector<double> o = d2h(h, out.p, 3);
  grad[0] = o[0];
  grad[1] = o[1];
  if (trace_out) *trace_out = o[2];
  if (iters_out) *iters_out = iters;
}

// ---------------------------------------------------------------------------
// dense exact AI step
struct DenseExact {
  bool init = false;
  int64_t n = 0, dim = 0;
  DevBuf<double> ZAZt;
  double log_det_A = 0;
};
static DenseExact& dense_state(cbx_handle* h) {
  if (!h->dense_slot) h->dense_slot = std::make_shared<DenseExact>();
  return *static_cast<DenseExact*>(h->dense_slot.get());
}

static void dense_init(cbx_handle* h, DenseExact& D) {
  Mme& m = *h->mme;
  CBX_REQUIRE(m.has_dense && !m.has_sparse && m.ng == m.q, CBX_ERR_UNSUPPORTED,
              "dense exact AI needs a dense Qinv");
  cudaStream_t s = h->stream;
  const int64_t q = m.q, n = m.n_rec, dim = m.dim;
  // A = Qinv^-1 via Cholesky (initialize_dense, vce.cpp:2890-2897); log|A| = -log|Qinv|
  DevBuf<double> A;
  A.resize((size_t)q * q);
  CBX_CUDA(cudaMemcpy2DAsync(A.p, q * sizeof(double), m.Qd64.p, m.ld * sizeof(double), q * sizeof(double), q,
                             cudaMemcpyDeviceToDevice, s));
  CBX_REQUIRE(potrf(h, A.p, q), CBX_ERR_FACTOR, "Qinv is not positive definite");
  D.log_det_A = -2.0 * log_diag(h, A.p, q);
  {
    Libs& L = libs(h);
    int lw = 0;
    CBX_SOLVER(cusolverDnDpotri_bufferSize(L.sol, CUBLAS_FILL_MODE_LOWER, (int)q, A.p, (int)q, &lw));
    DevBuf<double> work;
    work.resize(std::max(lw, 1));
    DevBuf<int> info;
    info.resize(1);
    CBX_SOLVER(cusolverDnDpotri(L.sol, CUBLAS_FILL_MODE_LOWER, (int)q, A.p, (int)q, work.p, lw, info.p));
    k_symmetrize_lower<<<gridn(q * q, 256, 8 * h->num_sms), 256, 0, s>>>(A.p, q);
    h->launched("k_symmetrize_lower");
  }
  D.ZAZt.resize((size_t)n * n);
  k_build_zazt<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(n, q, m.aid.p, A.p, D.ZAZt.p);
  h->launched("k_build_zazt");
  CBX_CUDA(cudaStreamSynchronize(s));
  D.n = n;
  D.dim = dim;
  D.init = true;
}

// Factor C(lambda) in C (dim x dim); returns false if not PD.
static bool factor_lhs(cbx_handle* h, double lam, DevBuf<double>& C) {
  Mme& m = *h->mme;
  cudaStream_t s = h->stream;
  const int64_t dim = m.dim;
  C.resize((size_t)dim * dim);
  k_build_lhs<<<gridn(dim * dim, 256, 8 * h->num_sms), 256, 0, s>>>(dim, m.p, m.D64.ptr.p, m.D64.col.p, m.D64.val.p,
                                                                     m.Qd64.p, m.ld, lam, C.p);
  h->launched("k_build_lhs");
  k_scatter_csr<<<gridn(dim, 256, 4 * h->num_sms), 256, 0, s>>>(dim, m.D64.ptr.p, m.D64.col.p, m.D64.val.p, C.p);
  h->launched("k_scatter_csr");
  return potrf(h, C.p, dim);
}

// compute_logL of run_dense_exact_step (vce.cpp:2974-3007); -1e18 if C is not PD
static double dense_logL(cbx_handle* h, DenseExact& D, double vu, double ve, DevBuf<double>& C, DevBuf<double>& sol,
                         double* ld_out = nullptr) {
  Mme& m = *h->mme;
  const int64_t n = m.n_rec, p = m.p, q = m.q, dim = m.dim;
  if (!factor_lhs(h, ve / vu, C)) return -1e18;
  const double ld_C = 2.0 * log_diag(h, C.p, dim);
  if (!std::isfinite(ld_C)) return -1e18;
  sol.resize(dim);
  CBX_CUDA(cudaMemcpyAsync(sol.p, m.rhs.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  potrs(h, C.p, dim, sol.p, 1);
  DevBuf<double> e;
  e.resize(n);
  record_residual(h, sol.p, e.p);
  const auto eh = d2h(h, e.p, n);
  const double yPy = dot_h(m.y_host, eh) / ve;
  if (ld_out) *ld_out = ld_C;
  const double m2 = ld_C + (double)(n - p - q) * std::log(ve) + (double)q * std::log(vu) + yPy + D.log_det_A;
  return -0.5 * m2;
}

static void project_spd_2x2(double A[2][2], double eps_rel = 1e-8, double eps_abs = 1e-12) {
  const double a = A[0][0], b = 0.5 * (A[0][1] + A[1][0]), d = A[1][1];
  // eigen-decomposition of [[a, b], [b, d]]
  const double tr = a + d, det = a * d - b * b;
  const double disc = std::sqrt(std::max(0.0, 0.25 * tr * tr - det));
  double l1 = 0.5 * tr - disc, l2 = 0.5 * tr + disc;  // ascending
  double v1x, v1y;
  if (std::abs(b) > 0) {
    v1x = l1 - d;
    v1y = b;
  } else {
    if (a <= d) { v1x = 1; v1y = 0; } else { v1x = 0; v1y = 1; }
    l1 = std::min(a, d);
    l2 = std::max(a, d);
  }
  const double nr = std::hypot(v1x, v1y);
  v1x /= nr;
  v1y /= nr;
  const double v2x = -v1y, v2y = v1x;
  const double floor_v = std::max(eps_abs, eps_rel * std::max(l2, 0.0));
  l1 = std::max(l1, floor_v);
  l2 = std::max(l2, floor_v);
  A[0][0] = l1 * v1x * v1x + l2 * v2x * v2x;
  A[0][1] = A[1][0] = l1 * v1x * v1y + l2 * v2x * v2y;
  A[1][1] = l1 * v1y * v1y + l2 * v2y * v2y;
}

static bool dense_exact_step(cbx_handle* h, double& vu_io, double& ve_io, IterInfo& info) {
  Mme& m = *h->mme;
  DenseExact& D = dense_state(h);
  if (!D.init || D.n != m.n_rec || D.dim != m.dim) dense_init(h, D);
  cudaStream_t s = h->stream;
  Libs& L = libs(h);
  const int64_t n = m.n_rec, dim = m.dim;
  const double vu = vu_io, ve = ve_io;
  DevBuf<double> C, sol;
  const double cur0 = dense_logL(h, D, vu, ve, C, sol);
  if (cur0 <= -1e18) return false;
  double cur = cur0;
  // P = (I - W C^-1 W^T) / ve from the explicit C^-1 (inverse of the factor),
  // then M_u = P ZAZ^T: the FP64 products on this library's kernels
  DevBuf<double> Ci;
  Ci.resize((size_t)dim * dim);
  CBX_CUDA(cudaMemcpyAsync(Ci.p, C.p, (size_t)dim * dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
  {
    int lw = 0;
    CBX_SOLVER(cusolverDnDpotri_bufferSize(L.sol, CUBLAS_FILL_MODE_LOWER, (int)dim, Ci.p, (int)dim, &lw));
    DevBuf<double> work;
    work.resize(std::max(lw, 1));
    DevBuf<int> info;
    info.resize(1);
    CBX_SOLVER(cusolverDnDpotri(L.sol, CUBLAS_FILL_MODE_LOWER, (int)dim, Ci.p, (int)dim, work.p, lw, info.p));
    k_symmetrize_lower<<<gridn(dim * dim, 256, 8 * h->num_sms), 256, 0, s>>>(Ci.p, dim);
    h->launched("k_symmetrize_lower");
  }
  DevBuf<double> P, Mu;
  P.resize((size_t)n * n);
  Mu.resize((size_t)n * n);
  k_build_P_ci<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(n, m.p, m.q, dim, m.aid.p, m.x_ptr.p, m.x_col.p,
                                                                  m.x_val.p, Ci.p, ve, P.p);
  h->launched("k_build_P_ci");
  k_dgemm_nn<<<dim3((unsigned)((n + 63) / 64), (unsigned)((n + 63) / 64)), 256, 0, s>>>(n, P.p, D.ZAZt.p, Mu.p);
  h->launched("k_dgemm_nn");
  const unsigned g = gridn(n * n, 256, 4 * h->num_sms);
  DevBuf<double> part;
  part.resize((size_t)g * 5);
  k_ai_traces<<<g, 256, 0, s>>>(Mu.p, P.p, n, part.p);
  h->launched("k_ai_traces");
  const auto ph = d2h(h, part.p, (size_t)g * 5);
  double sums[5] = {0, 0, 0, 0, 0};
  for (unsigned b = 0; b < g; ++b)
    for (int k = 0; k < 5; ++k) sums[k] += ph[(size_t)b * 5 + k];
  // Py = e / ve; score terms
  DevBuf<double> e, ZPy;
  e.resize(n);
  ZPy.resize(n);
  record_residual(h, sol.p, e.p);
  std::vector<double> Py = d2h(h, e.p, n);
  for (auto& v : Py) v /= ve;
  DevBuf<double> dPy;
  dPy.resize(n);
  CBX_CUDA(cudaMemcpyAsync(dPy.p, Py.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
  k_dgemv_n<<<gridn(n, 256, 4 * h->num_sms), 256, 0, s>>>(n, D.ZAZt.p, dPy.p, ZPy.p);
  h->launched("k_dgemv_n");
  const auto ZPyh = d2h(h, ZPy.p, n);
  const double score_u = dot_h(Py, ZPyh), score_e = dot_h(Py, Py);
  const double grad_u = -0.5 * sums[3] + 0.5 * score_u;
  const double grad_e = -0.5 * sums[4] + 0.5 * score_e;
  double AI[2][2] = {{0.5 * sums[0], 0.5 * sums[1]}, {0.5 * sums[1], 0.5 * sums[2]}};
  project_spd_2x2(AI);
  double delta[2];
  {
    // LLT of the 2x2 AI (AI is SPD after the projection)
    const double l11 = std::sqrt(AI[0][0]);
    const double l21 = AI[1][0] / l11;
    const double l22sq = AI[1][1] - l21 * l21;
    if (!(l11 > 0) || !(l22sq > 0)) {
      const double det = AI[0][0] * AI[1][1] - AI[0][1] * AI[1][0];
      if (std::abs(det) < 1e-20) return false;
      delta[0] = (AI[1][1] * grad_u - AI[0][1] * grad_e) / det;
      delta[1] = (-AI[1][0] * grad_u + AI[0][0] * grad_e) / det;
    } else {
      const double l22 = std::sqrt(l22sq);
      const double y0 = grad_u / l11, y1 = (grad_e - l21 * y0) / l22;
      delta[1] = y1 / l22;
      delta[0] = (y0 - l21 * delta[1]) / l11;
    }
  }
  // step halving on logL (vce.cpp:3150-3171)
  const int max_halving = 6;
  for (int k = 0; k < max_halving; ++k) {
    const double vu_n = vu + delta[0], ve_n = ve + delta[1];
    if (vu_n > 0 && ve_n > 0) {
      DevBuf<double> C2, s2;
      const double nl = dense_logL(h, D, vu_n, ve_n, C2, s2);
      if (nl > cur || k == max_halving - 1) {
        cur = nl;
        vu_io = vu_n;
        ve_io = ve_n;
        m.last_solution.resize(dim);
        CBX_CUDA(cudaMemcpyAsync(m.last_solution.p, sol.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
        m.has_last = true;
        info.kind = 1;
        info.logL = cur;
        info.var_u = vu_io;
        info.var_e = ve_io;
        return true;
      }
    }
    delta[0] *= 0.5;
    delta[1] *= 0.5;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Data-driven AI step: run_aireml_step (vce.cpp:2414-2857) for one random
// component, on the branch where the reference has a direct solver.  The LHS
// is factored densely on the device (Cholesky), which gives the exact
// tr(Qinv C^uu) (the reference's Takahashi value), the AI matrix from two extra
// solves and calc_logL_internal (vce.cpp:3533-3588) for the logL-checked step
// halving.  Without a factorization the reference cannot check logL and falls
// back to EM (vce.cpp:2791-2797); so does this step above kAiDenseMax.
constexpr int64_t kAiDenseMax = 24576;

// Dense q x q Qinv: the sparse part scattered row by row, then the dense block
// at its genotyped rows (each entry written by one thread).
__global__ void k_qinv_sparse_scatter(int64_t q, const int32_t* __restrict__ Sptr, const int32_t* __restrict__ Scol,
                                      const double* __restrict__ Sval, double* __restrict__ Q) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < q; r += (int64_t)gridDim.x * blockDim.x)
    for (int32_t j = Sptr[r]; j < Sptr[r + 1]; ++j) Q[(int64_t)Scol[j] * q + r] += Sval[j];
}
__global__ void k_qinv_dense_scatter(int64_t ng, const double* __restrict__ Qd, int64_t ld,
                                     const int32_t* __restrict__ gmap, int64_t q, double* __restrict__ Q) {
  const int64_t total = ng * ng;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = idx / ng, l = idx - k * ng;
    Q[(int64_t)gmap[l] * q + gmap[k]] += Qd[k * ld + l];
  }
}
// partial sums of sum_{i,j < q} Q[j q + i] Ci[(p + j) dim + p + i]: tr(Qinv C^uu)
__global__ void k_trace_qc(const double* __restrict__ Q, const double* __restrict__ Ci, int64_t q, int64_t p,
                           int64_t dim, double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  const int64_t total = q * q;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / q, i = idx - j * q;
    s += Q[idx] * Ci[(p + j) * dim + p + i];
  }
  const double t = sv::block_sum_cols<1>(s, red);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

static void dense_qinv(cbx_handle* h, DevBuf<double>& Q) {
  Mme& m = *h->mme;
  cudaStream_t s = h->stream;
  const int64_t q = m.q;
  Q.resize((size_t)q * q);
  Q.zero(s);
  if (m.has_sparse) {
    k_qinv_sparse_scatter<<<gridn(q, 256, 4 * h->num_sms), 256, 0, s>>>(q, m.Qs64.ptr.p, m.Qs64.col.p, m.Qs64.val.p,
                                                                       Q.p);
    h->launched("k_qinv_sparse_scatter");
  }
  if (m.has_dense) {
    k_qinv_dense_scatter<<<gridn(m.ng * m.ng, 256, 8 * h->num_sms), 256, 0, s>>>(m.ng, m.Qd64.p, m.ld, m.gmap.p,
                                                                                q, Q.p);
    h->launched("k_qinv_dense_scatter");
  }
}

// C = W'W + lam [0 0; 0 Q] (dim x dim) factored in place; false if not PD
static bool factor_lhs_q(cbx_handle* h, const double* Q, double lam, DevBuf<double>& C) {
  Mme& m = *h->mme;
  cudaStream_t s = h->stream;
  const int64_t dim = m.dim;
  C.resize((size_t)dim * dim);
  k_build_lhs<<<gridn(dim * dim, 256, 8 * h->num_sms), 256, 0, s>>>(dim, m.p, m.D64.ptr.p, m.D64.col.p, m.D64.val.p,
                                                                     Q, m.q, lam, C.p);
  h->launched("k_build_lhs");
  k_scatter_csr<<<gridn(dim, 256, 4 * h->num_sms), 256, 0, s>>>(dim, m.D64.ptr.p, m.D64.col.p, m.D64.val.p, C.p);
  h->launched("k_scatter_csr");
  return potrf(h, C.p, dim);
}

// calc_logL_internal: -1/2 (log|C| + (n - p - q) log ve + q log vu + (y'y - sol'W'y) / ve),
// log|C| from the Cholesky factor; -1e20 when C is not positive definite.  C
// keeps the factor and sol the data solution.
static double ai_logl(cbx_handle* h, const double* Q, double vu, double ve, DevBuf<double>& C,
                      std::vector<double>& sol) {
  Mme& m = *h->mme;
  const int64_t n = m.n_rec, p = m.p, q = m.q, dim = m.dim;
  if (!factor_lhs_q(h, Q, ve / std::max(vu, 1e-9), C)) return -1e20;
  const double ld = 2.0 * log_diag(h, C.p, dim);
  if (!std::isfinite(ld)) return -1e20;
  DevBuf<double> x;
  x.resize(dim);
  CBX_CUDA(cudaMemcpyAsync(x.p, m.rhs.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  potrs(h, C.p, dim, x.p, 1);
  sol = d2h(h, x.p, dim);
  const double yPy = (m.yty - dot_h(sol, m.rhs_host)) / ve;
  return -0.5 * (ld + (double)(n - p - q) * std::log(ve) + (double)q * std::log(std::max(vu, 1e-9)) + yPy);
}

// W'v (mult_transpose_design, mme_builder.cpp:330-388) and W x (mult_design,
// :390-423) over the host copy of the records, in record order
static std::vector<double> wt_v(const Mme& m, const std::vector<double>& v) {
  std::vector<double> out(m.dim, 0.0);
  for (int64_t i = 0; i < m.n_rec; ++i) {
    for (int32_t a = m.xp_host[i]; a < m.xp_host[i + 1]; ++a) out[m.xc_host[a]] += m.xv_host[a] * v[i];
    const int32_t an = m.aid_host[i];
    if (an > 0 && an <= m.q) out[m.p + an - 1] += v[i];
  }
  return out;
}
static std::vector<double> w_x(const Mme& m, const std::vector<double>& x) {
  std::vector<double> out(m.n_rec, 0.0);
  for (int64_t i = 0; i < m.n_rec; ++i) {
    double val = 0.0;
    for (int32_t a = m.xp_host[i]; a < m.xp_host[i + 1]; ++a)
      if (m.xc_host[a] < m.p) val += m.xv_host[a] * x[m.xc_host[a]];
    const int32_t an = m.aid_host[i];
    if (an > 0 && an <= m.q) val += x[m.p + an - 1];
    out[i] = val;
  }
  return out;
}

// Newton direction AI^-1 grad with the reference's fallbacks (vce.cpp:2697-2737):
// LLT of the 2x2; if that fails, a gradient-ascent step of 10 % of the variances
// when |det AI| < 1e-20, else the inverse.
static void ai_direction(const double AI[2][2], const double g[2], double vu, double ve, double d[2]) {
  const double l11sq = AI[0][0];
  const double l11 = l11sq > 0 ? std::sqrt(l11sq) : 0.0;
  const double l21 = l11 > 0 ? AI[1][0] / l11 : 0.0;
  const double l22sq = AI[1][1] - l21 * l21;
  if (l11 > 0 && l22sq > 0) {
    const double l22 = std::sqrt(l22sq);
    const double y0 = g[0] / l11, y1 = (g[1] - l21 * y0) / l22;
    d[1] = y1 / l22;
    d[0] = (y0 - l21 * d[1]) / l11;
    return;
  }
  const double det = AI[0][0] * AI[1][1] - AI[0][1] * AI[1][0];
  if (std::abs(det) < 1e-20) {
    const double mx = std::max(std::abs(g[0]) / vu, std::abs(g[1]) / ve);
    const double sc = mx > 0 ? 0.1 / mx : 0.0;
    d[0] = g[0] * sc;
    d[1] = g[1] * sc;
    return;
  }
  d[0] = (AI[1][1] * g[0] - AI[0][1] * g[1]) / det;
  d[1] = (-AI[1][0] * g[0] + AI[0][0] * g[1]) / det;
}

static bool ai_data_step(cbx_handle* h, double& vu_io, double& ve_io, IterInfo& info) {
  Mme& m = *h->mme;
  if (m.dim > kAiDenseMax) return false;
  // guard against non-finite variances entering the step (vce.cpp:2417-2419)
  if (!std::isfinite(vu_io) || vu_io <= 0.0) vu_io = 1e-6;
  if (!std::isfinite(ve_io) || ve_io <= 0.0) ve_io = 1e-6;
  const double vu = vu_io, ve = ve_io;
  const int64_t n = m.n_rec, p = m.p, q = m.q, dim = m.dim;
  const double lam = ve / std::max(vu, 1e-9);
  cudaStream_t s = h->stream;
  DevBuf<double> Q, C;
  dense_qinv(h, Q);
  std::vector<double> sol;
  const double cur0 = ai_logl(h, Q.p, vu, ve, C, sol);
  if (cur0 <= -1e20) return false;
  // data terms: u, e = y - W sol, u'Qinv u
  const std::vector<double> u(sol.begin() + p, sol.end());
  const std::vector<double> yhat = w_x(m, sol);
  std::vector<double> e(n);
  for (int64_t i = 0; i < n; ++i) e[i] = m.y_host[i] - yhat[i];
  DevBuf<double> du, dQu;
  du.resize(q);
  dQu.resize(q);
  CBX_CUDA(cudaMemcpyAsync(du.p, u.data(), q * sizeof(double), cudaMemcpyHostToDevice, s));
  qinv_apply(h, 1, du.p, dQu.p);
  const double uQu = dot_h(u, d2h(h, dQu.p, q));
  // exact tr(Qinv C^uu) from C^-1
  double tr = 0.0;
  {
    DevBuf<double> Ci;
    Ci.resize((size_t)dim * dim);
    k_build_lhs<<<gridn(dim * dim, 256, 8 * h->num_sms), 256, 0, s>>>(dim, p, m.D64.ptr.p, m.D64.col.p,
                                                                       m.D64.val.p, Q.p, q, lam, Ci.p);
    h->launched("k_build_lhs");
    k_scatter_csr<<<gridn(dim, 256, 4 * h->num_sms), 256, 0, s>>>(dim, m.D64.ptr.p, m.D64.col.p, m.D64.val.p, Ci.p);
    h->launched("k_scatter_csr");
    if (!chol_inverse_device(h, Ci.p, dim)) return false;
    const unsigned g = gridn(q * q, 256, 4 * h->num_sms);
    DevBuf<double> part;
    part.resize(g);
    k_trace_qc<<<g, 256, 0, s>>>(Q.p, Ci.p, q, p, dim, part.p);
    h->launched("k_trace_qc");
    for (double v : d2h(h, part.p, g)) tr += v;
  }
  // AI_ij = 1/2 v_i' P v_j from two extra solves (vce.cpp:2596-2633):
  // v_u = Z u / vu, v_e = e / ve; P v = (v - W C^-1 W'v) / ve
  std::vector<double> vu_v(n, 0.0), ve_v(n);
  for (int64_t i = 0; i < n; ++i) {
    const int32_t an = m.aid_host[i];
    if (an > 0 && an <= q) vu_v[i] = u[an - 1] / vu;
    ve_v[i] = e[i] / ve;
  }
  std::vector<double> rhs2 = wt_v(m, vu_v);
  {
    const std::vector<double> r2 = wt_v(m, ve_v);
    rhs2.insert(rhs2.end(), r2.begin(), r2.end());
  }
  DevBuf<double> B2;
  B2.resize((size_t)dim * 2);
  CBX_CUDA(cudaMemcpyAsync(B2.p, rhs2.data(), rhs2.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  potrs(h, C.p, dim, B2.p, 2);
  const std::vector<double> x2 = d2h(h, B2.p, (size_t)dim * 2);
  const std::vector<double> xu(x2.begin(), x2.begin() + dim), xe(x2.begin() + dim, x2.end());
  const std::vector<double> yu = w_x(m, xu), ye = w_x(m, xe);
  std::vector<double> Pvu(n), Pve(n);
  for (int64_t i = 0; i < n; ++i) {
    Pvu[i] = (vu_v[i] - yu[i]) / ve;
    Pve[i] = (ve_v[i] - ye[i]) / ve;
  }
  double AI[2][2];
  AI[0][0] = 0.5 * dot_h(vu_v, Pvu);
  AI[1][1] = 0.5 * dot_h(ve_v, Pve);
  AI[0][1] = AI[1][0] = 0.5 * dot_h(vu_v, Pve);
  // the EM-consistent score (vce.cpp:2648-2675)
  double lambda_tr = lam * tr;
  if (lambda_tr > (double)q - 1e-6) lambda_tr = (double)q - 1e-6;
  const double grad[2] = {0.5 * (uQu + tr * ve - (double)q * vu) / (vu * vu),
                          0.5 * (dot_h(e, e) - ve * ((double)(n - p - q) + lambda_tr)) / (ve * ve)};
  project_spd_2x2(AI);
  double d[2];
  ai_direction(AI, grad, vu, ve, d);
  if (!std::isfinite(d[0]) || !std::isfinite(d[1])) return false;
  if (std::abs(d[0]) > 100.0 * vu || std::abs(d[1]) > 100.0 * ve) return false;
  const double cur = std::isfinite(cur0) ? cur0 : -1e18;
  // at most 15 halvings; a candidate must keep both variances positive, move
  // neither by more than 5x, and raise logL (vce.cpp:2797-2839)
  for (int k = 0; k < 15; ++k) {
    const double vu_n = vu + d[0], ve_n = ve + d[1];
    if (vu_n <= 0.0 || ve_n <= 0.0 || std::abs(d[0]) > 5.0 * vu || std::abs(d[1]) > 5.0 * ve) {
      d[0] *= 0.5;
      d[1] *= 0.5;
      continue;
    }
    DevBuf<double> C2;
    std::vector<double> sol2;
    const double nl = ai_logl(h, Q.p, vu_n, ve_n, C2, sol2);
    if (std::isfinite(nl) && nl > cur) {
      vu_io = vu_n;
      ve_io = ve_n;
      m.last_solution.resize(dim);
      CBX_CUDA(cudaMemcpyAsync(m.last_solution.p, sol.data(), dim * sizeof(double), cudaMemcpyHostToDevice, s));
      CBX_CUDA(cudaStreamSynchronize(s));
      m.has_last = true;
      m.has_last_resid = false;
      info.kind = 2;
      info.logL = nl;
      info.trace = tr;
      info.e_sse = dot_h(e, e);
      info.uQu = uQu;
      info.var_u = vu_n;
      info.var_e = ve_n;
      return true;
    }
    d[0] *= 0.5;
    d[1] *= 0.5;
  }
  return false;
}

static void reml_iterate(cbx_handle* h, const RemlConfigI& cfg, double& vu, double& ve, IterInfo& info,
                         int extra = 0) {
  Mme& m = *h->mme;
  if (cfg.mode == 3) {
    if (ai_data_step(h, vu, ve, info)) return;
  } else {
    const bool dense = cfg.mode == 2 || (cfg.mode == 0 && m.dim < 5000);
    if (dense && dense_exact_step(h, vu, ve, info)) return;
  }
  em_iteration(h, cfg, vu, ve, info, extra);
}

}  // namespace cbx

using namespace cbx;

static RemlConfigI to_cfg(const cbx_reml_config* c) {
  RemlConfigI r;
  if (c) {
    r.max_iter = c->max_iter;
    r.tol = c->tol;
    r.mc_samples = c->mc_samples;
    r.pcg_max_iter = c->pcg_max_iter;
    r.pcg_tol = c->pcg_tol;
    r.precision = c->precision;
    r.mode = c->mode;
    r.seed = c->seed;
  }
  return r;
}
static void to_info(const IterInfo& i, cbx_reml_iter_info* o) {
  if (!o) return;
  o->kind = i.kind;
  o->var_u = i.var_u;
  o->var_e = i.var_e;
  o->logL = i.logL;
  o->trace = i.trace;
  o->probes = i.probes;
  o->pcg_iters = i.pcg_iters;
  o->matvecs = i.matvecs;
  o->e_sse = i.e_sse;
  o->uQu = i.uQu;
}

extern "C" void cbx_reml_config_default(cbx_reml_config* c) {
  if (!c) return;
  RemlConfigI d;
  c->max_iter = d.max_iter;
  c->tol = d.tol;
  c->mc_samples = d.mc_samples;
  c->pcg_max_iter = d.pcg_max_iter;
  c->pcg_tol = d.pcg_tol;
  c->precision = d.precision;
  c->mode = d.mode;
  c->seed = d.seed;
}

extern "C" int cbx_reml_iterate(cbx_handle* h, const cbx_reml_config* cfg, double* var_u, double* var_e,
                                cbx_reml_iter_info* info) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create and cbx_mme_set_qinv_* first");
    CBX_REQUIRE(var_u && var_e && *var_u > 0 && *var_e > 0, CBX_ERR_ARG, "variances must be positive");
    CBX_CUDA(cudaSetDevice(h->device));
    IterInfo it;
    reml_iterate(h, to_cfg(cfg), *var_u, *var_e, it);
    to_info(it, info);
  });
}

extern "C" int cbx_reml_iterate_grad(cbx_handle* h, const cbx_reml_config* cfg, int32_t nprobe, double* var_u,
                                     double* var_e, cbx_reml_iter_info* info, double* grad, double* trace,
                                     int64_t* grad_pcg_iters, double* solution) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create and cbx_mme_set_qinv_* first");
    CBX_REQUIRE(var_u && var_e && *var_u > 0 && *var_e > 0, CBX_ERR_ARG, "variances must be positive");
    CBX_REQUIRE(nprobe > 0 && grad, CBX_ERR_ARG, "nprobe must be positive and grad non-null");
    CBX_CUDA(cudaSetDevice(h->device));
    const RemlConfigI c = to_cfg(cfg);
    const double vu0 = *var_u, ve0 = *var_e;
    IterInfo it;
    reml_iterate(h, c, *var_u, *var_e, it, nprobe);
    to_info(it, info);
    cbx::reml_gradient(h, vu0, ve0, nprobe, c.seed, 0, c.precision, c.pcg_tol, c.pcg_max_iter, grad, trace,
                       grad_pcg_iters);
    if (solution && h->mme->has_last)
      CBX_CUDA(cudaMemcpy(solution, h->mme->last_solution.p, h->mme->dim * sizeof(double), cudaMemcpyDeviceToHost));
  });
}

extern "C" int cbx_reml_solve(cbx_handle* h, const cbx_reml_config* cfg, double* var_u, double* var_e,
                              int32_t* iterations, int32_t* converged, double* solution,
                              cbx_reml_iter_info* history) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create and cbx_mme_set_qinv_* first");
    CBX_REQUIRE(var_u && var_e && *var_u > 0 && *var_e > 0, CBX_ERR_ARG, "variances must be positive");
    CBX_CUDA(cudaSetDevice(h->device));
    const RemlConfigI c = to_cfg(cfg);
    int iters = 0, conv = 0;
    for (int it = 0; it < c.max_iter; ++it) {
      const double ou = *var_u, oe = *var_e;
      IterInfo info;
      reml_iterate(h, c, *var_u, *var_e, info);
      if (history) to_info(info, history + it);
      iters = it + 1;
      const double diff = std::abs(*var_e - oe) + std::abs(*var_u - ou);
      if (diff < c.tol) { conv = 1; break; }
    }
    if (iterations) *iterations = iters;
    if (converged) *converged = conv;
    if (solution && h->mme->has_last)
      CBX_CUDA(cudaMemcpy(solution, h->mme->last_solution.p, h->mme->dim * sizeof(double), cudaMemcpyDeviceToHost));
  });
}

namespace cbx {

// Absolute column sums of a symmetric n x n matrix (= its row sums), one block
// per column: their maximum bounds every |eigenvalue|.
__global__ void k_col_abs_sum(const double* __restrict__ M, int64_t n, double* __restrict__ out) {
  __shared__ double red[256];
  const int64_t c = blockIdx.x;
  double a = 0.0;
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) a += fabs(M[c * n + r]);
  red[threadIdx.x] = a;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = red[0];
}
// A += sum_i w_i u_i u_i^T (U: n x k column-major)
__global__ void k_add_lowrank(double* __restrict__ A, int64_t n, const double* __restrict__ U, const double* __restrict__ w,
                              int k) {
  const int64_t total = n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx % n, c = idx / n;
    double a = 0.0;
    for (int i = 0; i < k; ++i) a += w[i] * U[(int64_t)i * n + r] * U[(int64_t)i * n + c];
    A[idx] += a;
  }
}

// Eigen-bending inverse of a device matrix into out_dev (both n x n, column-major):
// invert_psd_matrix (matrix_io.cpp:488-501) raises every eigenvalue below
// eps = max(1e-12 lambda_max, 1e-6) to eps and returns U diag(1 / lambda) U^T.
// The same matrix is formed without the full eigendecomposition:
//  * lambda_max <= ||M||_inf, so eps = 1e-6 whenever 1e-12 ||M||_inf <= 1e-6;
//  * if M - eps I has a Cholesky factor, no eigenvalue is raised and the result
//    is M^-1 (Cholesky inverse);
//  * otherwise only the eigenpairs below eps are computed (syevdx), M is raised
//    to M + sum (eps - lambda_i) u_i u_i^T, whose eigenvalues are all >= eps,
//    and that is inverted by Cholesky.
//  * when the all-ones direction is (nearly) null -- every VanRaden G, whose
//    centred columns sum to zero -- the one eigenpair below eps is found by
//    inverse iteration instead (deflate_ones below), without syevdx.
// The full eigendecomposition (syevd, scaled columns, GEMM) remains for the
// other cases.  The four forms are the same matrix in exact arithmetic.
static int env_int_reml(const char* name, int def) {
  const char* e = std::getenv(name);
  return (e && *e) ? std::atoi(e) : def;
}

// The one-null-direction path of the eigen-bending inverse (environment
// CBX_DEFLATE_ONES=0 takes the syevdx path instead).
static bool use_deflate_ones() { return env_int_reml("CBX_DEFLATE_ONES", 1) != 0; }

static void invert_psd_full(cbx_handle* h, const double* M_dev, int64_t n, double ridge, double* out_dev) {
  cudaStream_t s = h->stream;
  Libs& L = libs(h);
  DevBuf<double> U, w;
  U.resize((size_t)n * n);
  w.resize(n);
  k_add_ridge_copy<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(M_dev, n, ridge > 0 ? ridge : 0.0, U.p);
  h->launched("k_add_ridge_copy");
  int lw = 0;
  CBX_SOLVER(cusolverDnDsyevd_bufferSize(L.sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)n, U.p,
                                         (int)n, w.p, &lw));
  {
    DevBuf<double> work;
    work.resize(std::max(lw, 1));
    DevBuf<int> info;
    info.resize(1);
    CBX_SOLVER(cusolverDnDsyevd(L.sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)n, U.p, (int)n, w.p,
                                work.p, lw, info.p));
    int hi = 0;
    CBX_CUDA(cudaMemcpyAsync(&hi, info.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    CBX_REQUIRE(hi == 0, CBX_ERR_FACTOR, "symmetric eigensolver failed, info " + std::to_string(hi));
  }
  std::vector<double> wh = d2h(h, w.p, n);
  double maxeig = wh[0];
  for (double v : wh) maxeig = std::max(maxeig, v);
  const double eps = std::max(1e-12 * maxeig, 1e-6);
  for (auto& v : wh) if (v < eps) v = eps;
  CBX_CUDA(cudaMemcpyAsync(w.p, wh.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
  DevBuf<double> V;
  V.resize((size_t)n * n);
  k_scale_cols<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(U.p, w.p, n, V.p);
  h->launched("k_scale_cols");
  const double one = 1.0, zero = 0.0;
  CBX_BLAS(cublasDgemm(L.blas, CUBLAS_OP_N, CUBLAS_OP_T, (int)n, (int)n, (int)n, &one, V.p, (int)n, U.p, (int)n,
                       &zero, out_dev, (int)n));
}

// One eigenvalue of Mr (M + ridge I, in out_dev) below eps, along a direction
// close to v = 1/sqrt(n) (v'Mr v < eps):
//  1. u from eight steps of inverse iteration with the Cholesky factor of
//     Mr + eps I (each step shrinks the other eigenvectors' share by
//     (lambda_1 + eps) / (lambda_i + eps));
//  2. check: Mr + c u u^T - 100 eps I (c = ||Mr||_inf + 1) has a Cholesky factor,
//     so every eigenvalue off u is above 100 eps and u is the only one raised;
//     the gap also bounds u's error after step 1 by (0.1 * 2 / 101)^8;
//  3. Mr + (eps - u'Mr u) u u^T, the raised matrix, inverted by Cholesky.
// Returns false, with out_dev untouched, when step 1 or 2 fails.
static bool deflate_ones(cbx_handle* h, const double* M_dev, int64_t n, double ridge, double eps, double rinf,
                         double* out_dev) {
  cudaStream_t s = h->stream;
  Libs& L = libs(h);
  const int ni = (int)n;
  DevBuf<double> T, u, y, w;
  T.resize((size_t)n * n);
  u.resize(n);
  y.resize(n);
  w.resize(1);
  k_add_ridge_copy<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(out_dev, n, eps, T.p);
  h->launched("k_add_ridge_copy");
  if (!potrf(h, T.p, n)) return false;
  std::vector<double> x(n, 1.0 / std::sqrt((double)n));
  CBX_CUDA(cudaMemcpyAsync(u.p, x.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
  for (int it = 0; it < 8; ++it) {
    potrs(h, T.p, n, u.p, 1);
    double nrm = 0.0;
    CBX_BLAS(cublasDnrm2(L.blas, ni, u.p, 1, &nrm));
    if (!(nrm > 0.0) || !std::isfinite(nrm)) return false;
    const double sc = 1.0 / nrm;
    CBX_BLAS(cublasDscal(L.blas, ni, &sc, u.p, 1));
  }
  const double one = 1.0, zero = 0.0;
  CBX_BLAS(cublasDgemv(L.blas, CUBLAS_OP_N, ni, ni, &one, out_dev, ni, u.p, 1, &zero, y.p, 1));
  double rho = 0.0;
  CBX_BLAS(cublasDdot(L.blas, ni, u.p, 1, y.p, 1, &rho));
  if (!(rho < eps)) return false;
  const double c = rinf + 1.0;
  k_add_ridge_copy<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(out_dev, n, -100.0 * eps, T.p);
  h->launched("k_add_ridge_copy");
  CBX_CUDA(cudaMemcpyAsync(w.p, &c, sizeof(double), cudaMemcpyHostToDevice, s));
  k_add_lowrank<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(T.p, n, u.p, w.p, 1);
  h->launched("k_add_lowrank");
  if (!potrf(h, T.p, n)) return false;
  const double raise = eps - rho;
  CBX_CUDA(cudaMemcpyAsync(w.p, &raise, sizeof(double), cudaMemcpyHostToDevice, s));
  k_add_lowrank<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(out_dev, n, u.p, w.p, 1);
  h->launched("k_add_lowrank");
  if (!chol_inverse_device(h, out_dev, n)) invert_psd_full(h, M_dev, n, ridge, out_dev);
  return true;
}

void invert_psd_device(cbx_handle* h, const double* M_dev, int64_t n, double ridge, double* out_dev) {
  cudaStream_t s = h->stream;
  const double r = ridge > 0 ? ridge : 0.0;
  // M + ridge I into out_dev (the working copy)
  k_add_ridge_copy<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(M_dev, n, r, out_dev);
  h->launched("k_add_ridge_copy");
  double rinf = 0.0;
  {
    DevBuf<double> cs;
    cs.resize(n);
    k_col_abs_sum<<<(unsigned)n, 256, 0, s>>>(out_dev, n, cs.p);
    h->launched("k_col_abs_sum");
    for (double v : d2h(h, cs.p, n)) rinf = std::max(rinf, v);
  }
  if (!(std::isfinite(rinf)) || 1e-12 * rinf > 1e-6) {
    invert_psd_full(h, M_dev, n, ridge, out_dev);
    return;
  }
  const double eps = 1e-6;
  if (n > 1 && use_deflate_ones()) {
    // the all-ones direction nearly null: M - eps I cannot be positive definite
    Libs& L = libs(h);
    const int ni = (int)n;
    DevBuf<double> v, y;
    v.resize(n);
    y.resize(n);
    std::vector<double> vh(n, 1.0 / std::sqrt((double)n));
    CBX_CUDA(cudaMemcpyAsync(v.p, vh.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    const double one = 1.0, zero = 0.0;
    CBX_BLAS(cublasDgemv(L.blas, CUBLAS_OP_N, ni, ni, &one, out_dev, ni, v.p, 1, &zero, y.p, 1));
    double rho0 = 0.0;
    CBX_BLAS(cublasDdot(L.blas, ni, v.p, 1, y.p, 1, &rho0));
    if (rho0 < eps && deflate_ones(h, M_dev, n, ridge, eps, rinf, out_dev)) return;
  }
  DevBuf<double> T;
  T.resize((size_t)n * n);
  // no eigenvalue below eps: M - eps I is positive definite
  k_add_ridge_copy<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(out_dev, n, -eps, T.p);
  h->launched("k_add_ridge_copy");
  if (potrf(h, T.p, n)) {
    if (chol_inverse_device(h, out_dev, n)) return;
    invert_psd_full(h, M_dev, n, ridge, out_dev);
    return;
  }
  // the eigenpairs below eps: lambda in (-||M||_inf - 1, eps)
  Libs& L = libs(h);
  CBX_CUDA(cudaMemcpyAsync(T.p, out_dev, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  DevBuf<double> w;
  w.resize(n);
  const double vl = -rinf - 1.0, vu = std::nextafter(eps, 0.0);
  int meig = 0, lw = 0;
  CBX_SOLVER(cusolverDnDsyevdx_bufferSize(L.sol, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_V,
                                          CUBLAS_FILL_MODE_LOWER, (int)n, T.p, (int)n, vl, vu, 0, 0, &meig, w.p,
                                          &lw));
  {
    DevBuf<double> work;
    work.resize(std::max(lw, 1));
    DevBuf<int> info;
    info.resize(1);
    CBX_SOLVER(cusolverDnDsyevdx(L.sol, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_V, CUBLAS_FILL_MODE_LOWER,
                                 (int)n, T.p, (int)n, vl, vu, 0, 0, &meig, w.p, work.p, lw, info.p));
    int hi = 0;
    CBX_CUDA(cudaMemcpyAsync(&hi, info.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    if (hi != 0 || meig < 0 || meig > n) {
      invert_psd_full(h, M_dev, n, ridge, out_dev);
      return;
    }
  }
  if (meig > 0) {
    std::vector<double> wh = d2h(h, w.p, meig);
    for (auto& v : wh) v = eps - v;
    CBX_CUDA(cudaMemcpyAsync(w.p, wh.data(), meig * sizeof(double), cudaMemcpyHostToDevice, s));
    k_add_lowrank<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, s>>>(out_dev, n, T.p, w.p, meig);
    h->launched("k_add_lowrank");
  }
  if (!chol_inverse_device(h, out_dev, n)) invert_psd_full(h, M_dev, n, ridge, out_dev);
}

// In-place inverse of an SPD device matrix by Cholesky; false if not PD.
bool chol_inverse_device(cbx_handle* h, double* A, int64_t n) {
  if (!potrf(h, A, n)) return false;
  Libs& L = libs(h);
  int lw = 0;
  CBX_SOLVER(cusolverDnDpotri_bufferSize(L.sol, CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n, &lw));
  DevBuf<double> work;
  work.resize(std::max(lw, 1));
  DevBuf<int> info;
  info.resize(1);
  CBX_SOLVER(cusolverDnDpotri(L.sol, CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n, work.p, lw, info.p));
  k_symmetrize_lower<<<gridn(n * n, 256, 8 * h->num_sms), 256, 0, h->stream>>>(A, n);
  h->launched("k_symmetrize_lower");
  return true;
}

}  // namespace cbx

extern "C" int cbx_reml_gradient(cbx_handle* h, double var_u, double var_e, int32_t nprobe, int32_t seed,
                                 int32_t exact_trace, int32_t precision, double pcg_tol, int32_t pcg_maxit,
                                 double* grad, double* trace, int64_t* pcg_iters) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create and cbx_mme_set_qinv_* first");
    CBX_REQUIRE(var_u > 0 && var_e > 0 && grad, CBX_ERR_ARG, "variances must be positive");
    CBX_CUDA(cudaSetDevice(h->device));
    cbx::reml_gradient(h, var_u, var_e, nprobe, seed, exact_trace, precision, pcg_tol, pcg_maxit, grad, trace,
                       pcg_iters);
  });
}

// REML log-likelihood by dense factorization (small problems; dense Qinv).
extern "C" int cbx_reml_logl_dense(cbx_handle* h, double var_u, double var_e, double* logL) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme && logL, CBX_ERR_STATE, "call cbx_mme_create and cbx_mme_set_qinv_dense first");
    CBX_CUDA(cudaSetDevice(h->device));
    const cbx::Mme& m = *h->mme;
    if (m.has_dense && !m.has_sparse && m.ng == m.q) {
      cbx::DenseExact& D = cbx::dense_state(h);
      if (!D.init || D.n != m.n_rec || D.dim != m.dim) cbx::dense_init(h, D);
      cbx::DevBuf<double> C, sol;
      *logL = cbx::dense_logL(h, D, var_u, var_e, C, sol);
    } else {
      // a split Qinv: calc_logL_internal, without the constant log|A|
      CBX_REQUIRE(m.dim <= cbx::kAiDenseMax, CBX_ERR_UNSUPPORTED, "LHS too large for a dense factorization");
      cbx::DevBuf<double> Q, C;
      cbx::dense_qinv(h, Q);
      std::vector<double> sol;
      *logL = cbx::ai_logl(h, Q.p, var_u, var_e, C, sol);
    }
  });
}

// Final MME solve and fixed-effect standard errors (GSSolve::solve,
// src/solve/mixed_model_solver.cpp:37-420): lambda = var_e / var_u (0 when
// var_u <= 1e-9); sol = C^-1 W'y; beta_se_i = sqrt(max(0, var_e (C^-1)_ii)),
// Cinv_beta = (C^-1)[0:p, 0:p] from p unit right-hand sides.
// solver 0: dense Cholesky when the Qinv is dense and dim < 10000 (the
// reference's direct LDLT), else as 1; 1: PCG with relative tolerance;
// 2: PCG with absolute tolerance warm-started from the last REML data solve
// (the matrix-free path of GSSolve, mixed_model_solver.cpp:239-256).
extern "C" int cbx_final_solve(cbx_handle* h, double var_u, double var_e, int32_t solver, double tol,
                               int32_t maxit, int32_t precision, int32_t calc_se, double* sol, double* beta_se,
                               double* Cinv_beta) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create and cbx_mme_set_qinv_* first");
    CBX_REQUIRE(sol && var_e > 0, CBX_ERR_ARG, "bad arguments");
    CBX_CUDA(cudaSetDevice(h->device));
    cbx::Mme& m = *h->mme;
    cudaStream_t s = h->stream;
    const int64_t p = m.p, dim = m.dim;
    const double lam = var_u > 1e-9 ? var_e / var_u : 0.0;
    const bool dense = solver == 0 && m.has_dense && !m.has_sparse && dim < 10000;
    cbx::DevBuf<double> x;
    x.resize(dim);
    std::vector<double> Ci((size_t)p * p, 0.0);
    if (dense) {
      cbx::DevBuf<double> C;
      CBX_REQUIRE(cbx::factor_lhs(h, lam, C), CBX_ERR_FACTOR, "Direct Solver Decomposition Failed");
      CBX_CUDA(cudaMemcpyAsync(x.p, m.rhs.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
      cbx::potrs(h, C.p, dim, x.p, 1);
      if (calc_se && p > 0) {
        std::vector<double> E((size_t)dim * p, 0.0);
        for (int64_t i = 0; i < p; ++i) E[(size_t)i * dim + i] = 1.0;
        cbx::DevBuf<double> Ed;
        Ed.resize(E.size());
        CBX_CUDA(cudaMemcpyAsync(Ed.p, E.data(), E.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        cbx::potrs(h, C.p, dim, Ed.p, p);
        std::vector<double> Eh = cbx::d2h(h, Ed.p, E.size());
        for (int64_t i = 0; i < p; ++i)
          for (int64_t j = 0; j < p; ++j) Ci[(size_t)i * p + j] = Eh[(size_t)i * dim + j];
      }
    } else {
      const bool abs_mode = solver == 2;
      const bool warm = abs_mode && m.has_last;
      if (warm) CBX_CUDA(cudaMemcpyAsync(x.p, m.last_solution.p, dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
      cbx::PcgResult r;
      cbx::pcg_solve(h, lam, 1, m.rhs.p, x.p, warm, tol, maxit, abs_mode ? 1 : 0, precision, r);
      if (r.status[0] == cbx::sv::COL_NONFINITE) throw cbx::Error(CBX_ERR_NONFINITE, "non-finite final solve");
      if (calc_se && p > 0) {
        std::vector<double> E((size_t)dim * p, 0.0);
        for (int64_t i = 0; i < p; ++i) E[(size_t)i * dim + i] = 1.0;
        cbx::DevBuf<double> Ed, Xd;
        Ed.resize(E.size());
        Xd.resize(E.size());
        CBX_CUDA(cudaMemcpyAsync(Ed.p, E.data(), E.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        cbx::PcgResult re;
        cbx::pcg_solve(h, lam, (int)p, Ed.p, Xd.p, false, tol, maxit, abs_mode ? 1 : 0, precision, re);
        std::vector<double> Xh = cbx::d2h(h, Xd.p, E.size());
        for (int64_t i = 0; i < p; ++i)
          for (int64_t j = 0; j < p; ++j) Ci[(size_t)i * p + j] = Xh[(size_t)i * dim + j];
      }
    }
    CBX_CUDA(cudaMemcpyAsync(sol, x.p, dim * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    if (calc_se) {
      for (int64_t i = 0; i < p; ++i) {
        if (beta_se) beta_se[i] = std::sqrt(std::max(0.0, var_e * Ci[(size_t)i * p + i]));
        if (Cinv_beta)
          for (int64_t j = 0; j < p; ++j) Cinv_beta[(size_t)i * p + j] = Ci[(size_t)i * p + j];
      }
    }
  });
}

// Eigen-bending inverse of M (n x n); M == NULL uses the device GRM of this
// handle.  The result stays on the device (cbx_mme_set_qinv_dense(h, NULL, n))
// and is copied to Minv when given.
extern "C" int cbx_invert_psd(cbx_handle* h, const double* M, int64_t n, double ridge, double* Minv) {
  return cbx_guard(h, [&] {
    CBX_CUDA(cudaSetDevice(h->device));
    CBX_REQUIRE(n > 0, CBX_ERR_ARG, "n must be positive");
    cudaStream_t s = h->stream;
    DevBuf<double> src;
    const double* sp = nullptr;
    if (M) {
      src.resize((size_t)n * n);
      CBX_CUDA(cudaMemcpyAsync(src.p, M, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice, s));
      sp = src.p;
    } else {
      CBX_REQUIRE(h->G.p && h->G_n == n, CBX_ERR_STATE, "no device GRM of this order (cbx_grm_bed)");
      sp = h->G.p;
    }
    h->Ginv.resize((size_t)n * n);
    ++h->Ginv_gen;
    invert_psd_device(h, sp, n, ridge, h->Ginv.p);
    h->Ginv_n = n;
    if (Minv) CBX_CUDA(cudaMemcpyAsync(Minv, h->Ginv.p, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
  });
}
