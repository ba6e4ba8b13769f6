// Multi-trait GBLUP on the device: the exact eigen-EM variance estimation and
// the multi-trait MME solve.
//
// Replaces:
//  * MvEigenVce::prepare / updateEM / runNullModel (src/core/eigen_vce.cpp:106-266)
//    as GSVce::run calls it for multi-trait runs
//    (src/variance/variance_estimator.cpp:86-325: projection on, max_iter =
//    max(500, 25 vce_max_iter), tol = vce_tol).  Y and G are projected onto
//    the null space of X' (Householder QR of X applied with ormqr, never
//    forming Q), the projected G is eigen-decomposed (negative eigenvalues set
//    to 0) and the whole EM loop runs in one persistent kernel;
//  * GSSolve::solveMultiTrait (src/solve/mixed_model_solver.cpp:425-524): the
//    explicit Kronecker-product LHS, built on the device in trait-major order,
//    solved by dense Cholesky.
//
// EM update used by the kernel.  With V_i = d_i Vg + Ve, P_i = V_i^-1 and
// q_i = P_i r_i, the reference's per-sample terms sum to
//   Vg_new = Vg + Vg [sum_{d_i > 1e-12} d_i (q_i q_i' - P_i)] Vg / n
//   Ve_new = Ve + Ve [sum_i (q_i q_i' - P_i)] Ve / n,
// because u_hat u_hat' / d_i + Vg - W_g Vg = Vg + d_i Vg (q q' - P) Vg and
// e_hat e_hat' + Ve - W_e Ve = Ve + Ve (q q' - P) Ve.  The two bracketed
// symmetric sums are all a thread accumulates; the block reduces them in a
// fixed order, so the result does not depend on scheduling.
#include <cmath>
#include <vector>
#include "dense.h"
#include "handle.h"

namespace cbx {
namespace mt {

constexpr int EM_NT = 512;
constexpr int kMaxTraits = 8;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Column means and covariance of Y (n x t, column-major) with divisor `div`;
// one block, fixed summation order.  VgVe[0..t*t) = VgVe[t*t..2t*t) = cov / 2.
__global__ void k_half_cov(const double* __restrict__ Y, int64_t n, int t, double div, double* __restrict__ VgVe) {
  __shared__ double red[32];
  __shared__ double mean[kMaxTraits];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int a = 0; a < t; ++a) {
    double s = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += Y[a * n + i];
    s = warp_sum(s);
    if (lane == 0) red[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0;
      for (int w = 0; w < nw; ++w) tot += red[w];
      mean[a] = tot / (double)n;
    }
    __syncthreads();
  }
  for (int a = 0; a < t; ++a)
    for (int b = a; b < t; ++b) {
      double s = 0;
      for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += (Y[a * n + i] - mean[a]) * (Y[b * n + i] - mean[b]);
      s = warp_sum(s);
      if (lane == 0) red[warp] = s;
      __syncthreads();
      if (threadIdx.x == 0) {
        double tot = 0;
        for (int w = 0; w < nw; ++w) tot += red[w];
        const double c = 0.5 * tot / div;
        VgVe[a * t + b] = VgVe[b * t + a] = c;
        VgVe[t * t + a * t + b] = VgVe[t * t + b * t + a] = c;
      }
      __syncthreads();
    }
}

// In-register inverse of an SPD T x T matrix by Cholesky; false if not PD.
template <int T>
__device__ __forceinline__ bool spd_inverse(const double (&V)[T][T], double (&P)[T][T]) {
  double L[T][T];
#pragma unroll
  for (int j = 0; j < T; ++j) {
    double d = V[j][j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= L[j][k] * L[j][k];
    if (!(d > 0.0)) return false;
    const double ljj = sqrt(d);
    L[j][j] = ljj;
#pragma unroll
    for (int i = j + 1; i < T; ++i) {
      double s = V[i][j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= L[i][k] * L[j][k];
      L[i][j] = s / ljj;
    }
  }
  // Linv (lower), then P = Linv' Linv
  double Li[T][T];
#pragma unroll
  for (int j = 0; j < T; ++j) {
#pragma unroll
    for (int i = 0; i < T; ++i) Li[i][j] = 0.0;
    Li[j][j] = 1.0 / L[j][j];
#pragma unroll
    for (int i = j + 1; i < T; ++i) {
      double s = 0;
#pragma unroll
      for (int k = j; k < i; ++k) s -= L[i][k] * Li[k][j];
      Li[i][j] = s / L[i][i];
    }
  }
#pragma unroll
  for (int a = 0; a < T; ++a)
#pragma unroll
    for (int b = a; b < T; ++b) {
      double s = 0;
#pragma unroll
      for (int k = (a > b ? a : b); k < T; ++k) s += Li[k][a] * Li[k][b];
      P[a][b] = s;
      P[b][a] = s;
    }
  return true;
}

// The whole MvEigenVce EM loop (runNullModel) in one block.  D: eigenvalues
// (clamped at 0 here), R: rotated responses (n x T, column-major).  VgVe holds
// the start values and receives the result; info = {iterations, converged,
// status (0 ok, 1 V_i not positive definite)}.
template <int T>
__global__ void __launch_bounds__(EM_NT) k_mv_em(const double* __restrict__ D, const double* __restrict__ R, int64_t n,
                                                 int max_iter, double tol, double* __restrict__ VgVe,
                                                 int* __restrict__ info) {
  constexpr int NS = T * (T + 1) / 2;  // packed upper triangle
  constexpr int K = 2 * NS;
  __shared__ double Vg[T][T], Ve[T][T];
  __shared__ double part[EM_NT / 32][K];
  __shared__ double tot[K];
  __shared__ int done, bad;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < T * T) {
    Vg[threadIdx.x / T][threadIdx.x % T] = VgVe[threadIdx.x];
    Ve[threadIdx.x / T][threadIdx.x % T] = VgVe[T * T + threadIdx.x];
  }
  if (threadIdx.x == 0) { done = 0; bad = 0; }
  __syncthreads();
  int it = 0;
  for (; it < max_iter && !done && !bad; ++it) {
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += EM_NT) {
      const double d = D[i] > 0.0 ? D[i] : 0.0;
      double V[T][T], P[T][T], r[T], q[T];
#pragma unroll
      for (int a = 0; a < T; ++a) {
        r[a] = R[a * n + i];
#pragma unroll
        for (int b = 0; b < T; ++b) V[a][b] = Vg[a][b] * d + Ve[a][b];
      }
      if (!spd_inverse<T>(V, P)) { atomicExch(&bad, 1); continue; }
#pragma unroll
      for (int a = 0; a < T; ++a) {
        double s = 0;
#pragma unroll
        for (int b = 0; b < T; ++b) s += P[a][b] * r[b];
        q[a] = s;
      }
      const bool big = d > 1e-12;
      int k = 0;
#pragma unroll
      for (int a = 0; a < T; ++a)
#pragma unroll
        for (int b = a; b < T; ++b, ++k) {
          const double m = q[a] * q[b] - P[a][b];
          acc[NS + k] += m;
          if (big) acc[k] += d * m;
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const double v = warp_sum(acc[k]);
      if (lane == 0) part[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < K) {
      double s = 0;
      for (int w = 0; w < EM_NT / 32; ++w) s += part[w][threadIdx.x];
      tot[threadIdx.x] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0 && !bad) {
      double Ag[T][T], Ae[T][T];
      int k = 0;
      for (int a = 0; a < T; ++a)
        for (int b = a; b < T; ++b, ++k) {
          Ag[a][b] = Ag[b][a] = tot[k];
          Ae[a][b] = Ae[b][a] = tot[NS + k];
        }
      double Ng[T][T], Ne[T][T], ng = 0, ne = 0, dg = 0, de = 0;
      const double inv_n = 1.0 / (double)n;
      for (int a = 0; a < T; ++a)
        for (int b = a; b < T; ++b) {
          double sg = 0, se = 0;
          for (int c = 0; c < T; ++c) {
            double tg = 0, te = 0;
            for (int e = 0; e < T; ++e) {
              tg += Ag[c][e] * Vg[e][b];
              te += Ae[c][e] * Ve[e][b];
            }
            sg += Vg[a][c] * tg;
            se += Ve[a][c] * te;
          }
          Ng[a][b] = Ng[b][a] = Vg[a][b] + sg * inv_n;
          Ne[a][b] = Ne[b][a] = Ve[a][b] + se * inv_n;
        }
      for (int a = 0; a < T; ++a)
        for (int b = 0; b < T; ++b) {
          ng += Vg[a][b] * Vg[a][b];
          ne += Ve[a][b] * Ve[a][b];
          dg += (Ng[a][b] - Vg[a][b]) * (Ng[a][b] - Vg[a][b]);
          de += (Ne[a][b] - Ve[a][b]) * (Ne[a][b] - Ve[a][b]);
        }
      const double rg = sqrt(dg) / fmax(sqrt(ng), 1e-12), re = sqrt(de) / fmax(sqrt(ne), 1e-12);
      for (int a = 0; a < T; ++a)
        for (int b = 0; b < T; ++b) {
          Vg[a][b] = Ng[a][b];
          Ve[a][b] = Ne[a][b];
        }
      if (rg < tol && re < tol) done = 1;
    }
    __syncthreads();
  }
  if (threadIdx.x < T * T) {
    VgVe[threadIdx.x] = Vg[threadIdx.x / T][threadIdx.x % T];
    VgVe[T * T + threadIdx.x] = Ve[threadIdx.x / T][threadIdx.x % T];
  }
  if (threadIdx.x == 0) {
    info[0] = it;
    info[1] = done;
    info[2] = bad;
  }
}

// dst (rows x cols, ld rows) = src[r0 + i, c0 + j] (src column-major, ld lds)
__global__ void k_copy_block(const double* __restrict__ src, int64_t lds, int64_t r0, int64_t c0, int64_t rows,
                             int64_t cols, double* __restrict__ dst) {
  const int64_t total = rows * cols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    dst[idx] = src[(c0 + j) * lds + r0 + i];
  }
}

// The multi-trait LHS (dim = (p + n) t, column-major, trait-major unknowns):
//   [ Vei (x) X'X   Vei (x) X'              ]
//   [ Vei (x) X     Vei (x) I + Vgi (x) Ginv ]
// VV = {Vei (t x t), Vgi (t x t)} row-major.
__global__ void k_mt_lhs(int64_t n, int t, int64_t p, const double* __restrict__ XtX, const double* __restrict__ X,
                         const double* __restrict__ Ginv, int64_t ldg, const double* __restrict__ VV,
                         double* __restrict__ L) {
  const int64_t pt = p * t, dim = (p + n) * t;
  const int64_t total = dim * dim;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx % dim, c = idx / dim;
    double v;
    if (r < pt && c < pt) {
      const int a = (int)(r / p), b = (int)(c / p);
      v = VV[a * t + b] * XtX[(c % p) * p + (r % p)];
    } else if (r < pt) {  // top-right: Vei(a,b) X'(row effect, column animal)
      const int a = (int)(r / p), b = (int)((c - pt) / n);
      v = VV[a * t + b] * X[(r % p) * n + (c - pt) % n];
    } else if (c < pt) {  // bottom-left
      const int a = (int)((r - pt) / n), b = (int)(c / p);
      v = VV[a * t + b] * X[(c % p) * n + (r - pt) % n];
    } else {
      const int a = (int)((r - pt) / n), b = (int)((c - pt) / n);
      const int64_t i = (r - pt) % n, j = (c - pt) % n;
      v = VV[t * t + a * t + b] * Ginv[j * ldg + i] + (i == j ? VV[a * t + b] : 0.0);
    }
    L[idx] = v;
  }
}

// rhs2 (n x t) = Y Vei', written at rhs + p t (trait-major)
__global__ void k_mt_rhs2(const double* __restrict__ Y, int64_t n, int t, const double* __restrict__ VV,
                          double* __restrict__ rhs2) {
  const int64_t total = n * t;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % n;
    const int a = (int)(idx / n);
    double s = 0;
    for (int b = 0; b < t; ++b) s += Y[b * n + i] * VV[a * t + b];
    rhs2[idx] = s;
  }
}

static void host_inverse(int t, const double* A, double* Ai) {
  // Gauss-Jordan with partial pivoting on a t x t (row-major) matrix
  std::vector<double> M(A, A + t * t), I(t * t, 0.0);
  for (int i = 0; i < t; ++i) I[i * t + i] = 1.0;
  for (int c = 0; c < t; ++c) {
    int piv = c;
    for (int r = c + 1; r < t; ++r)
      if (std::abs(M[r * t + c]) > std::abs(M[piv * t + c])) piv = r;
    CBX_REQUIRE(M[piv * t + c] != 0.0, CBX_ERR_FACTOR, "variance matrix is singular");
    if (piv != c)
      for (int k = 0; k < t; ++k) {
        std::swap(M[c * t + k], M[piv * t + k]);
        std::swap(I[c * t + k], I[piv * t + k]);
      }
    const double d = M[c * t + c];
    for (int k = 0; k < t; ++k) {
      M[c * t + k] /= d;
      I[c * t + k] /= d;
    }
    for (int r = 0; r < t; ++r)
      if (r != c) {
        const double f = M[r * t + c];
        if (f != 0.0)
          for (int k = 0; k < t; ++k) {
            M[r * t + k] -= f * M[c * t + k];
            I[r * t + k] -= f * I[c * t + k];
          }
      }
  }
  std::copy(I.begin(), I.end(), Ai);
}

// G from the handle's device G^-1 (the reference recovers G by an LDLT solve
// of G^-1 against I), or uploaded from the host.
static void load_g(cbx_handle* h, const double* G, int64_t n, DevBuf<double>& Gd) {
  cudaStream_t s = h->stream;
  Gd.resize((size_t)n * n);
  if (G) {
    CBX_CUDA(cudaMemcpyAsync(Gd.p, G, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice, s));
    return;
  }
  CBX_REQUIRE(h->Ginv.p && h->Ginv_n == n, CBX_ERR_STATE, "no device G^-1 of order n (cbx_invert_psd)");
  CBX_CUDA(cudaMemcpyAsync(Gd.p, h->Ginv.p, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CBX_REQUIRE(chol_inverse_device(h, Gd.p, n), CBX_ERR_FACTOR,
              "G^-1 is not positive-definite; cannot recover G");
}

template <int T>
static void launch_em(cbx_handle* h, const double* D, const double* R, int64_t n, int max_iter, double tol,
                      double* VgVe, int* info) {
  k_mv_em<T><<<1, EM_NT, 0, h->stream>>>(D, R, n, max_iter, tol, VgVe, info);
  h->launched("k_mv_em");
}

}  // namespace mt
}  // namespace cbx

using namespace cbx;

extern "C" int cbx_mt_vce(cbx_handle* h, int64_t n, int32_t t, int64_t p, const double* Y, const double* X,
                          const double* G, int32_t max_iter, double tol, double* Vg, double* Ve,
                          int32_t* iterations, int32_t* converged) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(n > 1 && t >= 1 && t <= mt::kMaxTraits && p >= 0 && p < n - 1 && Y && (p == 0 || X),
                CBX_ERR_ARG, "bad multi-trait dimensions (1 <= t <= 8, 0 <= p < n - 1)");
    CBX_REQUIRE(n <= 46000, CBX_ERR_ARG, "multi-trait eigen-EM is limited to n <= 46,000");
    CBX_REQUIRE(max_iter > 0 && Vg && Ve, CBX_ERR_ARG, "bad arguments");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    Libs& L = libs(h);
    const int64_t ne = n - p;  // samples after projection
    DevBuf<double> Gd, Yd, VgVe;
    DevBuf<int> info;
    mt::load_g(h, G, n, Gd);
    Yd.resize((size_t)n * t);
    CBX_CUDA(cudaMemcpyAsync(Yd.p, Y, (size_t)n * t * sizeof(double), cudaMemcpyHostToDevice, s));
    VgVe.resize(2 * t * t);
    info.resize(3);
    // start values from the unprojected Y (the divisor already uses n - p)
    mt::k_half_cov<<<1, 256, 0, s>>>(Yd.p, n, t, (double)(ne - 1), VgVe.p);
    h->launched("k_half_cov");
    DevBuf<double> Gr, Yr;
    if (p > 0) {
      // Householder QR of X; Q' G Q and Q' Y by ormqr (Q.rightCols(n - p) is the null space of X')
      DevBuf<double> Xd, tau, work;
      DevBuf<int> dinfo;
      Xd.resize((size_t)n * p);
      tau.resize(p);
      dinfo.resize(1);
      CBX_CUDA(cudaMemcpyAsync(Xd.p, X, (size_t)n * p * sizeof(double), cudaMemcpyHostToDevice, s));
      int lw = 0, lw2 = 0, lw3 = 0;
      CBX_SOLVER(cusolverDnDgeqrf_bufferSize(L.sol, (int)n, (int)p, Xd.p, (int)n, &lw));
      CBX_SOLVER(cusolverDnDormqr_bufferSize(L.sol, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, (int)n, (int)n, (int)p, Xd.p,
                                             (int)n, tau.p, Gd.p, (int)n, &lw2));
      CBX_SOLVER(cusolverDnDormqr_bufferSize(L.sol, CUBLAS_SIDE_RIGHT, CUBLAS_OP_N, (int)n, (int)n, (int)p, Xd.p,
                                             (int)n, tau.p, Gd.p, (int)n, &lw3));
      work.resize(std::max({lw, lw2, lw3, 1}));
      const int lwork = (int)std::max({lw, lw2, lw3, 1});
      CBX_SOLVER(cusolverDnDgeqrf(L.sol, (int)n, (int)p, Xd.p, (int)n, tau.p, work.p, lwork, dinfo.p));
      CBX_SOLVER(cusolverDnDormqr(L.sol, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, (int)n, (int)n, (int)p, Xd.p, (int)n, tau.p,
                                  Gd.p, (int)n, work.p, lwork, dinfo.p));
      CBX_SOLVER(cusolverDnDormqr(L.sol, CUBLAS_SIDE_RIGHT, CUBLAS_OP_N, (int)n, (int)n, (int)p, Xd.p, (int)n, tau.p,
                                  Gd.p, (int)n, work.p, lwork, dinfo.p));
      int lw4 = 0;
      CBX_SOLVER(cusolverDnDormqr_bufferSize(L.sol, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, (int)n, t, (int)p, Xd.p, (int)n,
                                             tau.p, Yd.p, (int)n, &lw4));
      DevBuf<double> Yq, work2;
      Yq.resize((size_t)n * t);
      CBX_CUDA(cudaMemcpyAsync(Yq.p, Yd.p, (size_t)n * t * sizeof(double), cudaMemcpyDeviceToDevice, s));
      work2.resize(std::max(lw4, 1));
      CBX_SOLVER(cusolverDnDormqr(L.sol, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, (int)n, t, (int)p, Xd.p, (int)n, tau.p, Yq.p,
                                  (int)n, work2.p, std::max(lw4, 1), dinfo.p));
      int hi = 0;
      CBX_CUDA(cudaMemcpyAsync(&hi, dinfo.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      CBX_CUDA(cudaStreamSynchronize(s));
      CBX_REQUIRE(hi == 0, CBX_ERR_FACTOR, "QR of the fixed-effect design failed");
      Gr.resize((size_t)ne * ne);
      Yr.resize((size_t)ne * t);
      mt::k_copy_block<<<gridn(ne * ne, 256, 8 * h->num_sms), 256, 0, s>>>(Gd.p, n, p, p, ne, ne, Gr.p);
      h->launched("k_copy_block");
      mt::k_copy_block<<<gridn(ne * t, 256, 2 * h->num_sms), 256, 0, s>>>(Yq.p, n, p, 0, ne, t, Yr.p);
      h->launched("k_copy_block");
      Gd.release();
    } else {
      Gr = std::move(Gd);
      Yr = std::move(Yd);
    }
    // eigen-decomposition of the projected G (ascending, as Eigen's solver)
    DevBuf<double> w;
    w.resize(ne);
    {
      int lw = 0;
      CBX_SOLVER(cusolverDnDsyevd_bufferSize(L.sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)ne, Gr.p,
                                             (int)ne, w.p, &lw));
      DevBuf<double> work;
      work.resize(std::max(lw, 1));
      DevBuf<int> dinfo;
      dinfo.resize(1);
      CBX_SOLVER(cusolverDnDsyevd(L.sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)ne, Gr.p, (int)ne,
                                  w.p, work.p, lw, dinfo.p));
      int hi = 0;
      CBX_CUDA(cudaMemcpyAsync(&hi, dinfo.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      CBX_CUDA(cudaStreamSynchronize(s));
      CBX_REQUIRE(hi == 0, CBX_ERR_FACTOR, "symmetric eigensolver failed, info " + std::to_string(hi));
    }
    // rotated responses U' Yr
    DevBuf<double> R;
    R.resize((size_t)ne * t);
    const double one = 1.0, zero = 0.0;
    CBX_BLAS(cublasDgemm(L.blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)ne, t, (int)ne, &one, Gr.p, (int)ne, Yr.p, (int)ne,
                         &zero, R.p, (int)ne));
    Gr.release();
    switch (t) {
      case 1: mt::launch_em<1>(h, w.p, R.p, ne, max_iter, tol, VgVe.p, info.p); break;
      case 2: mt::launch_em<2>(h, w.p, R.p, ne, max_iter, tol, VgVe.p, info.p); break;
      case 3: mt::launch_em<3>(h, w.p, R.p, ne, max_iter, tol, VgVe.p, info.p); break;
      case 4: mt::launch_em<4>(h, w.p, R.p, ne, max_iter, tol, VgVe.p, info.p); break;
      case 5: mt::launch_em<5>(h, w.p, R.p, ne, max_iter, tol, VgVe.p, info.p); break;
      case 6: mt::launch_em<6>(h, w.p, R.p, ne, max_iter, tol, VgVe.p, info.p); break;
      case 7: mt::launch_em<7>(h, w.p, R.p, ne, max_iter, tol, VgVe.p, info.p); break;
      default: mt::launch_em<8>(h, w.p, R.p, ne, max_iter, tol, VgVe.p, info.p); break;
    }
    CBX_CUDA(cudaGetLastError());
    const auto vv = d2h(h, VgVe.p, 2 * t * t);
    const auto inf = d2h(h, info.p, 3);
    CBX_REQUIRE(inf[2] == 0, CBX_ERR_FACTOR, "MvEigenVce::updateEM: V_i is not positive-definite");
    std::copy(vv.begin(), vv.begin() + t * t, Vg);
    std::copy(vv.begin() + t * t, vv.end(), Ve);
    if (iterations) *iterations = inf[0];
    if (converged) *converged = inf[1];
  });
}

extern "C" int cbx_mt_solve(cbx_handle* h, int64_t n, int32_t t, int64_t p, const double* Y, const double* X,
                            const double* Ginv, const double* Vg, const double* Ve, double* beta, double* u) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(n > 0 && t >= 1 && t <= mt::kMaxTraits && p >= 0 && Y && (p == 0 || X) && Vg && Ve && u,
                CBX_ERR_ARG, "bad multi-trait arguments");
    const int64_t dim = (p + n) * t;
    CBX_REQUIRE(dim <= 46000, CBX_ERR_ARG, "dense multi-trait MME is limited to (n + p) t <= 46,000");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    Libs& L = libs(h);
    std::vector<double> VV(2 * t * t);
    mt::host_inverse(t, Ve, VV.data());
    mt::host_inverse(t, Vg, VV.data() + t * t);
    DevBuf<double> vv, Yd, Xd, XtX, Gi, C, rhs;
    vv.resize(VV.size());
    CBX_CUDA(cudaMemcpyAsync(vv.p, VV.data(), VV.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    Yd.resize((size_t)n * t);
    CBX_CUDA(cudaMemcpyAsync(Yd.p, Y, (size_t)n * t * sizeof(double), cudaMemcpyHostToDevice, s));
    Xd.resize((size_t)std::max<int64_t>(1, n * p));
    XtX.resize((size_t)std::max<int64_t>(1, p * p));
    const double one = 1.0, zero = 0.0;
    if (p > 0) {
      CBX_CUDA(cudaMemcpyAsync(Xd.p, X, (size_t)n * p * sizeof(double), cudaMemcpyHostToDevice, s));
      CBX_BLAS(cublasDgemm(L.blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)p, (int)p, (int)n, &one, Xd.p, (int)n, Xd.p, (int)n,
                           &zero, XtX.p, (int)p));
    }
    const double* gi = nullptr;
    if (Ginv) {
      Gi.resize((size_t)n * n);
      CBX_CUDA(cudaMemcpyAsync(Gi.p, Ginv, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice, s));
      gi = Gi.p;
    } else {
      CBX_REQUIRE(h->Ginv.p && h->Ginv_n == n, CBX_ERR_STATE, "no device G^-1 of order n (cbx_invert_psd)");
      gi = h->Ginv.p;
    }
    C.resize((size_t)dim * dim);
    mt::k_mt_lhs<<<gridn(dim * dim, 256, 16 * h->num_sms), 256, 0, s>>>(n, t, p, XtX.p, Xd.p, gi, n, vv.p, C.p);
    h->launched("k_mt_lhs");
    Gi.release();
    rhs.resize(dim);
    mt::k_mt_rhs2<<<gridn(n * t, 256, 4 * h->num_sms), 256, 0, s>>>(Yd.p, n, t, vv.p, rhs.p + p * t);
    h->launched("k_mt_rhs2");
    if (p > 0)  // rhs1 (p x t) = X' rhs2
      CBX_BLAS(cublasDgemm(L.blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)p, t, (int)n, &one, Xd.p, (int)n, rhs.p + p * t,
                           (int)n, &zero, rhs.p, (int)p));
    CBX_REQUIRE(potrf(h, C.p, dim), CBX_ERR_FACTOR, "Multi-trait MME factorization failed.");
    potrs(h, C.p, dim, rhs.p, 1);
    if (beta && p > 0)
      CBX_CUDA(cudaMemcpyAsync(beta, rhs.p, (size_t)p * t * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaMemcpyAsync(u, rhs.p + p * t, (size_t)n * t * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
  });
}
