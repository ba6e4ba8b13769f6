// Mixed-model equations on the device and the multi-RHS PCG solver.
//
// Replaces, for one random component:
//  * MMELHSBuilder::initialize / build_lhs / build_rhs
//    (src/core/mme_builder.cpp:72-387): W'W and W'y are assembled on the host
//    in the reference's record order and uploaded once; lambda Qinv is applied
//    on the fly instead of being copied into the CSR;
//  * DenseMatrixAdapter / SplitMatrixAdapter products
//    (src/core/matrix_adapter.h:116-153, 232-373);
//  * PCGSolver::solve with the block-Jacobi preconditioner
//    (src/core/pcg_solver.h:60-128, 436-536) and MatrixFreePCG's absolute stop
//    (src/core/matrix_free_pcg.h:20-66).
#include <algorithm>
#include <cstdio>
#include <cmath>
#include <exception>
#include <thread>
#include <vector>
#include "handle.h"
#include "pcg.h"
#include "tune.h"
#include "solver.cuh"
#include "pcg_fused.cuh"
#include "dense_tc.h"
#include "dense.h"
#include <cstdlib>

namespace cbx {
namespace sv {

__global__ void k_resid_records(int64_t n_rec, int64_t p, const double* __restrict__ y,
                                const int32_t* __restrict__ aid, int64_t q,
                                const int32_t* __restrict__ xp, const int32_t* __restrict__ xc,
                                const double* __restrict__ xv, const double* __restrict__ sol,
                                double* __restrict__ e, double* __restrict__ part) {
  __shared__ double red[NT];
  double acc = 0;
  for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n_rec; i += (int64_t)gridDim.x * NT) {
    double t = 0.0;
    for (int32_t j = xp[i]; j < xp[i + 1]; ++j)
      if (xc[j] < p) t += xv[j] * sol[xc[j]];
    const int32_t a = aid[i];
    if (a > 0 && a <= q) t += sol[p + a - 1];
    const double ev = y[i] - t;
    if (e) e[i] = ev;
    acc += ev * ev;
  }
  const double s = block_sum_cols<1>(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

}  // namespace sv

// ---------------------------------------------------------------------------
// helper kernels
template <typename A, typename B>
__global__ void k_convert(const A* __restrict__ a, B* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = static_cast<B>(a[i]);
}

// dst[i * ld + k] = src[i * n + k] (k < n), 0 in the padding
template <typename T>
__global__ void k_pitch_copy(const double* __restrict__ src, int64_t n, int64_t ld, T* __restrict__ dst) {
  const int64_t total = n * ld;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / ld, k = idx - i * ld;
    dst[idx] = k < n ? static_cast<T>(src[i * n + k]) : T(0);
  }
}

// Low-precision copies of an n x n block (row-major, pitch n) minus a constant:
// hi[i * ld + k] = fl32(src - shift), lo = fl32(src - shift - hi) for k < n;
// padding columns are zero.
__global__ void k_lowp_block(const double* __restrict__ src, int64_t n, int64_t ld, double shift,
                             float* __restrict__ hi, float* __restrict__ lo) {
  const int64_t total = n * ld;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / ld, k = idx - i * ld;
    float h = 0.0f, l = 0.0f;
    if (k < n) {
      const double v = src[i * n + k] - shift;
      h = __double2float_rn(v);
      l = __double2float_rn(v - (double)h);
    }
    hi[idx] = h;
    lo[idx] = l;
  }
}

// Per-block partial sums of the off-diagonal entries of an n x n block.
__global__ void k_offdiag_part(const double* __restrict__ src, int64_t n, double* __restrict__ part) {
  __shared__ double red[256];
  double acc = 0.0;
  const int64_t total = n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x)
    if (idx / n != idx % n) acc += src[idx];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// column-major (dim x ncols) -> interleaved (dim x S), zero in unused columns
__global__ void k_to_inter(const double* __restrict__ cm, int64_t dim, int ncols, int S,
                           double* __restrict__ it) {
  const int64_t total = dim * S;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / S;
    const int c = (int)(idx - i * S);
    it[idx] = c < ncols ? cm[(int64_t)c * dim + i] : 0.0;
  }
}
__global__ void k_from_inter(const double* __restrict__ it, int64_t dim, int ncols, int S,
                             double* __restrict__ cm) {
  const int64_t total = dim * ncols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / dim, i = idx - c * dim;
    cm[idx] = it[i * S + c];
  }
}

template <typename T>
__global__ void k_dinv(const double* __restrict__ diagD, const double* __restrict__ diagQ, int64_t p,
                       int64_t q, double lam, T* __restrict__ dinv) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < q; u += (int64_t)gridDim.x * blockDim.x) {
    const double d = diagD[p + u] + lam * diagQ[u];
    dinv[u] = static_cast<T>(fabs(d) > 1e-12 ? 1.0 / d : 1.0);
  }
}

// r32 = (float)(r64 / s_c) for columns with s_c > 0, else 0
__global__ void k_scale_down(const double* __restrict__ r64, const double* __restrict__ sc, int64_t dim,
                             int S, float* __restrict__ r32) {
  const int64_t total = dim * S;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(idx % S);
    r32[idx] = sc[c] > 0 ? (float)(r64[idx] / sc[c]) : 0.0f;
  }
}
// Dc = s_c * (d32 + d32lo) (0 for columns with s_c = 0; d32lo may be null); x64 += Dc
__global__ void k_correction(double* __restrict__ x64, const float* __restrict__ d32,
                             const float* __restrict__ d32lo, const double* __restrict__ sc, int64_t dim, int S,
                             double* __restrict__ dc) {
  const int64_t total = dim * S;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(idx % S);
    const double dv = d32lo ? (double)d32[idx] + (double)d32lo[idx] : (double)d32[idx];
    const double d = sc[c] > 0 ? sc[c] * dv : 0.0;
    dc[idx] = d;
    x64[idx] += d;
  }
}
// Residual carried to a new lambda.  With r' = b - A(lam') x for lam' = lam -
// dlam, A(lam') x = W'W x + lam' [0; Qinv x_u] gives lam' [0; Qinv x_u] =
// b - r' - W'W x, so b - A(lam) x = r' - (dlam / lam') (b - r' - W'W x) on
// the random rows and r' on the fixed rows: only the sparse W'W is applied.
// Interleaved blocks (row i, column c at i * S + c); f = dlam / lam'.
__global__ void k_carry_resid(const int32_t* __restrict__ Dptr, const int32_t* __restrict__ Dcol,
                              const double* __restrict__ Dval, int64_t p, int64_t dim, int S,
                              const double* __restrict__ B, const double* __restrict__ X, double f,
                              double* __restrict__ R) {
  const int64_t total = (dim - p) * S;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = p + idx / S;
    const int c = (int)(idx % S);
    double t = 0.0;
    for (int32_t j = Dptr[i]; j < Dptr[i + 1]; ++j) t += Dval[j] * X[(int64_t)Dcol[j] * S + c];
    const int64_t e = i * S + c;
    const double r = R[e];
    R[e] = r - f * ((B[e] - r) - t);
  }
}
// R -= Y
__global__ void k_sub_inplace(double* __restrict__ R, const double* __restrict__ Y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    R[i] -= Y[i];
}
// R = B - Y
__global__ void k_sub(const double* __restrict__ B, const double* __restrict__ Y, int64_t n,
                      double* __restrict__ R) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    R[i] = B[i] - Y[i];
}

static inline unsigned grid_for(int64_t n, int threads, int cap) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

// ---------------------------------------------------------------------------
template <typename T>
sv::OpView<T> make_view(Mme& m, const T* dinv);
template <>
sv::OpView<double> make_view<double>(Mme& m, const double* dinv) {
  sv::OpView<double> v{};
  v.p = m.p; v.q = m.q; v.dim = m.dim;
  v.Dptr = m.D64.ptr.p; v.Dcol = m.D64.col.p; v.Dval = m.D64.val.p;
  if (m.has_sparse) { v.Sptr = m.Qs64.ptr.p; v.Scol = m.Qs64.col.p; v.Sval = m.Qs64.val.p; }
  if (m.has_dense) { v.Qd = m.Qd64.p; v.ng = m.ng; v.ld = m.ld; v.gmap = m.gmap.p; v.ginv = m.ginv.p; }
  v.A11inv = m.A11inv64.p;
  v.dinv = dinv;
  return v;
}
template <>
sv::OpView<float> make_view<float>(Mme& m, const float* dinv) {
  sv::OpView<float> v{};
  v.p = m.p; v.q = m.q; v.dim = m.dim;
  v.Dptr = m.D32.ptr.p; v.Dcol = m.D32.col.p; v.Dval = m.D32.val.p;
  if (m.has_sparse) { v.Sptr = m.Qs32.ptr.p; v.Scol = m.Qs32.col.p; v.Sval = m.Qs32.val.p; }
  if (m.has_dense) { v.Qd = m.Qd32.p; v.ng = m.ng; v.ld = m.ld; v.gmap = m.gmap.p; v.ginv = m.ginv.p; }
  v.A11inv = m.A11inv32.p;
  v.dinv = dinv;
  return v;
}

// rows per warp of the dense kernel: RPW * S accumulators <= 64 doubles / 128 floats
template <typename T, int S>
constexpr int rpw() {
  return sizeof(T) == 8 ? (S <= 8 ? 8 : (S == 16 ? 4 : (S == 32 ? 2 : 1))) : (S <= 16 ? 8 : (S == 32 ? 4 : 2));
}

static int env_int(const char* name, int def) {
  const char* e = std::getenv(name);
  return (e && *e) ? std::atoi(e) : def;
}

template <typename T, int S>
struct Workspace {
  DevBuf<T> R, Z, P, Q, Vt, Tout, X;
  DevBuf<uint16_t> Vbf;   // bf16 hi / lo rows of the gathered vectors (CBX_BF16=1)
  DevBuf<T> Pn;           // second direction buffer of the fused iteration
  DevBuf<double> part, pq_part, rz_fix, tol, colsum;
  DevBuf<double> fpart;   // per-block partials of the fused iteration (nb_fused x 4 x S)
  DevBuf<double> cpart;   // per-block column-sum partials of its direction (nb_fused x S)
  int nb_fused = 0;       // co-resident grid of the fused iteration (0: not available)
  DevBuf<T> seg_part;
  DevBuf<sv::Col> col;
  DevBuf<int> active;
  DevBuf<unsigned> done;  // arrival counter of k_scalar_beta_c (reset by its last block)
  int nblk_vec = 0, nblk_spmv = 0;
  int nblk_dadd = 0;      // blocks of k_dense_add (their pq partials follow k_spmv's)
  int64_t dim = -1, p_ = -1, ng_ = -1, ld_ = -1;
  int nseg_ = -1;
  void alloc(const Mme& m, int num_sms) {
    if (dim == m.dim && p_ == m.p && nseg_ == m.nseg && ng_ == m.ng && ld_ == m.ld &&
        (!m.has_dense || Vt.n == (size_t)S * m.ld))
      return;
    const int64_t n = m.dim * S;
    R.resize(n); Z.resize(n); P.resize(n); Q.resize(n); X.resize(n);
    if (m.has_dense) { Vt.resize((size_t)S * m.ld); Tout.resize((size_t)m.ng * S * 8); colsum.resize(S); }
    // enough warps per SM to keep the loads of these streaming kernels in flight
    // (2 blocks per SM ran k_update at about a quarter of HBM bandwidth)
    nblk_vec = (int)grid_for(n, sv::NT, 8 * num_sms);
    nblk_spmv = (int)m.p + (int)grid_for(m.dim - m.p, 8, 6 * num_sms);
    nblk_dadd = m.has_dense ? (int)grid_for(m.ng * S, sv::NT, 2 * num_sms) : 0;
    part.resize((size_t)nblk_vec * 3 * S);
    pq_part.resize((size_t)(nblk_spmv + nblk_dadd) * S);
    rz_fix.resize((size_t)std::max<int64_t>(m.p, 1) * S);
    tol.resize(S);
    col.resize(S);
    active.resize(1);
    done.resize(1);
    CBX_CUDA(cudaMemset(done.p, 0, sizeof(unsigned)));
    seg_part.resize((size_t)std::max<int32_t>(m.nseg, 1) * S);
    dim = m.dim;
    p_ = m.p;
    nseg_ = m.nseg;
    ng_ = m.ng;
    ld_ = m.ld;
    nb_fused = 0;
    if constexpr (sizeof(T) == 4) {
      int per_sm = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sv::k_pcg_iter<T, S>, sv::NT, 0) == cudaSuccess &&
          per_sm > 0) {
        nb_fused = std::min(per_sm, 2) * num_sms;  // 2 per SM measured best (1, 3, 4 slower)
        Pn.resize(n);
        fpart.resize((size_t)nb_fused * 4 * S);
        cpart.resize((size_t)nb_fused * S);
      } else {
        cudaGetLastError();
      }
    }
  }
};

// FP32 probe blocks of 16 or 32 columns use the tcgen05 3xTF32 product unless
// the environment sets CBX_DENSE_TC=0.
// The FP32 PCG bulk's block product from a bf16 copy of the block (half the
// bytes; the inner operator is then perturbed by the block's rounding, so the
// refinement takes more outer steps) when the environment sets CBX_BF16=1.
static bool use_bf16() {
  static int v = env_int("CBX_BF16", 0);
  return v != 0;
}

static bool use_dense_tc() {
  static int v = -1;
  if (v < 0) {
    const char* e = std::getenv("CBX_DENSE_TC");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v == 1;
}
// recursive refinement residuals r -= A d with the float-float block product
// in the mixed solver (CBX_RESID_FF=0 recomputes every r = b - A x in FP64)
static bool use_resid_ff() {
  static int v = -1;
  if (v < 0) {
    const char* e = std::getenv("CBX_RESID_FF");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v == 1;
}

// Recursive-residual threshold of the mixed solver: a correction d updates
// r -= A d in float-float when ||d|| <= 2^-recur_shift ||x|| in every column
// (environment CBX_RECUR_SHIFT, default 4).
static int recur_shift() {
  static int v = env_int("CBX_RECUR_SHIFT", 4);
  return v;
}

// Floor of the inner FP32 solve's relative tolerance in the mixed solver
// (environment CBX_INNER_TOL_MIN, default 1e-5).
static double inner_tol_min() {
  static double v = [] {
    const char* e = std::getenv("CBX_INNER_TOL_MIN");
    const double x = (e && *e) ? std::atof(e) : 1e-5;
    return (x > 0 && x < 1e-1) ? x : 1e-5;
  }();
  return v;
}

// The FP32 PCG iteration as one persistent cooperative kernel after the dense
// product, when the environment sets CBX_FUSED=1 (read at every solve).  Off
// by default: on GB300 its four grid-wide barriers and per-block redundant
// reductions cost 1-10 % more per iteration than the separate kernels replayed
// from a CUDA graph (measured at n = 2,000, 8,192 and 20,000).
static bool use_fused() { return env_int("CBX_FUSED", 0) != 0; }

// Floor of the first inner solve's tolerance (environment CBX_FIRST_ITOL,
// default 1e-3).  The correction is stored in FP32, and the eigen-bent direction
// of the dense block (eigenvalue clamp^-1) turns the rounding of its entries into
// a true residual of about eps32 (lambda_max / lambda_typical) of the correction
// equation's right-hand side: for the first correction of a warm-started solve
// the true residual stops falling near 1e-3..1e-2 of its start whatever the inner
// tolerance, so iterations past 1e-3 are wasted there (measured on GB300 at
// n = 20,000: 1e-5 -> 11.3, 1e-3 -> 12.9 REML it/s, same number of refinements).
// Later corrections reach their tolerance.
// With the float-float iterate (below) the floor is gone and the first inner
// solve takes the same tolerance as the others.
static bool use_xff();
static double inner_tol_min();
static double first_itol() {
  static double v = [] {
    const char* e = std::getenv("CBX_FIRST_ITOL");
    const double def = use_xff() ? inner_tol_min() : 1e-3;
    const double x = (e && *e) ? std::atof(e) : def;
    return (x > 0 && x < 1e-1) ? x : def;
  }();
  return v;
}

// The inner FP32 solve accumulates its iterate (the correction) as a
// float-float pair unless the environment sets CBX_XFF=0.  An FP32 iterate
// rounds each entry to 2^-24 of itself; multiplied by the largest eigenvalue of
// the operator, that rounding is a residual which no inner iteration removes
// (with an eigen-bent G^-1 it stalled the first correction near 1e-3 of its
// right-hand side).  The pair costs 8 bytes per entry and a few FP32
// operations in k_update.
static bool use_xff() {
  static int v = env_int("CBX_XFF", 1);
  return v != 0;
}

// FP64-accurate refinement products of 16 or more columns on the tensor cores
// (exact fixed-point digits, dense_fx.cu) instead of the CUDA-core float-float
// kernels; CBX_FX=0 selects the float-float kernels.
static bool use_fx() {
  static int v = env_int("CBX_FX", 1);
  return v != 0;
}

// Diagnostics: the environment CBX_LOG_REFINE=1 prints every refinement step
// of the mixed solver (inner iterations, worst relative true residual) to stderr.
static bool log_refine() {
  static int v = env_int("CBX_LOG_REFINE", 0);
  return v != 0;
}

// With CBX_OVERLAP=1 the FP32 operator's sparse part (W'W, the sparse Qinv,
// the fixed rows) runs on the handle's second stream beside the dense block
// product, and the block term is added to the genotyped rows afterwards.  Off
// by default: on GB300 at the 200k-animal / 20k-genotyped ssGBLUP step the
// co-resident SpMV blocks slowed the block product from 0.82 to 0.68 of the
// copy bandwidth, and the step from 66.4 to 68.6 ms.  Never on while a launch
// trace runs, whose per-launch attribution assumes one stream.
static bool use_overlap() { return env_int("CBX_OVERLAP", 0) != 0; }
template <typename T>
static bool matvec_split(const cbx_handle* h, const sv::OpView<T>& op) {
  return sizeof(T) == 4 && op.Qd && use_overlap() && !h->trace_on;
}

// CUDA graphs for the PCG iteration body (environment CBX_GRAPHS=0 launches
// every kernel from the host instead)
static bool use_graphs() {
  static int v = env_int("CBX_GRAPHS", 1);
  return v != 0;
}

// rows per warp of the float-float product (measured on GB300 at n = 16,384:
// 16 columns x 2 rows runs at ~58 % of FP32 issue, 32 columns at <= 40 %)
template <int S>
constexpr int rpw_ff() {
  return S >= 64 ? 1 : (S >= 16 ? 2 : (S >= 8 ? 4 : 8));
}

// Vt[c * ld + k] = X[(p + gmap[k]) * xs + c] for c < ncols, k < ng (the gathered
// dense-block rows of an interleaved block, as columns of a column-major
// ld x ncols matrix).
__global__ void k_gather_cols(const double* __restrict__ X, int xs, int ncols, double* __restrict__ Vt, int64_t p,
                              int64_t ng, int64_t ld, const int32_t* __restrict__ gmap) {
  const int64_t total = (int64_t)ncols * ld;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / ld, k = idx - c * ld;
    Vt[idx] = k < ng ? X[(p + gmap[k]) * xs + c] : 0.0;
  }
}

// Float-float block products are FP32-issue-bound, so they run on the
// populated columns only, in power-of-two pieces written into the S-wide output;
// R rows per warp.
template <int W, int R = rpw_ff<W>()>
static void ff_piece(cbx_handle* h, const sv::OpView<double>& op, const double* X, int xs, double* Vt,
                     double* Tout, const int* active) {
  cudaStream_t s = h->stream;
  const Mme& mm = *h->mme;
  // (hi, lo) pairs take the space of the FP64 gather buffer
  float2* vhl = reinterpret_cast<float2*>(Vt);
  sv::k_gather_hl<W><<<grid_for(W * op.ld, 256, 4 * h->num_sms), 256, 0, s>>>(X, vhl, op.p, op.ng, op.ld, op.gmap,
                                                                            xs);
  h->launched("k_gather_hl<f64>");
  const int smem = W * 256 * (int)sizeof(float2);
  ensure_smem((const void*)sv::k_dense_ff<W, R>, smem, h->device);
  sv::k_dense_ff<W, R><<<(unsigned)((op.ng + 8 * R - 1) / (8 * R)), 256, smem, s>>>(mm.Qd32.p, mm.Qlo32.p, op.ng,
                                                                                   op.ld, vhl, Tout, active, xs);
  h->launched("k_dense_ff<f64>");
}

// The same with the packed (f32x2) kernel, for an even width W.
template <int W, int R = rpw_ff<W>()>
static void ff_piece2(cbx_handle* h, const sv::OpView<double>& op, const double* X, int xs, double* Vt,
                      double* Tout, const int* active) {
  cudaStream_t s = h->stream;
  const Mme& mm = *h->mme;
  float2* vhl = reinterpret_cast<float2*>(Vt);
  sv::k_gather_hl<W><<<grid_for(W * op.ld, 256, 4 * h->num_sms), 256, 0, s>>>(X, vhl, op.p, op.ng, op.ld, op.gmap,
                                                                            xs);
  h->launched("k_gather_hl<f64>");
  const int smem = W * 256 * (int)sizeof(float2);
  ensure_smem((const void*)sv::k_dense_ff2<W, R>, smem, h->device);
  sv::k_dense_ff2<W, R><<<(unsigned)((op.ng + 8 * R - 1) / (8 * R)), 256, smem, s>>>(mm.Qd32.p, mm.Qlo32.p, op.ng,
                                                                                    op.ld, vhl, Tout, active, xs);
  h->launched("k_dense_ff2<f64>");
}

// The float-float product of ncols populated columns under one launch-shape plan
// (the autotuner's candidates; every plan gives the same bits, since each output's
// accumulation order depends only on the K tiling):
//   0: pieces of at most 16 columns, rows per warp by width (16 -> 2)
//   1: pieces of at most 16 columns, one row per warp at width 16
//   2: pieces of at most 8 columns (4 rows per warp)
//   3: pieces of at most 32 columns, one row per warp at width 32
//   4-7: plans 0-3 with the packed f32x2 kernel for pieces of 2 or more columns
constexpr int FF_PLANS = 8;
static void ff_plan(cbx_handle* h, const sv::OpView<double>& op, const double* X, int S, int ncols, double* Vt,
                    double* Tout, const int* active, int plan) {
  const bool packed = plan >= 4;
  const int base = plan & 3;
  const int cap = base == 2 ? 8 : (base == 3 ? 32 : 16);
  for (int c0 = 0; c0 < ncols;) {
    const int left = std::min(ncols - c0, cap);
    int w = 1;
    while (2 * w <= left) w <<= 1;
    const double* x = X + c0;
    double* t = Tout + c0;
    switch (w) {
      case 1: ff_piece<1>(h, op, x, S, Vt, t, active); break;
      case 2: packed ? ff_piece2<2>(h, op, x, S, Vt, t, active) : ff_piece<2>(h, op, x, S, Vt, t, active); break;
      case 4: packed ? ff_piece2<4>(h, op, x, S, Vt, t, active) : ff_piece<4>(h, op, x, S, Vt, t, active); break;
      case 8: packed ? ff_piece2<8>(h, op, x, S, Vt, t, active) : ff_piece<8>(h, op, x, S, Vt, t, active); break;
      case 16:
        if (base == 1) packed ? ff_piece2<16, 1>(h, op, x, S, Vt, t, active) : ff_piece<16, 1>(h, op, x, S, Vt, t, active);
        else packed ? ff_piece2<16>(h, op, x, S, Vt, t, active) : ff_piece<16>(h, op, x, S, Vt, t, active);
        break;
      default:
        packed ? ff_piece2<32, 1>(h, op, x, S, Vt, t, active) : ff_piece<32, 1>(h, op, x, S, Vt, t, active);
        break;
    }
    c0 += w;
  }
}

// Tout[:, 0:ncols] (rows S apart) of the dense block product in FP64
// accuracy: float-float on the CUDA cores (ff), or cuBLAS DGEMM / DGEMV on the
// gathered columns (the block is an ng x ng column-major matrix with leading
// dimension ld; it is symmetric, so either orientation gives Qinv X).
static void dense64(cbx_handle* h, const sv::OpView<double>& op, const double* X, int S, int ncols, double* Vt,
                    double* Tout, const int* active, bool ff, double* colsum) {
  if (ff) {
    // the compensated FP64 column sums that restore the block's shift
    sv::k_colsum_x<<<ncols, 256, 0, h->stream>>>(X, S, op.p, op.ng, op.gmap, colsum);
    h->launched("k_colsum_x<f64>");
    if (use_fx() && ncols >= 16) {
      // tensor-core fixed-point product, 32 columns at a time; fewer than 16
      // columns left over go to the float-float kernels below
      Mme& mm = *h->mme;
      if (!mm.fx_rows_ok) {
        mm.fx_rowexp.resize(op.ng);
        fx_row_scales(h, mm.Qd32.p, op.ng, op.ld, mm.fx_rowexp.p);
        mm.fx_rows_ok = true;
      }
      int c0 = 0;
      for (; ncols - c0 >= 16; c0 += 32) {
        const int nc = std::min(32, ncols - c0);
        fx_product(h, mm.Qd32.p, mm.Qlo32.p, mm.fx_rowexp.p, op.ng, op.ld, X + c0, S, op.p, op.gmap, nc, mm.fx_bdig,
                   mm.fx_cexp, mm.fx_part, Tout + c0, S, active);
      }
      if (c0 >= ncols) return;
      X += c0;
      Tout += c0;
      ncols -= c0;
    }
    // the launch shape is tuned per block order (two 16-column passes with 2 rows
    // per warp measured best at n = 20,000: register pressure, not the second read
    // of the block, limits the wider pieces)
    // one decision per block order, taken at the first product with at least 16
    // columns (narrower ones run the same pieces under every plan but the last)
    const int plan = tune::choose(
        h, tune::FF, tune::size_class(op.ng), 0, 16, FF_PLANS,
        [&](int c) { ff_plan(h, op, X, S, ncols, Vt, Tout, active, c); }, ncols >= 16);
    ff_plan(h, op, X, S, ncols, Vt, Tout, active, plan);
    return;
  }
  cudaStream_t s = h->stream;
  k_gather_cols<<<grid_for((int64_t)ncols * op.ld, 256, 4 * h->num_sms), 256, 0, s>>>(X, S, ncols, Vt, op.p, op.ng,
                                                                                     op.ld, op.gmap);
  h->launched("k_gather_cols<f64>");
  Libs& L = libs(h);
  const double one = 1.0, zero = 0.0;
  if (ncols == 1) {
    // Tout[i * S] = sum_k Q(k, i) v(k)
    CBX_BLAS(cublasDgemv(L.blas, CUBLAS_OP_T, (int)op.ng, (int)op.ng, &one, op.Qd, (int)op.ld, Vt, 1, &zero, Tout,
                         S));
  } else {
    // Tout^T (ncols x ng, leading dimension S) = Vt^T (ncols x ng) * Q (ng x ng)
    CBX_BLAS(cublasDgemm(L.blas, CUBLAS_OP_T, CUBLAS_OP_N, ncols, (int)op.ng, (int)op.ng, &one, Vt, (int)op.ld,
                         op.Qd, (int)op.ld, &zero, Tout, S));
  }
  h->launched("cublas_dgemm<f64>");
}

// FP32 dense block product Tout = Qd Vt^T from the gathered operand w.Vt (the
// tcgen05 3xTF32 kernel for 16, 32 or 64 columns, the HBM-streaming GEMV for
// one, the CUDA-core kernel otherwise); returns the number of K-split partials.
template <typename T, int S>
int product_from_vt(cbx_handle* h, const sv::OpView<T>& op, Workspace<T, S>& w, const int* active,
                    int ncols = S) {
  cudaStream_t s = h->stream;
  int tsplit = 1;
  cbx_handle::ProfRec pr{};
  if (h->prof_on) {
    CBX_CUDA(cudaEventCreate(&pr.a));
    CBX_CUDA(cudaEventCreate(&pr.b));
    CBX_CUDA(cudaEventRecord(pr.a, s));
  }
  bool bf = false;
  if ((S == 16 || S == 32 || S == 64 || S == 128) && sizeof(T) == 4 && h->mme->Qbf.p && use_dense_tc()) {
    w.Vbf.resize((size_t)2 * S * op.ld);
    tsplit = dense_bf(h, h->mme->Qbf.p, op.ng, op.ld, reinterpret_cast<const float*>(w.Vt.p), S, w.Vbf.p,
                      reinterpret_cast<float*>(w.Tout.p), active, ncols);
    bf = true;
  } else if ((S == 16 || S == 32 || S == 64 || S == 128) && use_dense_tc()) {
    tsplit = dense_tc_ksplit(op.ng, op.ld, h->num_sms);
    dense_tc(h, reinterpret_cast<const float*>(op.Qd), op.ng, op.ld, reinterpret_cast<const float*>(w.Vt.p), S,
             tsplit, reinterpret_cast<float*>(w.Tout.p), active, ncols);
  } else if constexpr (S == 128) {
    throw Error(CBX_ERR_UNSUPPORTED, "the 128-wide block needs the tensor-core product (CBX_DENSE_TC=1)");
  } else if (S == 1) {
    // rows per warp x loads in flight per lane, tuned per block order (all shapes
    // accumulate each row in the same order)
    auto gemv = [&](int c) {
      switch (c) {
        case 1: sv::k_gemv<T, 2, 4><<<(unsigned)((op.ng + 15) / 16), 256, 0, s>>>(op.Qd, op.ng, op.ld, w.Vt.p,
                                                                               w.Tout.p, active); break;
        case 2: sv::k_gemv<T, 8, 2><<<(unsigned)((op.ng + 63) / 64), 256, 0, s>>>(op.Qd, op.ng, op.ld, w.Vt.p,
                                                                               w.Tout.p, active); break;
        case 3: sv::k_gemv<T, 2, 8><<<(unsigned)((op.ng + 15) / 16), 256, 0, s>>>(op.Qd, op.ng, op.ld, w.Vt.p,
                                                                               w.Tout.p, active); break;
        default: sv::k_gemv<T, 4, 4><<<(unsigned)((op.ng + 31) / 32), 256, 0, s>>>(op.Qd, op.ng, op.ld, w.Vt.p,
                                                                                w.Tout.p, active); break;
      }
      h->launched("k_gemv<f32>");
    };
    gemv(tune::choose(h, tune::GEMV, tune::size_class(op.ng), (int)sizeof(T), 1, 4, gemv));
  } else {
    constexpr int R = rpw<T, S>();
    constexpr int KT = 32 * sv::Vec16<T>::n * 4;
    const int smem = S * KT * (int)sizeof(T);
    ensure_smem((const void*)sv::k_dense<T, S, R>, smem, h->device);
    sv::k_dense<T, S, R><<<(unsigned)((op.ng + 8 * R - 1) / (8 * R)), 256, smem, s>>>(op.Qd, op.ng, op.ld, w.Vt.p,
                                                                                     w.Tout.p, active);
    h->launched("k_dense<f32>");
  }
  if (h->prof_on) {
    CBX_CUDA(cudaEventRecord(pr.b, s));
    pr.bucket = 0;
    // algorithmic bytes: the dense block once (bf16 or FP32), the S gathered vectors, the outputs
    pr.bytes = (bf ? 2.0 : 4.0) * (double)op.ng * op.ld + 4.0 * ((double)S * op.ld + (double)op.ng * S * tsplit);
    h->prof.push_back(pr);
  }
  return tsplit;
}

// Y = use_D * W'W X + lam [0; Qinv X_u] for an S-wide interleaved block whose
// first ncols columns are populated (the rest are zero or ignored); optional
// pq partials sum_i P[i] Y[i] for the PCG step.
template <typename T, int S>
void matvec(cbx_handle* h, const sv::OpView<T>& op, Workspace<T, S>& w, const T* X, T* Y, double lam, int use_D,
            const T* P, double* pq_part, const int* active, bool ff = false, int ncols = S) {
  cudaStream_t s = h->stream;
  int tsplit = 1;
  // columns computed: the populated ones rounded up to whole 32-column groups
  // (the 128-wide block computes three groups)
  const int ncp = std::min(S, (ncols + 31) / 32 * 32);
  CBX_REQUIRE(S != 128 || ncols <= 96, CBX_ERR_ARG, "the 128-wide block takes at most 96 populated columns");
  // The FP32 and float-float products use the shifted copies and add
  // qshift * (column sums) back; the FP64 product uses the block itself.
  const double* colsum = op.Qd ? w.colsum.p : nullptr;
  const double tshift = h->mme->qshift;
  if (!op.Qd) {
  } else if constexpr (sizeof(T) == 8) {
    ff = ff && h->mme->Qlo32.p && h->mme->Qd32.p;
    if (!ff) colsum = nullptr;
    cbx_handle::ProfRec pr{};
    if (h->prof_on) {
      CBX_CUDA(cudaEventCreate(&pr.a));
      CBX_CUDA(cudaEventCreate(&pr.b));
      CBX_CUDA(cudaEventRecord(pr.a, s));
    }
    if (ncols < S) {
      CBX_CUDA(cudaMemsetAsync(w.Tout.p, 0, (size_t)op.ng * S * sizeof(double), s));
      CBX_CUDA(cudaMemsetAsync(w.colsum.p, 0, S * sizeof(double), s));
    }
    dense64(h, op, X, S, ncols, w.Vt.p, w.Tout.p, active, ff, w.colsum.p);
    if (h->prof_on) {
      CBX_CUDA(cudaEventRecord(pr.b, s));
      pr.bucket = 1;
      pr.bytes = 8.0 * (double)op.ng * op.ld + 8.0 * ncols * ((double)op.ld + (double)op.ng);
      h->prof.push_back(pr);
    }
  } else {
    // FP32: gather the dense-block rows, their FP64 column sums, the product
    // (the populated 32-column groups only)
    const bool split = matvec_split(h, op);
    if (split) {
      // the sparse part on the second stream, beside the block product: k_spmv
      // without the block term writes every row and its pq partials
      cudaStream_t s2 = h->stream2;
      CBX_CUDA(cudaEventRecord(h->ev_fork, s));
      CBX_CUDA(cudaStreamWaitEvent(s2, h->ev_fork, 0));
      sv::OpView<T> ops = op;
      ops.Qd = nullptr;
      if (use_D && h->mme->nseg > 0) {
        const Mme& mm = *h->mme;
        sv::k_fix_seg<T, S><<<mm.nseg, sv::NT, 0, s2>>>(ops, mm.seg_row.p, mm.seg_lo.p, mm.seg_hi.p, X,
                                                        w.seg_part.p, active, ncp);
        h->launched("k_fix_seg<f32>");
      }
      sv::k_spmv<T, S><<<w.nblk_spmv, sv::NT, 0, s2>>>(ops, X, nullptr, 1, nullptr, 0.0, h->mme->fix_seg_ptr.p,
                                                        w.seg_part.p, (T)lam, use_D, Y, P, pq_part, active, ncp);
      h->launched("k_spmv<f32>");
      CBX_CUDA(cudaEventRecord(h->ev_join, s2));
    }
    sv::k_gather_t<T, S><<<grid_for(ncp * op.ld, 256, 16 * h->num_sms), 256, 0, s>>>(X, w.Vt.p, op.p, op.ng, op.ld,
                                                                                 op.gmap, active, S, ncp);
    h->launched("k_gather_t<f32>");
    sv::k_colsum_vt<T><<<ncp, 1024, 0, s>>>(w.Vt.p, op.ld, op.ng, w.colsum.p);
    h->launched("k_colsum_vt<f32>");
    tsplit = product_from_vt<T, S>(h, op, w, active, ncols);
    if (split) {
      // the block term of the genotyped rows, once both are done
      CBX_CUDA(cudaStreamWaitEvent(s, h->ev_join, 0));
      sv::k_dense_add<T, S><<<w.nblk_dadd, sv::NT, 0, s>>>(op, w.Tout.p, tsplit, colsum, tshift, (T)lam, Y, P,
                                                           pq_part ? pq_part + (size_t)w.nblk_spmv * S : nullptr,
                                                           active, ncp);
      h->launched("k_dense_add<f32>");
      return;
    }
  }
  if (use_D && h->mme->nseg > 0) {
    const Mme& mm = *h->mme;
    sv::k_fix_seg<T, S><<<mm.nseg, sv::NT, 0, s>>>(op, mm.seg_row.p, mm.seg_lo.p, mm.seg_hi.p, X, w.seg_part.p, active,
                                                   ncp);
    h->launched(sizeof(T) == 4 ? "k_fix_seg<f32>" : "k_fix_seg<f64>");
  }
  sv::k_spmv<T, S><<<w.nblk_spmv, sv::NT, 0, s>>>(op, X, w.Tout.p, tsplit, colsum, tshift, h->mme->fix_seg_ptr.p,
                                                  w.seg_part.p,
                                                  (T)lam, use_D, Y, P, pq_part, active, ncp);
  h->launched(sizeof(T) == 4 ? "k_spmv<f32>" : "k_spmv<f64>");
}

// Multi-RHS PCG in precision T on interleaved vectors; X receives the solution
// (holds x0 when use_x0).  tol_col: per-column tolerance.
template <typename T, int S>
void run_pcg(cbx_handle* h, Mme& m, const sv::OpView<T>& op, Workspace<T, S>& w, double lam, const T* B, T* X,
             int ncols, const double* tol_col, int abs_tol, int maxit, bool use_x0, std::vector<sv::Col>& out,
             int64_t& matvecs, T* Xlo = nullptr) {
  cudaStream_t s = h->stream;
  const int64_t n = m.dim * S;
  if (use_x0) {
    matvec<T, S>(h, op, w, X, w.Q.p, lam, 1, nullptr, nullptr, nullptr, false, ncols);
    ++matvecs;
  } else {
    CBX_CUDA(cudaMemsetAsync(X, 0, n * sizeof(T), s));
  }
  if (Xlo) CBX_CUDA(cudaMemsetAsync(Xlo, 0, n * sizeof(T), s));
  sv::k_init_resid<T, S><<<w.nblk_vec, sv::NT, 0, s>>>(op, B, w.Q.p, use_x0 ? 1 : 0, w.R.p, w.Z.p, w.part.p);
  h->launched(sizeof(T) == 4 ? "k_init_resid<f32>" : "k_init_resid<f64>");
  if (m.p > 0) {
    sv::k_fixed<T, S><<<(unsigned)m.p, sv::NT_FIXED, 0, s>>>(op, w.R.p, w.Z.p, nullptr, w.rz_fix.p);
    h->launched(sizeof(T) == 4 ? "k_fixed<f32>" : "k_fixed<f64>");
  }
  std::vector<double> tolv(S, 1.0);
  for (int c = 0; c < ncols; ++c) tolv[c] = tol_col[c];
  CBX_CUDA(cudaMemcpyAsync(w.tol.p, tolv.data(), S * sizeof(double), cudaMemcpyHostToDevice, s));
  sv::k_scalar_init<S><<<1, sv::NTS, 0, s>>>(w.col.p, ncols, w.part.p, w.nblk_vec, w.rz_fix.p, m.p, abs_tol,
                                             w.active.p);
  h->launched(sizeof(T) == 4 ? "k_scalar_init<f32>" : "k_scalar_init<f64>");
  CBX_CUDA(cudaMemcpyAsync(w.P.p, w.Z.p, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
  int host_active = 1;
  // host check of the active-column count every CHECK iterations; the FP64
  // block product is slow enough (and cannot skip finished blocks) to check
  // after every iteration
  const int CHECK = (sizeof(T) == 8 && op.Qd) ? 1 : 8;
  // FP32: one persistent cooperative kernel per iteration after the dense
  // product (pcg_fused.cuh); CHECK is even, so the direction is back in w.P
  // after every block of CHECK iterations
  const bool fused = sizeof(T) == 4 && w.nb_fused > 0 && use_fused() && CHECK % 2 == 0 && !Xlo;
  const Mme& mm = m;
  if (fused && op.Qd) {
    sv::k_gather_t<T, S><<<grid_for(S * op.ld, 256, 4 * h->num_sms), 256, 0, s>>>(w.P.p, w.Vt.p, op.p, op.ng, op.ld,
                                                                               op.gmap, nullptr);
    h->launched("k_gather_t<f32>");
    sv::k_colsum_vt<T><<<S, 1024, 0, s>>>(w.Vt.p, op.ld, op.ng, w.colsum.p);
    h->launched("k_colsum_vt<f32>");
  }
  auto fused_step = [&](const T* P, T* Pn, bool first) {
    int tsplit = 1;
    if (op.Qd) tsplit = product_from_vt<T, S>(h, op, w, w.active.p, ncols);
    sv::FusedArgs<T> a{};
    a.op = op;
    a.Tout = w.Tout.p;
    a.tsplit = tsplit;
    // the first step's direction sums come from k_colsum_vt, later ones from
    // the previous step's per-block partials
    a.colsum = (op.Qd && first) ? w.colsum.p : nullptr;
    a.cpart_in = (op.Qd && !first) ? w.cpart.p : nullptr;
    a.cpart_out = op.Qd ? w.cpart.p : nullptr;
    a.tshift = mm.qshift;
    a.lam = (T)lam;
    a.seg_lo = mm.seg_lo.p;
    a.seg_hi = mm.seg_hi.p;
    a.nseg = mm.nseg;
    a.fix_seg_ptr = mm.fix_seg_ptr.p;
    a.seg_part = w.seg_part.p;
    a.X = X;
    a.R = w.R.p;
    a.Z = w.Z.p;
    a.P = P;
    a.Pn = Pn;
    a.Q = w.Q.p;
    a.Vt = op.Qd ? w.Vt.p : nullptr;
    a.col = w.col.p;
    a.tol_col = w.tol.p;
    a.abs_tol = abs_tol;
    a.maxit = maxit;
    a.active = w.active.p;
    a.part = w.fpart.p;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)w.nb_fused);
    cfg.blockDim = dim3(sv::NT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CBX_CUDA(cudaLaunchKernelEx(&cfg, sv::k_pcg_iter<T, S>, a));
    h->launched("k_pcg_iter<f32>");
  };
  auto iterations = [&](bool first_block) {
    if (fused) {
      for (int j = 0; j < CHECK; j += 2) {
        fused_step(w.P.p, w.Pn.p, first_block && j == 0);
        fused_step(w.Pn.p, w.P.p, false);
      }
      return;
    }
    for (int j = 0; j < CHECK; ++j) {
      matvec<T, S>(h, op, w, w.P.p, w.Q.p, lam, 1, w.P.p, w.pq_part.p, w.active.p, false, ncols);
      sv::k_scalar_alpha_c<S><<<S, sv::NTC, 0, s>>>(w.col.p, w.pq_part.p,
                                                    w.nblk_spmv + (matvec_split(h, op) ? w.nblk_dadd : 0));
      h->launched(sizeof(T) == 4 ? "k_scalar_alpha<f32>" : "k_scalar_alpha<f64>");
      sv::k_update<T, S><<<w.nblk_vec, sv::NT, 0, s>>>(op, w.col.p, X, Xlo, w.R.p, w.P.p, w.Q.p, w.part.p);
      h->launched(sizeof(T) == 4 ? "k_update<f32>" : "k_update<f64>");
      if (m.p > 0) {
        sv::k_fixed<T, S><<<(unsigned)m.p, sv::NT_FIXED, 0, s>>>(op, w.R.p, w.Z.p, w.col.p, w.rz_fix.p);
        h->launched(sizeof(T) == 4 ? "k_fixed<f32>" : "k_fixed<f64>");
      }
      sv::k_scalar_beta_c<S><<<S, sv::NTC, 0, s>>>(w.col.p, w.part.p, w.nblk_vec, w.rz_fix.p, m.p, w.tol.p, abs_tol,
                                                   maxit, w.active.p, w.done.p);
      h->launched(sizeof(T) == 4 ? "k_scalar_beta<f32>" : "k_scalar_beta<f64>");
      sv::k_pupdate<T, S><<<grid_for(m.dim * S, sv::NT, 16 * h->num_sms), sv::NT, 0, s>>>(
          m.dim, m.p, op.dinv, w.col.p, w.R.p, w.Z.p, w.P.p);
      h->launched(sizeof(T) == 4 ? "k_pupdate<f32>" : "k_pupdate<f64>");
    }
  };
  // After the first CHECK iterations (run eagerly: short solves pay no graph
  // set-up, and one-time function attributes are set outside any capture),
  // the CHECK-iteration body is captured once as a CUDA graph and replayed:
  // one launch per CHECK iterations instead of ~10 per iteration.  Every
  // kernel in it still skips its work once no column is active.
  const bool graphs = CHECK > 1 && !h->prof_on && !h->trace_on && use_graphs();
  cudaGraphExec_t gexec = nullptr;
  bool graph_failed = false;
  int64_t graph_launches = 0;
  try {
    for (int it = 0; it < maxit && host_active; it += CHECK) {
      if (it > 0 && graphs && !gexec && !graph_failed) {
        // A body that cannot be captured (or instantiated) runs eagerly: the
        // capture launched nothing, so nothing is lost.
        cudaGraph_t g = nullptr;
        const int64_t l0 = h->launches;
        bool ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
          try {
            iterations(false);
          } catch (...) {
            ok = false;
          }
          ok = (cudaStreamEndCapture(s, &g) == cudaSuccess) && ok && g;
        }
        if (ok) ok = cudaGraphInstantiate(&gexec, g, 0) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
        graph_launches = h->launches - l0;
        h->launches = l0;
        if (!ok) {
          gexec = nullptr;
          graph_failed = true;
          cudaGetLastError();
        }
      }
      if (gexec) {
        CBX_CUDA(cudaGraphLaunch(gexec, s));
        h->launches += graph_launches;
      } else {
        iterations(it == 0);
      }
      matvecs += CHECK;
      CBX_CUDA(cudaMemcpyAsync(&host_active, w.active.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      CBX_CUDA(cudaStreamSynchronize(s));
    }
  } catch (...) {
    if (gexec) cudaGraphExecDestroy(gexec);
    throw;
  }
  if (gexec) CBX_CUDA(cudaGraphExecDestroy(gexec));
  out.resize(S);
  CBX_CUDA(cudaMemcpyAsync(out.data(), w.col.p, S * sizeof(sv::Col), cudaMemcpyDeviceToHost, s));
  CBX_CUDA(cudaStreamSynchronize(s));
}

template <int S>
struct Solver : public SolverBase {
  Workspace<double, S> w64;
  Workspace<float, S> w32;
  DevBuf<double> dinv64, Bi, Xi, R64, Y64, part, scale, Dc64;
  DevBuf<float> dinv32, R32, D32, D32lo;
  double dinv_lam = std::nan("");

  void rebind() override {
    dinv_lam = std::nan("");
    w64.dim = w32.dim = -1;  // the next prepare re-checks every size and clears the counters
  }

  void prepare(cbx_handle* h, Mme& m, double lam, bool need32) {
    cudaStream_t s = h->stream;
    w64.alloc(m, h->num_sms);
    const int64_t n = m.dim * S;
    Bi.resize(n); Xi.resize(n); R64.resize(n); Y64.resize(n);
    part.resize((size_t)w64.nblk_vec * S);
    scale.resize(S);
    if (!(dinv_lam == lam) || dinv64.n != (size_t)m.q) {
      dinv64.resize(m.q);
      k_dinv<double><<<grid_for(m.q, 256, 1024), 256, 0, s>>>(m.diagD.p, m.diagQ.p, m.p, m.q, lam, dinv64.p);
      h->launched("k_dinv");
      dinv32.resize(m.q);
      k_dinv<float><<<grid_for(m.q, 256, 1024), 256, 0, s>>>(m.diagD.p, m.diagQ.p, m.p, m.q, lam, dinv32.p);
      h->launched("k_dinv");
      dinv_lam = lam;
    }
    if (need32) {
      w32.alloc(m, h->num_sms);
      R32.resize(n);
      D32.resize(n);
      Dc64.resize(n);
      if (use_xff() && !use_fused()) D32lo.resize(n);
    }
  }

  // column norms of an interleaved FP64 block (2 blocks per SM: the partials
  // come back to the host)
  std::vector<double> norms(cbx_handle* h, Mme& m, const double* V) {
    cudaStream_t s = h->stream;
    const int nb = std::min(w64.nblk_vec, 2 * h->num_sms);
    sv::k_colnorm2<S><<<nb, sv::NT, 0, s>>>(V, m.dim, part.p);
    h->launched("k_colnorm2");
    std::vector<double> ph((size_t)nb * S);
    CBX_CUDA(cudaMemcpyAsync(ph.data(), part.p, ph.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    std::vector<double> r(S, 0.0);
    for (int c = 0; c < S; ++c) {
      double t = 0;
      for (int b = 0; b < nb; ++b) t += ph[(size_t)b * S + c];
      r[c] = std::sqrt(t);
    }
    return r;
  }

  // R64 = B - A X in FP64; returns ||R64|| per column
  // R64 = B - A X in FP64 accuracy (ff: the float-float product of the shifted
  // block, whose error is relative to the block without its common offset)
  std::vector<double> residual(cbx_handle* h, Mme& m, const sv::OpView<double>& op, double lam, int64_t& mv,
                               int ncols, bool ff = false) {
    cudaStream_t s = h->stream;
    matvec<double, S>(h, op, w64, Xi.p, Y64.p, lam, 1, nullptr, nullptr, nullptr, ff, ncols);
    ++mv;
    const int64_t n = m.dim * S;
    k_sub<<<grid_for(n, 256, 4 * h->num_sms), 256, 0, s>>>(Bi.p, Y64.p, n, R64.p);
    h->launched("k_sub");
    return norms(h, m, R64.p);
  }

  // have_r0: R64 holds b - A(lam - dlam) X on entry (see ResidCarry)
  void solve(cbx_handle* h, Mme& m, double lam, int ncols, bool use_x0, double tol, int maxit, int abs_tol,
             int precision, PcgResult& res, bool have_r0 = false, double dlam = 0.0) {
    cudaStream_t s = h->stream;
    prepare(h, m, lam, precision != 0);
    auto op64 = make_view<double>(m, dinv64.p);
    res.iters.assign(ncols, 0);
    res.status.assign(ncols, 0);
    res.relres.assign(ncols, 0.0);
    res.refinements = 0;
    res.matvecs = 0;
    std::vector<double> tolv(ncols, tol);
    if (precision == 0) {
      std::vector<sv::Col> cols;
      run_pcg<double, S>(h, m, op64, w64, lam, Bi.p, Xi.p, ncols, tolv.data(), abs_tol, maxit, use_x0, cols,
                         res.matvecs);
      bool need_true = false;
      for (int c = 0; c < ncols; ++c) need_true |= cols[c].status != sv::COL_CONVERGED;
      std::vector<double> rn, bn;
      if (need_true) {
        rn = residual(h, m, op64, lam, res.matvecs, ncols);
        bn = norms(h, m, Bi.p);
      }
      for (int c = 0; c < ncols; ++c) {
        res.iters[c] = cols[c].iters;
        res.status[c] = cols[c].status;
        const double b = cols[c].bnorm2 > 0 ? std::sqrt(cols[c].bnorm2) : 1.0;
        if (cols[c].status == sv::COL_CONVERGED)
          res.relres[c] = abs_tol ? std::sqrt(cols[c].rr) : std::sqrt(cols[c].rr) / b;
        else
          res.relres[c] = abs_tol ? rn[c] : (bn[c] > 0 ? rn[c] / bn[c] : 0.0);
      }
      return;
    }
    // ---- mixed precision: FP32 PCG on A d = r, x += d, r = b - A x in FP64
    auto op32 = make_view<float>(m, dinv32.p);
    const int64_t n = m.dim * S;
    if (!use_x0) CBX_CUDA(cudaMemsetAsync(Xi.p, 0, n * sizeof(double), s));
    std::vector<double> bn = norms(h, m, Bi.p);
    std::vector<double> rn;
    if (use_x0 && have_r0 && lam - dlam > 0.0) {
      // b - A(lam) x0 from the carried b - A(lam - dlam) x0, without a dense product
      if (dlam != 0.0) {
        k_carry_resid<<<grid_for((m.dim - m.p) * S, 256, 4 * h->num_sms), 256, 0, s>>>(
            m.D64.ptr.p, m.D64.col.p, m.D64.val.p, m.p, m.dim, S, Bi.p, Xi.p, dlam / (lam - dlam), R64.p);
        h->launched("k_carry_resid");
      }
      rn = norms(h, m, R64.p);
    } else if (use_x0) {
      rn = residual(h, m, op64, lam, res.matvecs, ncols, use_resid_ff());
    } else {
      // x0 = 0: the residual is b itself, no FP64 operator application needed
      CBX_CUDA(cudaMemcpyAsync(R64.p, Bi.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      rn = bn;
    }
    for (auto& b : bn) if (!(b > 0)) b = 1.0;
    std::vector<int> done(ncols, 0);
    double worst0 = 0.0;
    for (int c = 0; c < ncols; ++c) {
      const double rel = abs_tol ? rn[c] : rn[c] / bn[c];
      worst0 = std::max(worst0, rel);
      if (rel < tol) done[c] = 1;
    }
    if (log_refine())
      std::fprintf(stderr, "[cbx refine] S=%d cols=%d start warm=%d carried=%d worst_relres=%.3e\n", S, ncols,
                   use_x0 ? 1 : 0, (use_x0 && have_r0) ? 1 : 0, worst0);
    for (int outer = 0; outer < 60; ++outer) {
      std::vector<double> sc(S, 0.0), itol(S, 1.0);
      int inner_max = 0;
      for (int c = 0; c < ncols; ++c)
        if (!done[c] && res.iters[c] < maxit) {
          sc[c] = rn[c] > 0 ? rn[c] : 1.0;
          const double need = abs_tol ? tol / rn[c] : tol * bn[c] / rn[c];
          itol[c] = std::min(1e-2, std::max(outer == 0 ? first_itol() : inner_tol_min(), 0.5 * need));
          inner_max = std::max(inner_max, maxit - res.iters[c]);
        }
      if (inner_max == 0) break;
      CBX_CUDA(cudaMemcpyAsync(scale.p, sc.data(), S * sizeof(double), cudaMemcpyHostToDevice, s));
      k_scale_down<<<grid_for(n, 256, 4 * h->num_sms), 256, 0, s>>>(R64.p, scale.p, m.dim, S, R32.p);
      h->launched("k_scale_down");
      std::vector<sv::Col> cols;
      float* dlo = (use_xff() && !use_fused()) ? D32lo.p : nullptr;
      run_pcg<float, S>(h, m, op32, w32, lam, R32.p, D32.p, ncols, itol.data(), 0, inner_max, false, cols,
                        res.matvecs, dlo);
      k_correction<<<grid_for(n, 256, 4 * h->num_sms), 256, 0, s>>>(Xi.p, D32.p, dlo, scale.p, m.dim, S, Dc64.p);
      h->launched("k_correction");
      res.refinements += 1;
      // Residual of the new iterate, with the float-float product of the
      // shifted block: its error is ~2^-46 of |Qd - shift| |v| per row, below
      // the rounding of an FP64 product with the unshifted block when the
      // block carries a large common offset (an eigen-bent G^-1).  A
      // correction that is small next to the solution (||d|| <= 2^-4 ||x|| in
      // every column) updates r -= A d; otherwise (the first correction from
      // x0 = 0, where d = x) r = b - A x is formed afresh.
      bool recursive = use_resid_ff() && m.Qlo32.p;
      if (recursive) {
        const std::vector<double> dn = norms(h, m, Dc64.p), xn = norms(h, m, Xi.p);
        for (int c = 0; c < ncols; ++c)
          if (sc[c] > 0 && !(dn[c] <= std::ldexp(xn[c], -recur_shift()))) recursive = false;
      }
      std::vector<double> rn_new;
      if (recursive) {
        matvec<double, S>(h, op64, w64, Dc64.p, Y64.p, lam, 1, nullptr, nullptr, nullptr, true, ncols);
        ++res.matvecs;
        k_sub_inplace<<<grid_for(n, 256, 4 * h->num_sms), 256, 0, s>>>(R64.p, Y64.p, n);
        h->launched("k_sub_inplace");
        rn_new = norms(h, m, R64.p);
      } else {
        rn_new = residual(h, m, op64, lam, res.matvecs, ncols, use_resid_ff());
      }
      double worst = 0.0;
      int inner = 0;
      for (int c = 0; c < ncols; ++c) {
        if (sc[c] <= 0) continue;
        res.iters[c] += cols[c].iters;
        inner = std::max(inner, cols[c].iters);
        const double rel = abs_tol ? rn_new[c] : rn_new[c] / bn[c];
        worst = std::max(worst, rel);
        if (rel < tol) done[c] = 1;
        else if (!(rn_new[c] < 0.9 * rn[c])) done[c] = 2;  // FP32 refinement stalled
        rn[c] = rn_new[c];
      }
      if (log_refine())
        std::fprintf(stderr, "[cbx refine] S=%d cols=%d outer=%d inner_iters=%d recursive=%d worst_relres=%.3e\n",
                     S, ncols, outer, inner, recursive ? 1 : 0, worst);
    }
    for (int c = 0; c < ncols; ++c) {
      res.relres[c] = abs_tol ? rn[c] : rn[c] / bn[c];
      res.status[c] = done[c] == 1 ? sv::COL_CONVERGED : sv::COL_MAXIT;
    }
  }

  // Y = Qinv X on interleaved blocks (u part only is meaningful)
  void qinv(cbx_handle* h, Mme& m, int ncols) {
    prepare(h, m, 1.0, false);
    auto op = make_view<double>(m, dinv64.p);
    matvec<double, S>(h, op, w64, Xi.p, Y64.p, 1.0, 0, nullptr, nullptr, nullptr, false, ncols);
  }
};

template <int S>
static Solver<S>& solver_for(Mme& m) {
  constexpr int idx = S == 1 ? 0 : S == 2 ? 1 : S == 4 ? 2 : S == 8 ? 3 : S == 16 ? 4 : S == 32 ? 5 : S == 64 ? 6 : 7;
  if (!m.solvers[idx]) m.solvers[idx].reset(new Solver<S>());
  return *static_cast<Solver<S>*>(m.solvers[idx].get());
}

static int block_width(int ncols, int max_w = 32) {
  int S = 1;
  while (S < ncols && S < max_w) S <<= 1;
  return S;
}

template <int S>
static void solve_chunk(cbx_handle* h, Mme& m, double lam, int nc, const double* B_cm, double* X_cm, bool use_x0,
                        double tol, int maxit, int abs_tol, int precision, PcgResult& r, const double* r_prev,
                        double dlam, double* r_out) {
  Solver<S>& sv_ = solver_for<S>(m);
  sv_.prepare(h, m, lam, precision != 0);
  cudaStream_t s = h->stream;
  const int64_t n = m.dim * S;
  k_to_inter<<<grid_for(n, 256, 4 * h->num_sms), 256, 0, s>>>(B_cm, m.dim, nc, S, sv_.Bi.p);
  h->launched("k_to_inter");
  if (use_x0) {
    k_to_inter<<<grid_for(n, 256, 4 * h->num_sms), 256, 0, s>>>(X_cm, m.dim, nc, S, sv_.Xi.p);
    h->launched("k_to_inter");
  }
  const bool have_r0 = use_x0 && precision != 0 && r_prev;
  if (have_r0) {
    k_to_inter<<<grid_for(n, 256, 4 * h->num_sms), 256, 0, s>>>(r_prev, m.dim, nc, S, sv_.R64.p);
    h->launched("k_to_inter");
  }
  sv_.solve(h, m, lam, nc, use_x0, tol, maxit, abs_tol, precision, r, have_r0, dlam);
  k_from_inter<<<grid_for(m.dim * nc, 256, 4 * h->num_sms), 256, 0, s>>>(sv_.Xi.p, m.dim, nc, S, X_cm);
  h->launched("k_from_inter");
  if (r_out && precision != 0) {
    k_from_inter<<<grid_for(m.dim * nc, 256, 4 * h->num_sms), 256, 0, s>>>(sv_.R64.p, m.dim, nc, S, r_out);
    h->launched("k_from_inter");
  }
}

void pcg_solve(cbx_handle* h, double lam, int ncols, const double* B_cm, double* X_cm, bool use_x0, double tol,
               int maxit, int abs_tol, int precision, PcgResult& res, const ResidCarry* carry) {
  CBX_REQUIRE(h->mme, CBX_ERR_STATE, "no mixed-model equations on this handle (cbx_mme_create)");
  Mme& m = *h->mme;
  CBX_REQUIRE(m.has_dense || m.has_sparse, CBX_ERR_STATE, "Qinv not set (cbx_mme_set_qinv_*)");
  res = PcgResult{};
  // Mixed precision takes up to 64 columns per block, or up to 80 in a
  // 128-wide block when there are more than 64: its PCG bulk reads the FP32
  // block once per iteration for all of them (the tensor-core product takes at
  // most 80 populated columns), and the FP64-class refinement products run on
  // the populated columns only.  The FP64 solver's product is FP64-bound, so it
  // stays at 32.
  const int chunk = precision != 0 ? (ncols > 64 ? 80 : 64) : 32;
  for (int c0 = 0; c0 < ncols; c0 += chunk) {
    const int nc = std::min(chunk, ncols - c0);
    PcgResult r;
    const double* B = B_cm + (int64_t)c0 * m.dim;
    double* X = X_cm + (int64_t)c0 * m.dim;
    const double* rp = carry && carry->r_prev ? carry->r_prev + (int64_t)c0 * m.dim : nullptr;
    double* ro = carry && carry->r_out ? carry->r_out + (int64_t)c0 * m.dim : nullptr;
    const double dl = carry ? carry->dlam : 0.0;
#define CBX_CHUNK(W) solve_chunk<W>(h, m, lam, nc, B, X, use_x0, tol, maxit, abs_tol, precision, r, rp, dl, ro)
    switch (block_width(nc, 128)) {
      case 1: CBX_CHUNK(1); break;
      case 2: CBX_CHUNK(2); break;
      case 4: CBX_CHUNK(4); break;
      case 8: CBX_CHUNK(8); break;
      case 16: CBX_CHUNK(16); break;
      case 32: CBX_CHUNK(32); break;
      case 64: CBX_CHUNK(64); break;
      default: CBX_CHUNK(128); break;
    }
#undef CBX_CHUNK
    res.iters.insert(res.iters.end(), r.iters.begin(), r.iters.end());
    res.status.insert(res.status.end(), r.status.begin(), r.status.end());
    res.relres.insert(res.relres.end(), r.relres.begin(), r.relres.end());
    res.refinements += r.refinements;
    res.matvecs += r.matvecs;
  }
}

template <int S>
static void qinv_chunk(cbx_handle* h, Mme& m, int nc, const double* X_cm, double* Y_cm) {
  Solver<S>& sv_ = solver_for<S>(m);
  sv_.prepare(h, m, 1.0, false);
  cudaStream_t s = h->stream;
  const int64_t n = m.dim * S;
  // place the q-vectors in rows [p, dim) of a dim x nc column-major scratch
  DevBuf<double>& tmp = m.io_x;
  tmp.resize((size_t)m.dim * nc);
  CBX_CUDA(cudaMemsetAsync(tmp.p, 0, (size_t)m.dim * nc * sizeof(double), s));
  CBX_CUDA(cudaMemcpy2DAsync(tmp.p + m.p, m.dim * sizeof(double), X_cm, m.q * sizeof(double), m.q * sizeof(double),
                             nc, cudaMemcpyDeviceToDevice, s));
  k_to_inter<<<grid_for(n, 256, 4 * h->num_sms), 256, 0, s>>>(tmp.p, m.dim, nc, S, sv_.Xi.p);
  h->launched("k_to_inter");
  sv_.qinv(h, m, nc);
  k_from_inter<<<grid_for(m.dim * nc, 256, 4 * h->num_sms), 256, 0, s>>>(sv_.Y64.p, m.dim, nc, S, tmp.p);
  h->launched("k_from_inter");
  CBX_CUDA(cudaMemcpy2DAsync(Y_cm, m.q * sizeof(double), tmp.p + m.p, m.dim * sizeof(double), m.q * sizeof(double),
                             nc, cudaMemcpyDeviceToDevice, s));
}

void qinv_apply(cbx_handle* h, int ncols, const double* X_cm, double* Y_cm) {
  CBX_REQUIRE(h->mme, CBX_ERR_STATE, "no mixed-model equations on this handle");
  Mme& m = *h->mme;
  for (int c0 = 0; c0 < ncols; c0 += 32) {
    const int nc = std::min(32, ncols - c0);
    const double* X = X_cm + (int64_t)c0 * m.q;
    double* Y = Y_cm + (int64_t)c0 * m.q;
    switch (block_width(nc)) {
      case 1: qinv_chunk<1>(h, m, nc, X, Y); break;
      case 2: qinv_chunk<2>(h, m, nc, X, Y); break;
      case 4: qinv_chunk<4>(h, m, nc, X, Y); break;
      case 8: qinv_chunk<8>(h, m, nc, X, Y); break;
      case 16: qinv_chunk<16>(h, m, nc, X, Y); break;
      default: qinv_chunk<32>(h, m, nc, X, Y); break;
    }
  }
}

// Y[c * q + u] = ((B - R)[c * dim + p + u] - (D X)[c * dim + p + u]) / lam: the
// random rows of lam [0; Qinv u] = (b - r) - W'W x for a solution x whose true
// residual r = b - A x is known.
__global__ void k_qinv_from_solution(const int32_t* __restrict__ Dptr, const int32_t* __restrict__ Dcol,
                                     const double* __restrict__ Dval, int64_t p, int64_t q, int64_t dim, int ncols,
                                     const double* __restrict__ B, const double* __restrict__ X,
                                     const double* __restrict__ R, double inv_lam, double* __restrict__ Y) {
  const int64_t total = q * ncols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / q, u = idx - c * q, i = p + u;
    const double* x = X + c * dim;
    double t = 0.0;
    for (int32_t j = Dptr[i]; j < Dptr[i + 1]; ++j) t += Dval[j] * x[Dcol[j]];
    Y[idx] = ((B[c * dim + i] - R[c * dim + i]) - t) * inv_lam;
  }
}

void qinv_from_solution(cbx_handle* h, double lam, int ncols, const double* B_cm, const double* X_cm,
                        const double* R_cm, double* Y_cm) {
  CBX_REQUIRE(h->mme, CBX_ERR_STATE, "no mixed-model equations on this handle");
  CBX_REQUIRE(lam > 0, CBX_ERR_ARG, "lambda must be positive");
  Mme& m = *h->mme;
  k_qinv_from_solution<<<grid_for(m.q * ncols, 256, 4 * h->num_sms), 256, 0, h->stream>>>(
      m.D64.ptr.p, m.D64.col.p, m.D64.val.p, m.p, m.q, m.dim, ncols, B_cm, X_cm, R_cm, 1.0 / lam, Y_cm);
  h->launched("k_qinv_from_solution");
}

double record_residual(cbx_handle* h, const double* sol_dev, double* e_dev) {
  Mme& m = *h->mme;
  cudaStream_t s = h->stream;
  const unsigned g = grid_for(m.n_rec, sv::NT, 2 * h->num_sms);
  DevBuf<double> part;
  part.resize(g);
  sv::k_resid_records<<<g, sv::NT, 0, s>>>(m.n_rec, m.p, m.y.p, m.aid.p, m.q, m.x_ptr.p, m.x_col.p, m.x_val.p,
                                           sol_dev, e_dev, part.p);
  h->launched("k_resid_records");
  std::vector<double> ph(g);
  CBX_CUDA(cudaMemcpyAsync(ph.data(), part.p, g * sizeof(double), cudaMemcpyDeviceToHost, s));
  CBX_CUDA(cudaStreamSynchronize(s));
  double t = 0;
  for (double v : ph) t += v;
  return t;
}

// ---------------------------------------------------------------------------
// host assembly helpers
__global__ void k_d2f(const double* __restrict__ a, int64_t n, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// A CSR straight from the caller's arrays (page-locked ones are copied by DMA)
// into its FP64 copy, and on the device into the FP32 copy.
static void upload_csr_pair(cbx_handle* h, int64_t rows, const std::vector<int32_t>& ptr, const int32_t* col,
                            const double* val, Csr<double>& d, Csr<float>& f) {
  cudaStream_t s = h->stream;
  const int64_t nnz = ptr[rows];
  d.rows = (int32_t)rows;
  d.nnz = nnz;
  f.rows = (int32_t)rows;
  f.nnz = nnz;
  d.ptr.resize(rows + 1);
  f.ptr.resize(rows + 1);
  d.col.resize(std::max<int64_t>(nnz, 1));
  f.col.resize(std::max<int64_t>(nnz, 1));
  d.val.resize(std::max<int64_t>(nnz, 1));
  f.val.resize(std::max<int64_t>(nnz, 1));
  CBX_CUDA(cudaMemcpyAsync(d.ptr.p, ptr.data(), (rows + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  CBX_CUDA(cudaMemcpyAsync(f.ptr.p, d.ptr.p, (rows + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  if (nnz > 0) {
    CBX_CUDA(cudaMemcpyAsync(d.col.p, col, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(f.col.p, d.col.p, nnz * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(d.val.p, val, nnz * sizeof(double), cudaMemcpyHostToDevice, s));
    k_d2f<<<grid_for(nnz, 256, 4 * h->num_sms), 256, 0, s>>>(d.val.p, nnz, f.val.p);
    h->launched("k_d2f");
  }
  CBX_CUDA(cudaStreamSynchronize(s));  // the caller's arrays are read before return
}


// W'W as CSR and W'y from the records (mme_builder.cpp:107-176, 321-387) on
// host threads: every record emits its triplets (fixed x fixed pairs, fixed x
// animal, animal x animal) in record order; the threads take contiguous record
// ranges, count their triplets per row, and place them at offsets that keep the
// record order within each row, so each row's entries come out as from one
// sequential pass (a stable counting sort).  Each row is then sorted stably by
// column and its duplicates summed in that order, so W'W does not depend on the
// number of threads.
struct WtW {
  std::vector<int32_t> ptr, col;
  std::vector<double> val;
};

// The records' checks, W'y and y'y (mme_builder.cpp:321-387), in record order.
static void records_rhs(int64_t n_rec, int64_t p, int64_t q, const double* y, const int32_t* aid,
                        const int64_t* fx_ptr, const int32_t* fx_col, const double* fx_val, std::vector<double>& rhs,
                        double& yty) {
  rhs.assign(p + q, 0.0);
  yty = 0.0;
  for (int64_t i = 0; i < n_rec; ++i) {
    CBX_REQUIRE(fx_ptr[i + 1] >= fx_ptr[i], CBX_ERR_ARG, "fx_ptr not monotone");
    CBX_REQUIRE(std::isfinite(y[i]), CBX_ERR_NONFINITE, "non-finite phenotype");
    for (int64_t a = fx_ptr[i]; a < fx_ptr[i + 1]; ++a) {
      CBX_REQUIRE(fx_col[a] >= 0 && fx_col[a] < p, CBX_ERR_ARG, "fixed-effect column out of range");
      rhs[fx_col[a]] += fx_val[a] * y[i];
    }
    const int32_t an = aid[i];
    if (an > 0 && an <= q) rhs[p + an - 1] += y[i];
    yty += y[i] * y[i];
  }
  CBX_REQUIRE(fx_ptr[n_rec] < (int64_t)INT32_MAX, CBX_ERR_UNSUPPORTED, "more than 2^31 fixed-effect entries");
}

// W'W on the device from the uploaded records (wtw.cu); the host assembly below
// builds the same CSR bit for bit and runs when the environment sets CBX_WTW_HOST=1.
void wtw_device(cbx_handle* h, Mme& m, std::vector<int32_t>& ptr_fix, std::vector<double>& A11);
static bool use_host_wtw() { return env_int("CBX_WTW_HOST", 0) != 0; }

static void assemble_wtw(int64_t n_rec, int64_t p, int64_t q, const double* y, const int32_t* aid,
                         const int64_t* fx_ptr, const int32_t* fx_col, const double* fx_val, WtW& out) {
  const int64_t dim = p + q;
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int T = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::min(hw, 16), n_rec / 2000));
  struct Part {
    int64_t r0 = 0, r1 = 0;
    std::vector<int64_t> cnt;   // triplets per row, then the running placement offsets
    int err = CBX_OK;
    const char* what = nullptr;
  };
  std::vector<Part> part(T);
  for (int t = 0; t < T; ++t) {
    part[t].r0 = n_rec * t / T;
    part[t].r1 = n_rec * (t + 1) / T;
  }
  // fn(t) on T threads; an exception in a thread is rethrown after the join
  auto run = [&](auto&& fn) {
    std::vector<std::exception_ptr> fail(T);
    auto body = [&](int t) {
      try {
        fn(t);
      } catch (...) {
        fail[t] = std::current_exception();
      }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T; ++t) pool.emplace_back(body, t);
    body(0);
    for (auto& th : pool) th.join();
    for (auto& f : fail)
      if (f) std::rethrow_exception(f);
  };
  // the triplets of record i, in order, to emit(row, col, value)
  auto record = [&](int64_t i, auto&& emit) {
    const int64_t a0 = fx_ptr[i], a1 = fx_ptr[i + 1];
    for (int64_t a = a0; a < a1; ++a)
      for (int64_t b = a; b < a1; ++b) {
        const double v = fx_val[a] * fx_val[b];
        emit(fx_col[a], fx_col[b], v);
        if (fx_col[a] != fx_col[b]) emit(fx_col[b], fx_col[a], v);
      }
    const int32_t an = aid[i];
    if (an > 0 && an <= q) {
      const int64_t ck = p + an - 1;
      for (int64_t a = a0; a < a1; ++a) {
        emit(fx_col[a], ck, fx_val[a]);
        emit(ck, (int64_t)fx_col[a], fx_val[a]);
      }
      emit(ck, ck, 1.0);
    }
  };
  // 1. per thread: checks and triplet counts per row
  run([&](int t) {
    Part& pt = part[t];
    pt.cnt.assign(dim, 0);
    for (int64_t i = pt.r0; i < pt.r1; ++i) {
      if (fx_ptr[i + 1] < fx_ptr[i]) { pt.err = CBX_ERR_ARG; pt.what = "fx_ptr not monotone"; return; }
      if (!std::isfinite(y[i])) { pt.err = CBX_ERR_NONFINITE; pt.what = "non-finite phenotype"; return; }
      for (int64_t a = fx_ptr[i]; a < fx_ptr[i + 1]; ++a) {
        if (fx_col[a] < 0 || fx_col[a] >= p) {
          pt.err = CBX_ERR_ARG;
          pt.what = "fixed-effect column out of range";
          return;
        }
      }
      record(i, [&](int64_t r, int64_t, double) { pt.cnt[r]++; });
    }
  });
  for (const Part& pt : part) CBX_REQUIRE(pt.err == CBX_OK, pt.err, pt.what);
  // 2. row starts; each thread's offsets in a row follow the earlier threads'
  // (row ranges in parallel: offsets within the range, then the range bases)
  std::vector<int64_t> start(dim + 1, 0), base(T + 1, 0);
  run([&](int t) {
    int64_t o = 0;
    for (int64_t r = dim * t / T; r < dim * (t + 1) / T; ++r) {
      start[r] = o;
      for (int k = 0; k < T; ++k) {
        const int64_t c = part[k].cnt[r];
        part[k].cnt[r] = o;
        o += c;
      }
    }
    base[t + 1] = o;
  });
  for (int t = 0; t < T; ++t) base[t + 1] += base[t];
  start[dim] = base[T];
  run([&](int t) {
    const int64_t b = base[t];
    for (int64_t r = dim * t / T; r < dim * (t + 1) / T; ++r) {
      start[r] += b;
      for (int k = 0; k < T; ++k) part[k].cnt[r] += b;
    }
  });
  struct Ent {
    int32_t c;
    double v;
  };
  std::unique_ptr<Ent[]> ent(new Ent[(size_t)std::max<int64_t>(start[dim], 1)]);
  // 3. placement in record order
  run([&](int t) {
    Part& pt = part[t];
    for (int64_t i = pt.r0; i < pt.r1; ++i)
      record(i, [&](int64_t r, int64_t c, double v) { ent[pt.cnt[r]++] = Ent{(int32_t)c, v}; });
  });
  // 4. each row's entries sorted stably by column (insertion sort for short rows,
  // an LSD radix sort on 8-bit column digits for long ones), then each run of
  // equal columns summed in order from 0.0 and the row compacted at its start:
  // the result of one stable sort by (row, column) and a sequential sum.  The
  // threads take row ranges of about equal numbers of entries.
  std::vector<int64_t> rb(T + 1, dim);
  rb[0] = 0;
  for (int t = 1; t < T; ++t)
    rb[t] = std::lower_bound(start.begin(), start.end(), start[dim] * t / T) - start.begin();
  for (int t = 1; t <= T; ++t) rb[t] = std::min(dim, std::max(rb[t], rb[t - 1]));
  std::vector<int32_t> uniq(dim, 0);
  int key_bits = 1;
  while (key_bits < 31 && (int64_t(1) << key_bits) < dim) ++key_bits;
  run([&](int t) {
    std::vector<Ent> tmp;
    for (int64_t r = rb[t]; r < rb[t + 1]; ++r) {
      const int64_t e0 = start[r], e1 = start[r + 1], n = e1 - e0;
      if (n <= 48) {
        for (int64_t e = e0 + 1; e < e1; ++e) {
          const Ent x = ent[e];
          int64_t k = e;
          for (; k > e0 && ent[k - 1].c > x.c; --k) ent[k] = ent[k - 1];
          ent[k] = x;
        }
      } else {
        if ((int64_t)tmp.size() < n) tmp.resize(n);
        Ent* a = &ent[e0];
        Ent* b = tmp.data();
        for (int sh = 0; sh < key_bits; sh += 8) {
          int64_t cnt[257] = {0};
          for (int64_t i = 0; i < n; ++i) cnt[((a[i].c >> sh) & 255) + 1]++;
          if (cnt[((a[0].c >> sh) & 255) + 1] == n) continue;  // one digit value: already in order
          for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
          for (int64_t i = 0; i < n; ++i) b[cnt[(a[i].c >> sh) & 255]++] = a[i];
          std::swap(a, b);
        }
        if (a != &ent[e0]) std::copy(a, a + n, &ent[e0]);
      }
      int32_t u = 0;
      for (int64_t e = e0; e < e1;) {
        const int32_t c = ent[e].c;
        double v = 0.0;
        while (e < e1 && ent[e].c == c) v += ent[e++].v;
        ent[e0 + u++] = Ent{c, v};
      }
      uniq[r] = u;
    }
  });
  int64_t nnz = 0;
  for (int64_t r = 0; r < dim; ++r) nnz += uniq[r];
  CBX_REQUIRE(nnz < (int64_t)INT32_MAX, CBX_ERR_UNSUPPORTED, "W'W has more than 2^31 entries");
  out.ptr.assign(dim + 1, 0);
  for (int64_t r = 0; r < dim; ++r) out.ptr[r + 1] = out.ptr[r] + uniq[r];
  out.col.resize(out.ptr[dim]);
  out.val.resize(out.ptr[dim]);
  // 5. the compacted rows into the CSR arrays
  run([&](int t) {
    for (int64_t r = rb[t]; r < rb[t + 1]; ++r)
      for (int32_t k = 0; k < uniq[r]; ++k) {
        out.col[out.ptr[r] + k] = ent[start[r] + k].c;
        out.val[out.ptr[r] + k] = ent[start[r] + k].v;
      }
  });
}

}  // namespace cbx

using namespace cbx;

extern "C" int cbx_mme_create(cbx_handle* h, int64_t n_rec, int64_t p, int64_t q, const double* y,
                              const int32_t* aid, const int64_t* fx_ptr, const int32_t* fx_col,
                              const double* fx_val) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(n_rec > 0 && p >= 0 && q > 0, CBX_ERR_ARG, "n_rec, q must be positive and p >= 0");
    CBX_REQUIRE(y && aid && fx_ptr, CBX_ERR_ARG, "null record arrays");
    CBX_REQUIRE(fx_ptr[0] == 0, CBX_ERR_ARG, "fx_ptr[0] must be 0");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    auto m = std::make_unique<Mme>();
    m->n_rec = n_rec; m->p = p; m->q = q; m->dim = p + q;
    const int64_t dim = p + q;
    // checks, W'y and y'y on the host (record order)
    std::vector<double> rhs;
    double yty = 0.0;
    records_rhs(n_rec, p, q, y, aid, fx_ptr, fx_col, fx_val, rhs, yty);
    // records
    m->y.resize(n_rec);
    CBX_CUDA(cudaMemcpyAsync(m->y.p, y, n_rec * sizeof(double), cudaMemcpyHostToDevice, s));
    m->aid.resize(n_rec);
    CBX_CUDA(cudaMemcpyAsync(m->aid.p, aid, n_rec * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    std::vector<int32_t> xp(n_rec + 1);
    for (int64_t i = 0; i <= n_rec; ++i) xp[i] = (int32_t)fx_ptr[i];
    const int64_t nx = fx_ptr[n_rec];
    m->x_ptr.resize(n_rec + 1);
    CBX_CUDA(cudaMemcpyAsync(m->x_ptr.p, xp.data(), (n_rec + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    m->x_col.resize(std::max<int64_t>(nx, 1));
    m->x_val.resize(std::max<int64_t>(nx, 1));
    if (nx > 0) {
      CBX_CUDA(cudaMemcpyAsync(m->x_col.p, fx_col, nx * sizeof(int32_t), cudaMemcpyHostToDevice, s));
      CBX_CUDA(cudaMemcpyAsync(m->x_val.p, fx_val, nx * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    // W'W (mme_builder.cpp:107-176): its CSR, diagonal, fixed block X'X and the
    // row pointers of the fixed rows
    std::vector<int32_t> ptr;
    std::vector<double> A11;
    if (use_host_wtw()) {
      WtW wtw;
      assemble_wtw(n_rec, p, q, y, aid, fx_ptr, fx_col, fx_val, wtw);
      std::vector<double> diag(dim, 0.0);
      A11.assign((size_t)p * p, 0.0);
      for (int64_t i = 0; i < dim; ++i)
        for (int32_t j = wtw.ptr[i]; j < wtw.ptr[i + 1]; ++j) {
          if (wtw.col[j] == i) diag[i] = wtw.val[j];
          if (i < p && wtw.col[j] < p) A11[i * p + wtw.col[j]] = wtw.val[j];
        }
      upload_csr_pair(h, dim, wtw.ptr, wtw.col.data(), wtw.val.data(), m->D64, m->D32);
      m->diagD.resize(dim);
      CBX_CUDA(cudaMemcpyAsync(m->diagD.p, diag.data(), dim * sizeof(double), cudaMemcpyHostToDevice, s));
      ptr.assign(wtw.ptr.begin(), wtw.ptr.begin() + p + 1);
    } else {
      wtw_device(h, *m, ptr, A11);
    }
    {
      // segments of the fixed-effect rows (sv::FIX_SEG entries at most)
      std::vector<int32_t> srow, slo, shi, sptr(p + 1, 0);
      for (int64_t f = 0; f < p; ++f) {
        for (int32_t j = ptr[f]; j < ptr[f + 1]; j += sv::FIX_SEG) {
          srow.push_back((int32_t)f);
          slo.push_back(j);
          shi.push_back(std::min<int32_t>(ptr[f + 1], j + sv::FIX_SEG));
        }
        sptr[f + 1] = (int32_t)srow.size();
      }
      m->nseg = (int32_t)srow.size();
      m->fix_seg_ptr.resize(p + 1);
      CBX_CUDA(cudaMemcpyAsync(m->fix_seg_ptr.p, sptr.data(), (p + 1) * 4, cudaMemcpyHostToDevice, s));
      if (m->nseg > 0) {
        m->seg_row.resize(m->nseg); m->seg_lo.resize(m->nseg); m->seg_hi.resize(m->nseg);
        CBX_CUDA(cudaMemcpyAsync(m->seg_row.p, srow.data(), m->nseg * 4, cudaMemcpyHostToDevice, s));
        CBX_CUDA(cudaMemcpyAsync(m->seg_lo.p, slo.data(), m->nseg * 4, cudaMemcpyHostToDevice, s));
        CBX_CUDA(cudaMemcpyAsync(m->seg_hi.p, shi.data(), m->nseg * 4, cudaMemcpyHostToDevice, s));
      }
      CBX_CUDA(cudaStreamSynchronize(s));
    }
    m->rhs.resize(dim);
    CBX_CUDA(cudaMemcpyAsync(m->rhs.p, rhs.data(), dim * sizeof(double), cudaMemcpyHostToDevice, s));
    // block-Jacobi fixed block: (X'X + ridge I)^-1, ridge = max(1e-8 max|diag|, 1e-6) (pcg_solver.h:78-85)
    if (p > 0) {
      double maxd = 0.0;
      for (int64_t i = 0; i < p; ++i) maxd = std::max(maxd, std::fabs(A11[i * p + i]));
      const double ridge = std::max(1e-8 * maxd, 1e-6);
      std::vector<double> M(A11);
      for (int64_t i = 0; i < p; ++i) M[i * p + i] += ridge;
      bool diagonal = true;
      for (int64_t i = 0; i < p && diagonal; ++i)
        for (int64_t j = 0; j < p; ++j)
          if (j != i && M[i * p + j] != 0.0) { diagonal = false; break; }
      m->A11inv64.resize((size_t)p * p);
      bool ok = true;
      if (diagonal) {
        // one fixed factor: X'X is diagonal and so is its inverse
        for (int64_t i = 0; i < p; ++i) {
          ok = ok && M[i * p + i] > 0.0;
          M[i * p + i] = 1.0 / M[i * p + i];
        }
        if (ok)
          CBX_CUDA(cudaMemcpyAsync(m->A11inv64.p, M.data(), M.size() * sizeof(double), cudaMemcpyHostToDevice, s));
      } else {
        // Cholesky inverse on the device (cuSOLVER potrf / potri)
        CBX_CUDA(cudaMemcpyAsync(m->A11inv64.p, M.data(), M.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        ok = chol_inverse_device(h, m->A11inv64.p, p);
      }
      if (!ok) {
        // reference fallback: diagonal scaling of the fixed block (pcg_solver.h:108-116)
        M.assign((size_t)p * p, 0.0);
        for (int64_t i = 0; i < p; ++i) {
          const double d = A11[i * p + i];
          M[i * p + i] = std::fabs(d) > 1e-14 ? 1.0 / d : 1.0;
        }
        CBX_CUDA(cudaMemcpyAsync(m->A11inv64.p, M.data(), M.size() * sizeof(double), cudaMemcpyHostToDevice, s));
      }
      m->A11inv32.resize((size_t)p * p);
      k_convert<double, float><<<grid_for(p * p, 256, 1024), 256, 0, s>>>(m->A11inv64.p, m->A11inv32.p, p * p);
      h->launched("k_convert");
    }
    m->y_host.assign(y, y + n_rec);
    m->yty = yty;
    m->aid_host.assign(aid, aid + n_rec);
    m->xp_host = xp;
    m->xc_host.assign(fx_col, fx_col + nx);
    m->xv_host.assign(fx_val, fx_val + nx);
    m->rhs_host = rhs;
    CBX_CUDA(cudaStreamSynchronize(s));
    if (h->mme) {
      // The device buffers whose sizes follow the shapes go to the new MME, whose
      // set-up and solves size-check and rewrite them before use: a rebuild of
      // the same shape (a new set of records) then neither frees nor allocates
      // the dense planes (several GB) or the solver workspaces.
      Mme& o = *h->mme;
      CBX_CUDA(cudaStreamSynchronize(s));
      m->Qd64 = std::move(o.Qd64);
      m->Qd32 = std::move(o.Qd32);
      m->Qlo32 = std::move(o.Qlo32);
      m->Qbf = std::move(o.Qbf);
      m->fx_rowexp = std::move(o.fx_rowexp);
      m->fx_bdig = std::move(o.fx_bdig);
      m->fx_cexp = std::move(o.fx_cexp);
      m->fx_part = std::move(o.fx_part);
      // the copies stay tied to their source block (upload_dense keeps them when
      // the new MME takes the same, unchanged block)
      m->ng = o.ng;
      m->ld = o.ld;
      m->qshift = o.qshift;
      m->fx_rows_ok = o.fx_rows_ok;
      m->planes_src = o.planes_src;
      m->planes_gen = o.planes_gen;
      if (o.dim == m->dim)
        for (int i = 0; i < 8; ++i)
          if (o.solvers[i]) {
            o.solvers[i]->rebind();
            m->solvers[i] = std::move(o.solvers[i]);
          }
      if (h->keep_warm && o.dim == m->dim && o.p == m->p && o.q == m->q) {
        // the last data and probe solutions start the new MME's solves; the probe
        // right-hand sides [0; z_j] depend only on the seed, p and q (column 0,
        // W'y, is rewritten by every iteration); residual carries and the
        // forward state belong to the old operator and are not kept
        m->last_solution = std::move(o.last_solution);
        m->has_last = o.has_last;
        m->last_lam = o.last_lam;
        m->probe_x = std::move(o.probe_x);
        m->probe_r = std::move(o.probe_r);
        m->probe_lam = o.probe_lam;
        m->probe_r_ok.assign(o.probe_r_ok.size(), 0);
        m->probe_seed = o.probe_seed;
        m->em_B = std::move(o.em_B);
        m->probe_have = o.probe_have;
        m->em_B_seed = o.em_B_seed;
        m->probe_cap = o.probe_cap;
        m->probe_zv = std::move(o.probe_zv);
      }
    }
    h->mme = std::move(m);
  });
}

// The dense block on the device: the FP64 copy (pitch ld) and the shifted
// low-precision copies (see Mme::qshift).  The shift
// is the mean off-diagonal entry, summed in a fixed order.
// gen >= 0: src is a device block of the handle at that generation; an MME
// whose copies were made from it keeps them.
static void upload_dense(cbx_handle* h, Mme& m, const double* src, int64_t ng, int64_t gen = -1) {
  cudaStream_t s = h->stream;
  if (gen >= 0 && m.planes_src == src && m.planes_gen == gen && m.ng == ng && m.Qd64.p && m.Qd32.p &&
      m.Qlo32.p && (m.Qbf.p != nullptr) == (use_bf16() && m.ld % 8 == 0))
    return;
  m.planes_src = nullptr;
  m.planes_gen = -1;
  m.ng = ng;
  m.ld = (ng + 3) / 4 * 4;
  m.Qd64.resize((size_t)ng * m.ld);
  k_pitch_copy<double><<<grid_for(ng * m.ld, 256, 8 * h->num_sms), 256, 0, s>>>(src, ng, m.ld, m.Qd64.p);
  h->launched("k_pitch_copy");
  double shift = 0.0;
  if (ng > 1) {
    const unsigned g = (unsigned)(4 * h->num_sms);
    DevBuf<double> part;
    part.resize(g);
    k_offdiag_part<<<g, 256, 0, s>>>(src, ng, part.p);
    h->launched("k_offdiag_part");
    std::vector<double> ph(g);
    CBX_CUDA(cudaMemcpyAsync(ph.data(), part.p, g * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    double t = 0.0;
    for (double v : ph) t += v;
    shift = t / ((double)ng * (double)(ng - 1));
  }
  m.qshift = std::isfinite(shift) ? shift : 0.0;
  m.Qd32.resize((size_t)ng * m.ld);
  m.Qlo32.resize((size_t)ng * m.ld);
  k_lowp_block<<<grid_for(ng * m.ld, 256, 8 * h->num_sms), 256, 0, s>>>(src, ng, m.ld, m.qshift, m.Qd32.p,
                                                                       m.Qlo32.p);
  h->launched("k_lowp_block");
  m.fx_rows_ok = false;
  if (use_bf16() && m.ld % 8 == 0) {
    m.Qbf.resize((size_t)ng * m.ld);
    dense_bf_block(h, m.Qd64.p, ng, m.ld, m.qshift, m.Qbf.p);
  } else {
    m.Qbf.release();
  }
  if (gen >= 0) {
    m.planes_src = src;
    m.planes_gen = gen;
  }
}

// Dense Qinv (q x q, symmetric, row- or column-major alike).  Qinv == NULL uses
// the matrix left on the device by cbx_invert_psd.
extern "C" int cbx_mme_set_qinv_dense(cbx_handle* h, const double* Qinv, int64_t q) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create first");
    Mme& m = *h->mme;
    CBX_REQUIRE(q == m.q, CBX_ERR_ARG, "Qinv order does not match q");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const double* src = nullptr;
    DevBuf<double> tmp;
    if (Qinv) {
      tmp.resize((size_t)q * q);
      CBX_CUDA(cudaMemcpyAsync(tmp.p, Qinv, (size_t)q * q * sizeof(double), cudaMemcpyHostToDevice, s));
      src = tmp.p;
    } else {
      CBX_REQUIRE(h->Ginv.p && h->Ginv_n == q, CBX_ERR_STATE, "no device G inverse of matching order");
      src = h->Ginv.p;
    }
    upload_dense(h, m, src, q, Qinv ? -1 : h->Ginv_gen);
    std::vector<int32_t> idm(q);
    for (int64_t i = 0; i < q; ++i) idm[i] = (int32_t)i;
    m.gmap.resize(q);
    m.ginv.resize(q);
    CBX_CUDA(cudaMemcpyAsync(m.gmap.p, idm.data(), q * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(m.ginv.p, idm.data(), q * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    // diag(Qinv)
    m.diagQ.resize(q);
    CBX_CUDA(cudaMemcpy2DAsync(m.diagQ.p, sizeof(double), src, (q + 1) * sizeof(double), sizeof(double), q,
                               cudaMemcpyDeviceToDevice, s));
    m.has_dense = true;
    m.has_sparse = false;
    m.drop_carry(h->keep_warm);
    CBX_CUDA(cudaStreamSynchronize(s));
    for (auto& sp : m.solvers)
      if (sp) sp->rebind();  // workspaces kept; everything derived from the operator recomputed
  });
}

// Split Qinv = A (CSR, q x q) + S Gd S^T with Gd dense ng x ng (row-major) and
// gmap[k] the u-index of dense row k (SplitMatrixAdapter::operator*).  Gd ==
// NULL with ng > 0 uses the block cbx_ssgblup_qinv left on the device.
extern "C" int cbx_mme_set_qinv_split(cbx_handle* h, const int64_t* a_ptr, const int32_t* a_col,
                                      const double* a_val, const double* Gd, int64_t ng,
                                      const int32_t* gmap) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create first");
    Mme& m = *h->mme;
    CBX_REQUIRE(a_ptr && a_ptr[0] == 0, CBX_ERR_ARG, "bad A^-1 CSR");
    CBX_REQUIRE(ng >= 0 && ng <= m.q, CBX_ERR_ARG, "bad dense block order");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const int64_t q = m.q;
    CBX_REQUIRE(a_ptr[q] < (int64_t)INT32_MAX, CBX_ERR_UNSUPPORTED, "A^-1 has more than 2^31 entries");
    std::vector<int32_t> ptr(q + 1);
    std::vector<double> diag(q, 0.0);
    for (int64_t i = 0; i < q; ++i) {
      CBX_REQUIRE(a_ptr[i + 1] >= a_ptr[i], CBX_ERR_ARG, "A^-1 row pointers not monotone");
      ptr[i] = (int32_t)a_ptr[i];
      for (int64_t j = a_ptr[i]; j < a_ptr[i + 1]; ++j) {
        CBX_REQUIRE(a_col[j] >= 0 && a_col[j] < q, CBX_ERR_ARG, "A^-1 column out of range");
        if (a_col[j] == i) diag[i] += a_val[j];
      }
    }
    ptr[q] = (int32_t)a_ptr[q];
    upload_csr_pair(h, q, ptr, a_col, a_val, m.Qs64, m.Qs32);
    m.has_sparse = true;
    m.has_dense = ng > 0;
    m.drop_carry(h->keep_warm);
    if (ng > 0) {
      CBX_REQUIRE(gmap, CBX_ERR_ARG, "genotyped map missing");
      CBX_REQUIRE(Gd || (h->Hd.p && h->Hd_n == ng), CBX_ERR_STATE,
                  "no dense block: pass Gd or run cbx_ssgblup_qinv with this ng first");
      std::vector<int32_t> inv(q, -1);
      for (int64_t k = 0; k < ng; ++k) {
        CBX_REQUIRE(gmap[k] >= 0 && gmap[k] < q, CBX_ERR_ARG, "genotyped map out of range");
        CBX_REQUIRE(inv[gmap[k]] < 0, CBX_ERR_ARG, "genotyped map has duplicates");
        inv[gmap[k]] = (int32_t)k;
      }
      DevBuf<double> tmp;
      const double* src = h->Hd.p;
      if (Gd) {
        tmp.resize((size_t)ng * ng);
        CBX_CUDA(cudaMemcpyAsync(tmp.p, Gd, (size_t)ng * ng * sizeof(double), cudaMemcpyHostToDevice, s));
        src = tmp.p;
      }
      // diagonal of the dense block, for diag(Qinv)
      std::vector<double> dd(ng);
      CBX_CUDA(cudaMemcpy2DAsync(dd.data(), sizeof(double), src, (ng + 1) * sizeof(double), sizeof(double), ng,
                                 cudaMemcpyDeviceToHost, s));
      CBX_CUDA(cudaStreamSynchronize(s));
      for (int64_t k = 0; k < ng; ++k) diag[gmap[k]] += dd[k];
      upload_dense(h, m, src, ng, Gd ? -1 : h->Hd_gen);
      m.gmap.resize(ng);
      m.ginv.resize(q);
      CBX_CUDA(cudaMemcpyAsync(m.gmap.p, gmap, ng * sizeof(int32_t), cudaMemcpyHostToDevice, s));
      CBX_CUDA(cudaMemcpyAsync(m.ginv.p, inv.data(), q * sizeof(int32_t), cudaMemcpyHostToDevice, s));
      CBX_CUDA(cudaStreamSynchronize(s));
    }
    m.diagQ.resize(q);
    CBX_CUDA(cudaMemcpyAsync(m.diagQ.p, diag.data(), q * sizeof(double), cudaMemcpyHostToDevice, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    for (auto& sp : m.solvers)
      if (sp) sp->rebind();  // workspaces kept; everything derived from the operator recomputed
  });
}

extern "C" int cbx_pcg_solve(cbx_handle* h, double lambda, int32_t nrhs, const double* B, double* X,
                             int32_t use_x0, double tol, int32_t maxit, int32_t tol_mode,
                             int32_t precision, int32_t* iters, double* relres) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create first");
    CBX_REQUIRE(nrhs > 0 && B && X, CBX_ERR_ARG, "bad right-hand sides");
    CBX_REQUIRE(maxit > 0 && tol > 0, CBX_ERR_ARG, "tol and maxit must be positive");
    CBX_REQUIRE(precision == 0 || precision == 1, CBX_ERR_ARG, "precision must be 0 (fp64) or 1 (mixed)");
    CBX_REQUIRE(std::isfinite(lambda), CBX_ERR_NONFINITE, "non-finite lambda");
    CBX_CUDA(cudaSetDevice(h->device));
    Mme& m = *h->mme;
    cudaStream_t s = h->stream;
    const size_t n = (size_t)m.dim * nrhs;
    m.io_b.resize(n);
    DevBuf<double> xb;
    xb.resize(n);
    CBX_CUDA(cudaMemcpyAsync(m.io_b.p, B, n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (use_x0) CBX_CUDA(cudaMemcpyAsync(xb.p, X, n * sizeof(double), cudaMemcpyHostToDevice, s));
    PcgResult r;
    pcg_solve(h, lambda, nrhs, m.io_b.p, xb.p, use_x0 != 0, tol, maxit, tol_mode, precision, r);
    CBX_CUDA(cudaMemcpyAsync(X, xb.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    // A column that breaks down twice (|p'Ap| < 1e-300 after the restart) stops
    // with its iterate, as PCGSolver::solve does (pcg_solver.h:482-495): the
    // reference leaves its loop, reports max_iter iterations and the true
    // residual (pcg_solver.h:530-534) and raises nothing; so does this call.
    for (int c = 0; c < nrhs; ++c) {
      if (iters) iters[c] = r.status[c] == sv::COL_BREAKDOWN ? maxit : r.iters[c];
      if (relres) relres[c] = r.relres[c];
    }
    for (int c = 0; c < nrhs; ++c)
      if (r.status[c] == sv::COL_NONFINITE) throw Error(CBX_ERR_NONFINITE, "non-finite PCG iterate");
  });
}

extern "C" int cbx_mme_keep_warm(cbx_handle* h, int32_t on) {
  return cbx_guard(h, [&] { h->keep_warm = on != 0; });
}

// Kernel timing of the dense block product (see include/cbx.h).
extern "C" int cbx_profile_enable(cbx_handle* h, int32_t on) {
  return cbx_guard(h, [&] {
    CBX_CUDA(cudaSetDevice(h->device));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
    for (auto& r : h->prof) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    h->prof.clear();
    h->prof_on = on != 0;
  });
}

extern "C" int cbx_profile_read(cbx_handle* h, int32_t bucket, int64_t* launches, double* total_ms,
                                double* total_bytes) {
  return cbx_guard(h, [&] {
    CBX_CUDA(cudaSetDevice(h->device));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
    int64_t n = 0;
    double ms = 0, bytes = 0;
    for (auto& r : h->prof) {
      if (r.bucket != bucket) continue;
      float t = 0;
      CBX_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
      ms += t;
      bytes += r.bytes;
      ++n;
    }
    if (launches) *launches = n;
    if (total_ms) *total_ms = ms;
    if (total_bytes) *total_bytes = bytes;
  });
}

extern "C" int cbx_qinv_apply(cbx_handle* h, int32_t nrhs, const double* X, double* Y) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create first");
    CBX_REQUIRE(nrhs > 0 && X && Y, CBX_ERR_ARG, "bad vectors");
    CBX_CUDA(cudaSetDevice(h->device));
    Mme& m = *h->mme;
    cudaStream_t s = h->stream;
    const size_t n = (size_t)m.q * nrhs;
    DevBuf<double> xd, yd;
    xd.resize(n);
    yd.resize(n);
    CBX_CUDA(cudaMemcpyAsync(xd.p, X, n * sizeof(double), cudaMemcpyHostToDevice, s));
    qinv_apply(h, nrhs, xd.p, yd.p);
    CBX_CUDA(cudaMemcpyAsync(Y, yd.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
  });
}
