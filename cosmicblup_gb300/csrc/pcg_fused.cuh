// One PCG iteration after the dense block product, as one persistent
// cooperative kernel (the FP32 bulk of the mixed solver).
//
// The separate-kernel iteration of solver.cuh launches nine kernels per
// iteration (gather, column sums, fixed-row segments, SpMV, alpha, update,
// fixed-row preconditioner, beta, direction update); most of them move a few
// MB and are bound by launch and reduction latency.  Here one grid of
// co-resident blocks runs the whole step with four grid-wide barriers:
//
//   1  fixed-row segment partials of W'W p; random rows of q = A p (W'W, the
//      sparse Qinv, the dense product partials and the shift term); p'q
//      partials per block
//   2  fixed rows of q from their segment partials; p'q partials complete
//   3  alpha per column (every block sums the partials in the same order, so
//      all blocks hold identical scalars); x += alpha p, r -= alpha q, Jacobi
//      z on the random rows; r'r, r'z partials
//   4  block-Jacobi z on the fixed rows (the dense (X'X)^-1 block); r'z
//      partials of the fixed rows
//   5  beta, the stop tests (block 0 writes the column states); the next
//      direction p' = z + beta p into the second direction buffer, its
//      gathered dense-block rows (the next product's operand) and their FP64
//      column sums
//
// It is selected with CBX_FUSED=1.  Measured on GB300 it is 1-10 % slower per
// iteration than the separate kernels replayed from a CUDA graph, so the
// separate kernels are the default.
//
// The per-column recurrences, breakdown restart and stop tests are those of
// k_scalar_alpha / k_update / k_fixed / k_scalar_beta / k_pupdate (the
// reference's PCGSolver::solve, src/core/pcg_solver.h:436-536); every
// reduction is a fixed-order sum of per-block partials, so results do not
// depend on timing.
#pragma once
#include <cooperative_groups.h>
#include "solver.cuh"

namespace cbx {
namespace sv {

template <typename T>
struct FusedArgs {
  OpView<T> op;
  const T* Tout;             // dense product partials (tsplit x ng x S)
  int tsplit;
  const double* colsum;      // column sums of the gathered direction (shift term), or null
  double tshift;
  T lam;
  const int32_t* seg_lo;     // fixed-row segments of W'W
  const int32_t* seg_hi;
  int nseg;
  const int32_t* fix_seg_ptr;
  T* seg_part;               // nseg x S
  T* X;
  T* R;
  T* Z;
  const T* P;                // this iteration's direction
  T* Pn;                     // the next direction
  T* Q;                      // A p
  T* Vt;                     // next gathered operand (S x ld), null without a dense part
  const double* cpart_in;    // per-block column-sum partials of this step's direction (replaces colsum), or null
  double* cpart_out;         // per-block column-sum partials of the next direction (gridDim x S; may alias cpart_in)
  Col* col;
  const double* tol_col;
  int abs_tol;
  int maxit;
  int* active;
  double* part;              // gridDim x 4 x S
};

// Fixed-order sum over blocks of base[b * stride + c] (b < nb) for every
// column c; thread tid < S receives column tid's total.  Every block reads all
// partials, so the loads are issued 16 at a time to hide their latency.
template <int S>
__device__ __forceinline__ double col_total(const double* __restrict__ base, int64_t stride, int nb,
                                            double* red /*[NT]*/) {
  const int t = threadIdx.x;
  constexpr int G = NT / S;
  constexpr int U = 16;
  const int c = t % S, g = t / S;
  double v[U];
#pragma unroll
  for (int u = 0; u < U; ++u) v[u] = 0.0;
  int b = g;
  for (; b + (U - 1) * G < nb; b += U * G) {
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] += base[(int64_t)(b + u * G) * stride + c];
  }
  for (; b < nb; b += G) v[0] += base[(int64_t)b * stride + c];
#pragma unroll
  for (int w = U / 2; w > 0; w >>= 1)
#pragma unroll
    for (int u = 0; u < w; ++u) v[u] += v[u + w];
  red[t] = v[0];
  __syncthreads();
  double a = 0.0;
  if (t < S)
    for (int k = 0; k < G; ++k) a += red[k * S + t];
  __syncthreads();
  return a;
}

// p' = z + beta p as one rounded FMA, so that the stored direction, its
// gathered rows and their column sums agree exactly
__device__ __forceinline__ float dir_next(float z, float beta, float p) { return __fmaf_rn(beta, p, z); }
__device__ __forceinline__ double dir_next(double z, double beta, double p) { return __fma_rn(beta, p, z); }

template <typename T, int S>
__global__ void __launch_bounds__(NT) k_pcg_iter(FusedArgs<T> a) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  if (*a.active == 0) return;  // uniform: written by the previous step
  __shared__ double red[NT];
  __shared__ T redT[NT];
  __shared__ Col cs[S];
  __shared__ double blk[S];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nb = gridDim.x, b = blockIdx.x;
  const OpView<T>& op = a.op;
  const int64_t p = op.p, dim = op.dim;
  constexpr int G = NT / S;
  const int gc = tid % S, gg = tid / S;

  // column sums of the direction's dense-block rows: from the previous step's
  // per-block partials (fixed order), else given
  __shared__ double csum[S];
  const double* colsum = a.colsum;
  if (a.cpart_in) {
    const double t = col_total<S>(a.cpart_in, S, nb, red);
    if (tid < S) csum[tid] = t;
    __syncthreads();
    colsum = csum;
  }

  // ---- phase 1: segment partials; random rows of q = A p -------------------
  for (int sg = b; sg < a.nseg; sg += nb) {
    T acc[4] = {T(0), T(0), T(0), T(0)};
    const int32_t hi = a.seg_hi[sg];
    int32_t j = a.seg_lo[sg] + gg;
    for (; j + 3 * G < hi; j += 4 * G) {
#pragma unroll
      for (int u = 0; u < 4; ++u) acc[u] += op.Dval[j + u * G] * a.P[(int64_t)op.Dcol[j + u * G] * S + gc];
    }
    for (; j < hi; j += G) acc[0] += op.Dval[j] * a.P[(int64_t)op.Dcol[j] * S + gc];
    redT[tid] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
    __syncthreads();
    if (tid < S) {
      T sum = T(0);
      for (int k = 0; k < G; ++k) sum += redT[k * S + tid];
      a.seg_part[(int64_t)sg * S + tid] = sum;
    }
    __syncthreads();
  }
  {
    DotAcc<T> pqa[RowLayout<S>::CPL];
    const int64_t nwarps = (int64_t)nb * (NT / 32);
    for (int64_t i = p + (int64_t)b * (NT / 32) + warp; i < dim; i += nwarps)
      spmv_random_row<T, S>(op, i, a.P, a.Tout, a.tsplit, colsum, a.tshift, a.lam, 1, a.Q, a.P, pqa, lane);
    double pq[RowLayout<S>::CPL];
#pragma unroll
    for (int j = 0; j < RowLayout<S>::CPL; ++j) pq[j] = pqa[j].value();
    block_sum_row_pq<S>(pq, red, blk);  // blk[c] = this block's random-row p'q
  }
  grid.sync();

  // ---- phase 2: fixed rows of q; p'q partials -------------------------------
  for (int64_t f = b; f < p; f += nb) {
    T s = T(0);
    for (int32_t k = a.fix_seg_ptr[f] + gg; k < a.fix_seg_ptr[f + 1]; k += G) s += a.seg_part[(int64_t)k * S + gc];
    redT[tid] = s;
    __syncthreads();
    if (tid < S) {
      T t = T(0);
      for (int k = 0; k < G; ++k) t += redT[k * S + tid];
      a.Q[f * S + tid] = t;
      blk[tid] += (double)a.P[f * S + tid] * (double)t;
    }
    __syncthreads();
  }
  if (tid < S) a.part[(int64_t)b * 4 * S + tid] = blk[tid];
  grid.sync();

  // ---- phase 3: alpha; x, r, z updates; r'r and r'z partials ----------------
  {
    const double pq = col_total<S>(a.part, 4 * S, nb, red);
    if (tid < S) {
      Col s = a.col[tid];
      s.skip = 0;
      if (s.active) {
        s.pq = pq;
        if (fabs(pq) < 1e-300) {
          if (!s.restarted) {
            s.restarted = 1;
            s.skip = 1;  // restart: p = z, rz unchanged; no update this iteration
          } else {
            s.active = 0;
            s.status = COL_BREAKDOWN;
          }
        } else {
          s.alpha = s.rz / pq;
        }
      }
      cs[tid] = s;
    }
    __syncthreads();
  }
  {
    DotAcc<T> arr, arz;
    const int c = tid % S;
    const bool upd = cs[c].active != 0 && !cs[c].skip;
    const T alpha = (T)cs[c].alpha;
    const int64_t total = dim * S;
    for (int64_t idx = (int64_t)b * NT + tid; idx < total; idx += (int64_t)nb * NT) {
      const int64_t i = idx / S;
      T r = a.R[idx];
      if (upd) {
        a.X[idx] += alpha * a.P[idx];
        r -= alpha * a.Q[idx];
        a.R[idx] = r;
      }
      arr.add(r, r);
      if (i >= p) {
        T z = a.Z[idx];
        if (upd) {
          z = op.dinv[i - p] * r;
          a.Z[idx] = z;
        }
        arz.add(r, z);
      }
    }
    const double rr = arr.value(), rz = arz.value();
    double t = block_sum_cols<S>(rr, red);
    if (tid < S) a.part[(int64_t)b * 4 * S + 1 * S + tid] = t;
    t = block_sum_cols<S>(rz, red);
    if (tid < S) a.part[(int64_t)b * 4 * S + 2 * S + tid] = t;
  }
  grid.sync();

  // ---- phase 4: block-Jacobi z on the fixed rows; their r'z -----------------
  if (tid < S) blk[tid] = 0.0;
  __syncthreads();
  for (int64_t f = b; f < p; f += nb) {
    T acc = T(0);
    for (int64_t k = gg; k < p; k += G) acc += op.A11inv[f * p + k] * a.R[k * S + gc];
    redT[tid] = acc;
    __syncthreads();
    if (tid < S) {
      T s = T(0);
      for (int k = 0; k < G; ++k) s += redT[k * S + tid];
      const bool act = cs[tid].active != 0;
      if (act) a.Z[f * S + tid] = s;
      const T zf = act ? s : a.Z[f * S + tid];
      blk[tid] += (double)a.R[f * S + tid] * (double)zf;
    }
    __syncthreads();
  }
  if (tid < S) a.part[(int64_t)b * 4 * S + 3 * S + tid] = blk[tid];
  grid.sync();

  // ---- phase 5: beta and the stop tests; the next direction -----------------
  {
    const double rr = col_total<S>(a.part + S, 4 * S, nb, red);
    const double rzr = col_total<S>(a.part + 2 * S, 4 * S, nb, red);
    const double rzf = col_total<S>(a.part + 3 * S, 4 * S, nb, red);
    if (tid < S) {
      Col s = cs[tid];
      if (s.active) {
        const double rz = rzr + rzf;
        s.rr = rr;
        if (s.skip) {
          s.beta = 0.0;
          s.rz = rz;
        } else {
          s.iters += 1;
          const double bn = s.bnorm2 > 0 ? sqrt(s.bnorm2) : 1.0;
          const double res = sqrt(rr);
          const double tol = a.tol_col[tid];
          const bool conv = a.abs_tol ? (res < tol) : (res / bn < tol);
          if (conv) {
            s.active = 0;
            s.status = COL_CONVERGED;
          } else if (!isfinite(rr) || !isfinite(rz)) {
            s.active = 0;
            s.status = COL_NONFINITE;
          } else if (s.iters >= a.maxit) {
            s.active = 0;
            s.status = COL_MAXIT;
          } else {
            s.beta = rz / s.rz;
            s.rz = rz;
          }
        }
      }
      cs[tid] = s;
      if (b == 0) a.col[tid] = s;
    }
    __syncthreads();
    if (b == 0 && tid == 0) {
      int n_act = 0;
      for (int k = 0; k < S; ++k) n_act += cs[k].active;
      *a.active = n_act;
    }
  }
  {
    const int c = tid % S;
    const bool act = cs[c].active != 0;
    const T beta = (T)cs[c].beta;
    const int64_t total = dim * S;
    for (int64_t idx = (int64_t)b * NT + tid; idx < total; idx += (int64_t)nb * NT)
      a.Pn[idx] = act ? dir_next(a.Z[idx], beta, a.P[idx]) : a.P[idx];
  }
  if (a.Vt) {
    // the next product's operand: rows of the new direction at the dense block
    const int64_t ld = op.ld, ng = op.ng;
    const int64_t total = (int64_t)S * ld;
    for (int64_t idx = (int64_t)b * NT + tid; idx < total; idx += (int64_t)nb * NT) {
      const int64_t c = idx / ld, k = idx - c * ld;
      T v = T(0);
      if (k < ng) {
        const int64_t e = (p + op.gmap[k]) * S + c;
        v = cs[c].active ? dir_next(a.Z[e], (T)cs[c].beta, a.P[e]) : a.P[e];
      }
      a.Vt[idx] = v;
    }
    // per-block FP64 column-sum partials of those rows over a contiguous
    // slice of the dense block (summed by the next step in a fixed order)
    const int64_t k0 = (int64_t)b * ng / nb, k1 = (int64_t)(b + 1) * ng / nb;
    double acc = 0.0;
    const bool act = cs[gc].active != 0;
    const T beta = (T)cs[gc].beta;
    for (int64_t k = k0 + gg; k < k1; k += G) {
      const int64_t e = (p + op.gmap[k]) * S + gc;
      acc += (double)(act ? dir_next(a.Z[e], beta, a.P[e]) : a.P[e]);
    }
    red[tid] = acc;
    __syncthreads();
    if (tid < S) {
      double t = 0.0;
      for (int k = 0; k < G; ++k) t += red[k * S + tid];
      a.cpart_out[(int64_t)b * S + tid] = t;
    }
  }
}

}  // namespace sv
}  // namespace cbx
