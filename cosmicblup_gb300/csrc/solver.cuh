// Kernels of the mixed-model operator and of the multi-right-hand-side PCG.
//
// Vectors hold S right-hand sides interleaved: element (row i, column c) at
// v[i * S + c].  Every column runs its own CG recurrence (the reference's
// PCGSolver::solve, src/core/pcg_solver.h:436-536, applied to S systems at
// once); the matrix is read once per iteration for all columns.  All
// reductions are deterministic: per-block partial sums are combined in a fixed
// order by the scalar kernels.
#pragma once
#include <cuda_fp16.h>
#include "mme.h"

namespace cbx {
namespace sv {

constexpr int NT = 256;    // threads per block of the vector kernels
constexpr int NTS = 1024;  // threads of the single-block scalar steps (partial sums read in parallel)

// Per-column CG state (device).
struct Col {
  double rz, pq, rr, bnorm2, alpha, beta;
  int active, iters, restarted, skip, status;
  int pad;
};
enum ColStatus : int { COL_RUNNING = 0, COL_CONVERGED = 1, COL_MAXIT = 2, COL_BREAKDOWN = 3,
                       COL_NONFINITE = 4 };

// Read-only view of the operator in one precision.
template <typename T>
struct OpView {
  int64_t p, q, dim;
  const int32_t* Dptr; const int32_t* Dcol; const T* Dval;
  const int32_t* Sptr; const int32_t* Scol; const T* Sval;  // null if no sparse part
  const T* Qd; int64_t ng, ld; const int32_t* gmap; const int32_t* ginv;  // null if no dense part
  const T* A11inv;  // p x p
  const T* dinv;    // q (Jacobi of the random part)
};

// Per-thread dot-product accumulator.  The FP64 solver sums in FP64.  The
// FP32 solver sums its FP32 products with Kahan compensation in FP32: GB300
// runs FP64 arithmetic at 1/64 of the FP32 rate, so one FP64 multiply-add per
// vector element made the FP32 vector kernels FP64-bound; the compensated
// FP32 sum keeps the error of the per-thread sums near one FP32 rounding of
// the sum, and the block and grid sums stay in FP64.
template <typename T> struct DotAcc;
template <> struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s += a * b; }
  __device__ __forceinline__ double value() const { return s; }
};
template <> struct DotAcc<float> {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float a, float b) {
    const float y = fmaf(a, b, -c);
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int n = 2; };

__device__ __forceinline__ float dot16(const float4& a, const float4& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}
__device__ __forceinline__ double dot16(const double2& a, const double2& b) {
  return a.x * b.x + a.y * b.y;
}

// Vt[c * ld + k] = X[(p + gmap[k]) * xs + c] for k < ng, 0 for ng <= k < ld
// (S columns of a block whose rows are xs apart; xs = S for the whole block).
template <typename T, int S>
__global__ void k_gather_t(const T* __restrict__ X, T* __restrict__ Vt, int64_t p, int64_t ng,
                           int64_t ld, const int32_t* __restrict__ gmap,
                           const int* __restrict__ active, int xs = S, int nc = S) {
  if (active && *active == 0) return;
  const int64_t total = (int64_t)nc * ld;  // the first nc columns (the populated ones)
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / ld, k = idx - c * ld;
    Vt[idx] = k < ng ? X[(p + gmap[k]) * xs + c] : T(0);
  }
}

// Dense block product Tout[i * os + c] = sum_k Qd[i * ld + k] * Vt[c * ld + k]
// (os = S unless the S columns are a piece of a wider block).
// 8 warps per block, RPW rows per warp; lanes stream 16-byte vectors of each
// row; the S right-hand sides of a K tile are staged in shared memory.
template <typename T, int S, int RPW>
__global__ void __launch_bounds__(256) k_dense(const T* __restrict__ Qd, int64_t ng, int64_t ld,
                                               const T* __restrict__ Vt, T* __restrict__ Tout,
                                               const int* __restrict__ active, int os = S) {
  if (active && *active == 0) return;
  using V = typename Vec16<T>::type;
  constexpr int VEC = Vec16<T>::n;
  constexpr int KT = 32 * VEC * 4;
  extern __shared__ __align__(16) uint8_t dsm[];
  T* vt = reinterpret_cast<T*>(dsm);  // [S][KT]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t row0 = (int64_t)blockIdx.x * (8 * RPW) + warp * RPW;
  T acc[RPW][S];
#pragma unroll
  for (int r = 0; r < RPW; ++r)
#pragma unroll
    for (int c = 0; c < S; ++c) acc[r][c] = T(0);
  for (int64_t k0 = 0; k0 < ld; k0 += KT) {
    __syncthreads();
    for (int v = tid; v < S * (KT / VEC); v += 256) {
      const int c = v / (KT / VEC), kk = (v % (KT / VEC)) * VEC;
      V val;
      if (k0 + kk < ld) val = *reinterpret_cast<const V*>(Vt + (int64_t)c * ld + k0 + kk);
      else memset(&val, 0, sizeof(V));
      *reinterpret_cast<V*>(vt + c * KT + kk) = val;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int kk = u * 32 * VEC + lane * VEC;
      if (k0 + kk < ld) {
        V a[RPW];
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          if (row0 + r < ng) a[r] = __ldg(reinterpret_cast<const V*>(Qd + (row0 + r) * ld + k0 + kk));
          else memset(&a[r], 0, sizeof(V));
        }
#pragma unroll
        for (int c = 0; c < S; ++c) {
          const V b = *reinterpret_cast<const V*>(vt + c * KT + kk);
#pragma unroll
          for (int r = 0; r < RPW; ++r) acc[r][c] += dot16(a[r], b);
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
#pragma unroll
    for (int c = 0; c < S; ++c) {
      T v = acc[r][c];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      acc[r][c] = v;
    }
    if (lane == 0 && row0 + r < ng) {
#pragma unroll
      for (int c = 0; c < S; ++c) Tout[(row0 + r) * os + c] = acc[r][c];
    }
  }
}

// Single right-hand side: Tout[i] = sum_k Qd[i * ld + k] v[k].  A pure HBM
// stream: each warp owns RPW rows and keeps U x (RPW + 1) 16-byte loads in
// flight per lane; v (ld values) is read through the read-only cache.
template <typename T, int RPW, int U>
__global__ void __launch_bounds__(256) k_gemv(const T* __restrict__ Qd, int64_t ng, int64_t ld,
                                              const T* __restrict__ v, T* __restrict__ Tout,
                                              const int* __restrict__ active, int os = 1) {
  if (active && *active == 0) return;
  using V = typename Vec16<T>::type;
  constexpr int VEC = Vec16<T>::n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row0 = ((int64_t)blockIdx.x * 8 + warp) * RPW;
  if (row0 >= ng) return;
  const int64_t nvec = ld / VEC;
  const V* vv = reinterpret_cast<const V*>(v);
  const V* rows[RPW];
#pragma unroll
  for (int r = 0; r < RPW; ++r)
    rows[r] = reinterpret_cast<const V*>(Qd + (row0 + r < ng ? row0 + r : row0) * ld);
  T acc[RPW];
#pragma unroll
  for (int r = 0; r < RPW; ++r) acc[r] = T(0);
  for (int64_t j0 = lane; j0 < nvec; j0 += 32 * U) {
    V a[U][RPW], b[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t j = j0 + u * 32;
      if (j < nvec) {
        b[u] = __ldg(vv + j);
#pragma unroll
        for (int r = 0; r < RPW; ++r) a[u][r] = __ldg(rows[r] + j);
      } else {
        memset(&b[u], 0, sizeof(V));
#pragma unroll
        for (int r = 0; r < RPW; ++r) memset(&a[u][r], 0, sizeof(V));
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int r = 0; r < RPW; ++r) acc[r] += dot16(a[u][r], b[u]);
  }
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    T t = acc[r];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (lane == 0 && row0 + r < ng) Tout[(row0 + r) * os] = t;
  }
}

// ---------------------------------------------------------------------------
// Float-float ("double-single") block product for the refinement residual.
//
// GB300 runs FP64 at 1.25 TFLOP/s, so an FP64 product with 32 right-hand
// sides is FP64-bound (2 ng^2 S flops).  The mixed solver's recursive
// residual update r -= A d for a correction d that is small next to x needs
// the product only to ~46 bits, relative to |Qd| |d|: with Qd = Qh + Ql
// (Qh = fl32(Qd), Ql = fl32(Qd - Qh)) and
// x = xh + xl likewise, each term is
//   Qh xh  exactly, as p + e with p = fl(Qh xh), e = fma(Qh, xh, -p),
//   + Qh xl + Ql xh (FP32, relative 2^-24 of terms that are 2^-24 small),
// accumulated in an unevaluated (hi, lo) pair by Knuth's two-sum.  Every
// dropped or rounded part is below 2^-46 of |Qd| |x| per term; the pair is
// renormalised after each K tile so lo stays below ulp(hi).  All arithmetic is
// FP32 (the __f*_rn intrinsics keep the compiler from contracting or
// reassociating the error-free steps).
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  const float t = __fadd_rn(hi, p);
  const float z = __fsub_rn(t, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(p, z));
  hi = t;
  lo = __fadd_rn(lo, __fadd_rn(err, e));
}
// (hi, lo) += (h2, l2)
__device__ __forceinline__ void ff_add(float& hi, float& lo, float h2, float l2) {
  const float t = __fadd_rn(hi, h2);
  const float z = __fsub_rn(t, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(h2, z));
  const float l = __fadd_rn(__fadd_rn(lo, l2), err);
  hi = __fadd_rn(t, l);
  lo = __fsub_rn(l, __fsub_rn(hi, t));
}
__device__ __forceinline__ void ff_norm(float& hi, float& lo) {
  const float t = __fadd_rn(hi, lo);
  lo = __fsub_rn(lo, __fsub_rn(t, hi));
  hi = t;
}

// Vhl[c * ld + k] = (hi, lo) FP32 parts of X[(p + gmap[k]) * S + c] for k < ng,
// (0, 0) in the padding: the gathered vectors of the float-float product, split
// once here so that the product kernel does no FP64 arithmetic.
template <int S>
__global__ void k_gather_hl(const double* __restrict__ X, float2* __restrict__ Vhl, int64_t p, int64_t ng,
                            int64_t ld, const int32_t* __restrict__ gmap, int xs = S) {
  const int64_t total = (int64_t)S * ld;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / ld, k = idx - c * ld;
    const double x = k < ng ? X[(p + gmap[k]) * xs + c] : 0.0;
    const float xh = __double2float_rn(x);
    Vhl[idx] = make_float2(xh, __double2float_rn(x - (double)xh));
  }
}

// out[c] = sum_k X[(p + gmap[k]) * xs + c] over the dense-block rows, in FP64
// with Neumaier compensation (the column sums that restore the shift of the
// float-float block: the sum cancels almost completely for a solution with a
// small component along an eigen-bent direction, so plain summation would
// lose the digits that the shift multiplies).  One block of 256 threads per
// column, combined in a fixed order.
__device__ __forceinline__ void two_sum_acc(double& s, double& e, double x) {
  const double t = __dadd_rn(s, x);
  const double z = __dsub_rn(t, s);
  e = __dadd_rn(e, __dadd_rn(__dsub_rn(s, __dsub_rn(t, z)), __dsub_rn(x, z)));
  s = t;
}
static __global__ void __launch_bounds__(256) k_colsum_x(const double* __restrict__ X, int xs, int64_t p,
                                                         int64_t ng, const int32_t* __restrict__ gmap,
                                                         double* __restrict__ out) {
  __shared__ double rs[256], re[256];
  const int c = blockIdx.x, tid = threadIdx.x;
  double s = 0.0, e = 0.0;
  for (int64_t k = tid; k < ng; k += 256) two_sum_acc(s, e, X[(p + gmap[k]) * xs + c]);
  rs[tid] = s;
  re[tid] = e;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (tid < o) {
      double a = rs[tid], ea = re[tid];
      two_sum_acc(a, ea, rs[tid + o]);
      rs[tid] = a;
      re[tid] = __dadd_rn(ea, re[tid + o]);
    }
    __syncthreads();
  }
  if (tid == 0) out[c] = __dadd_rn(rs[0], re[0]);
}

// out[c] = sum_k Vt[c * ld + k] (k < ng): the column sums of the gathered
// vectors of an FP32 product with the shifted block.  Each thread sums with
// Kahan compensation (error about one rounding of its sum plus n eps^2 of the
// magnitudes, far below the FP32 product's), the threads' sums are combined in
// FP64.  One block of 1024 threads per column, fixed order.
template <typename T>
__global__ void __launch_bounds__(1024) k_colsum_vt(const T* __restrict__ Vt, int64_t ld, int64_t ng,
                                                    double* __restrict__ out) {
  __shared__ double red[1024];
  const int c = blockIdx.x, tid = threadIdx.x;
  // per-thread sums compensated in the vectors' own precision (no FP64
  // arithmetic per element), combined in FP64
  DotAcc<T> acc[4];
  const T* col = Vt + (int64_t)c * ld;
  int64_t k = tid;
  for (; k + 3 * 1024 < ng; k += 4 * 1024) {
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u].add(col[k + u * 1024], T(1));
  }
  for (; k < ng; k += 1024) acc[0].add(col[k], T(1));
  red[tid] = (acc[0].value() + acc[1].value()) + (acc[2].value() + acc[3].value());
  __syncthreads();
  for (int o = 512; o > 0; o >>= 1) {
    if (tid < o) red[tid] += red[tid + o];
    __syncthreads();
  }
  if (tid == 0) out[c] = red[0];
}

// Tout[i * S + c] = sum_k Qd[i][k] V[c][k] in float-float; Qh / Ql are the
// hi / lo FP32 parts of the ng x ld row-major block, Vhl the (hi, lo) parts of
// the gathered vectors.  8 warps, RPW rows per warp, lanes stream float4s of
// both block parts; the K tile of the S vectors is staged in shared memory.
template <int S, int RPW>
__global__ void __launch_bounds__(256) k_dense_ff(const float* __restrict__ Qh, const float* __restrict__ Ql,
                                                  int64_t ng, int64_t ld, const float2* __restrict__ Vhl,
                                                  double* __restrict__ Tout, const int* __restrict__ active,
                                                  int os = S) {
  if (active && *active == 0) return;
  constexpr int KT = 32 * 4 * 2;
  extern __shared__ __align__(16) uint8_t dsm[];
  float2* vt = reinterpret_cast<float2*>(dsm);  // [S][KT] (hi, lo)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t row0 = (int64_t)blockIdx.x * (8 * RPW) + warp * RPW;
  float hi[RPW][S], lo[RPW][S];
#pragma unroll
  for (int r = 0; r < RPW; ++r)
#pragma unroll
    for (int c = 0; c < S; ++c) hi[r][c] = lo[r][c] = 0.0f;
  for (int64_t k0 = 0; k0 < ld; k0 += KT) {
    __syncthreads();
    for (int v = tid; v < S * KT; v += 256) {
      const int c = v / KT, kk = v % KT;
      vt[v] = (k0 + kk < ld) ? Vhl[(int64_t)c * ld + k0 + kk] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < KT / 128; ++u) {
      const int kk = u * 128 + lane * 4;
      if (k0 + kk < ld) {
        float4 ah[RPW], al[RPW];
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          if (row0 + r < ng) {
            ah[r] = __ldg(reinterpret_cast<const float4*>(Qh + (row0 + r) * ld + k0 + kk));
            al[r] = __ldg(reinterpret_cast<const float4*>(Ql + (row0 + r) * ld + k0 + kk));
          } else {
            ah[r] = make_float4(0.f, 0.f, 0.f, 0.f);
            al[r] = ah[r];
          }
        }
#pragma unroll
        for (int c = 0; c < S; ++c) {
          const float4 b01 = *reinterpret_cast<const float4*>(vt + c * KT + kk);
          const float4 b23 = *reinterpret_cast<const float4*>(vt + c * KT + kk + 2);
#pragma unroll
          for (int r = 0; r < RPW; ++r) {
            ff_acc(hi[r][c], lo[r][c], ah[r].x, al[r].x, b01.x, b01.y);
            ff_acc(hi[r][c], lo[r][c], ah[r].y, al[r].y, b01.z, b01.w);
            ff_acc(hi[r][c], lo[r][c], ah[r].z, al[r].z, b23.x, b23.y);
            ff_acc(hi[r][c], lo[r][c], ah[r].w, al[r].w, b23.z, b23.w);
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RPW; ++r)
#pragma unroll
      for (int c = 0; c < S; ++c) ff_norm(hi[r][c], lo[r][c]);
  }
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
#pragma unroll
    for (int c = 0; c < S; ++c) {
      float h = hi[r][c], l = lo[r][c];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, h, off);
        const float l2 = __shfl_xor_sync(0xffffffffu, l, off);
        ff_add(h, l, h2, l2);
      }
      hi[r][c] = h;
      lo[r][c] = l;
    }
    if (lane == 0 && row0 + r < ng) {
#pragma unroll
      for (int c = 0; c < S; ++c) Tout[(row0 + r) * os + c] = (double)hi[r][c] + (double)lo[r][c];
    }
  }
}

// ---- packed (f32x2) float-float product -----------------------------------
// The same float-float accumulation as k_dense_ff for two columns per instruction
// with the sm_100-family packed FP32 operations (fma/add/sub/mul .rn.f32x2).  Each
// lane of a packed operation rounds exactly as the scalar operation does, and the
// order of every accumulation is unchanged, so the results are bit-identical to
// k_dense_ff's; only the instruction count per column halves.
typedef unsigned long long f32x2_t;
__device__ __forceinline__ f32x2_t f2_pack(float a, float b) {
  f32x2_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2_unpack(f32x2_t v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f32x2_t f2_add(f32x2_t a, f32x2_t b) {
  f32x2_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2_t f2_sub(f32x2_t a, f32x2_t b) {
  f32x2_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2_t f2_mul(f32x2_t a, f32x2_t b) {
  f32x2_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2_t f2_fma(f32x2_t a, f32x2_t b, f32x2_t c) {
  f32x2_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
// ff_acc on a column pair.  With na = -ah, np = na bh = -fl(ah bh) exactly, so every
// step below is the scalar step with a sign moved into an exact negation:
//   e = fma(ah, bh, -p), t = hi + p, err = (hi - (t - z)) + (p - z) = (hi - (t - z)) - (np + z).
__device__ __forceinline__ void ff_acc2(f32x2_t& hi, f32x2_t& lo, f32x2_t a, f32x2_t na, f32x2_t al, f32x2_t bh,
                                        f32x2_t bl) {
  const f32x2_t np = f2_mul(na, bh);
  f32x2_t e = f2_fma(a, bh, np);
  e = f2_fma(a, bl, e);
  e = f2_fma(al, bh, e);
  const f32x2_t t = f2_sub(hi, np);
  const f32x2_t z = f2_sub(t, hi);
  const f32x2_t err = f2_sub(f2_sub(hi, f2_sub(t, z)), f2_add(np, z));
  hi = t;
  lo = f2_add(lo, f2_add(err, e));
}

// Tout as k_dense_ff for an even S.  The staged K tile holds, per column pair q and
// k, the float4 (hi_2q, hi_2q+1, lo_2q, lo_2q+1); lane l of the warp reads k = 4 (u 32
// + l) + j at vt4[(q 4 + j) (KT / 4) + u 32 + l], so a warp's 16-byte reads are
// contiguous.
template <int S, int RPW>
__global__ void __launch_bounds__(256) k_dense_ff2(const float* __restrict__ Qh, const float* __restrict__ Ql,
                                                   int64_t ng, int64_t ld, const float2* __restrict__ Vhl,
                                                   double* __restrict__ Tout, const int* __restrict__ active,
                                                   int os = S) {
  static_assert(S % 2 == 0, "column pairs");
  if (active && *active == 0) return;
  constexpr int KT = 32 * 4 * 2;
  constexpr int NP = S / 2;
  extern __shared__ __align__(16) uint8_t dsm[];
  float4* vt4 = reinterpret_cast<float4*>(dsm);  // [NP * 4][KT / 4]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t row0 = (int64_t)blockIdx.x * (8 * RPW) + warp * RPW;
  f32x2_t hi[RPW][NP], lo[RPW][NP];
#pragma unroll
  for (int r = 0; r < RPW; ++r)
#pragma unroll
    for (int q = 0; q < NP; ++q) hi[r][q] = lo[r][q] = 0ull;
  for (int64_t k0 = 0; k0 < ld; k0 += KT) {
    __syncthreads();
    for (int v = tid; v < NP * KT; v += 256) {
      const int q = v / KT, kk = v % KT;
      float2 b0 = make_float2(0.f, 0.f), b1 = b0;
      if (k0 + kk < ld) {
        b0 = Vhl[(int64_t)(2 * q) * ld + k0 + kk];
        b1 = Vhl[(int64_t)(2 * q + 1) * ld + k0 + kk];
      }
      vt4[(q * 4 + (kk & 3)) * (KT / 4) + (kk >> 2)] = make_float4(b0.x, b1.x, b0.y, b1.y);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < KT / 128; ++u) {
      const int kk = u * 128 + lane * 4;
      if (k0 + kk < ld) {
        float4 ah[RPW], al[RPW];
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          if (row0 + r < ng) {
            ah[r] = __ldg(reinterpret_cast<const float4*>(Qh + (row0 + r) * ld + k0 + kk));
            al[r] = __ldg(reinterpret_cast<const float4*>(Ql + (row0 + r) * ld + k0 + kk));
          } else {
            ah[r] = make_float4(0.f, 0.f, 0.f, 0.f);
            al[r] = ah[r];
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          f32x2_t a2[RPW], na2[RPW], al2[RPW];
#pragma unroll
          for (int r = 0; r < RPW; ++r) {
            const float a = j == 0 ? ah[r].x : (j == 1 ? ah[r].y : (j == 2 ? ah[r].z : ah[r].w));
            const float l = j == 0 ? al[r].x : (j == 1 ? al[r].y : (j == 2 ? al[r].z : al[r].w));
            a2[r] = f2_pack(a, a);
            na2[r] = f2_pack(-a, -a);
            al2[r] = f2_pack(l, l);
          }
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            const float4 b = vt4[(q * 4 + j) * (KT / 4) + u * 32 + lane];
            const f32x2_t bh = f2_pack(b.x, b.y), bl = f2_pack(b.z, b.w);
#pragma unroll
            for (int r = 0; r < RPW; ++r) ff_acc2(hi[r][q], lo[r][q], a2[r], na2[r], al2[r], bh, bl);
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RPW; ++r)
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        float h0, h1, l0, l1;
        f2_unpack(hi[r][q], h0, h1);
        f2_unpack(lo[r][q], l0, l1);
        ff_norm(h0, l0);
        ff_norm(h1, l1);
        hi[r][q] = f2_pack(h0, h1);
        lo[r][q] = f2_pack(l0, l1);
      }
  }
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    float h[S], l[S];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      f2_unpack(hi[r][q], h[2 * q], h[2 * q + 1]);
      f2_unpack(lo[r][q], l[2 * q], l[2 * q + 1]);
    }
#pragma unroll
    for (int c = 0; c < S; ++c) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, h[c], off);
        const float l2 = __shfl_xor_sync(0xffffffffu, l[c], off);
        ff_add(h[c], l[c], h2, l2);
      }
    }
    if (lane == 0 && row0 + r < ng) {
#pragma unroll
      for (int c = 0; c < S; ++c) Tout[(row0 + r) * os + c] = (double)h[c] + (double)l[c];
    }
  }
}

// Block-level sum of one double per thread, grouped by column c = tid % S.
// Returns the total for column (tid % S) in threads tid < S.
template <int S>
__device__ __forceinline__ double block_sum_cols(double v, double* red /*[NT]*/) {
  const int tid = threadIdx.x;
  if constexpr (S > 32) {
    // a warp spans part of one column set: sum the S-strided threads directly
    red[tid] = v;
    __syncthreads();
    double t = 0.0;
    if (tid < S)
      for (int w = 0; w < (int)blockDim.x / S; ++w) t += red[w * S + tid];
    __syncthreads();
    return t;
  } else {
#pragma unroll
    for (int off = 16; off >= S; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    // now lanes < S of each warp hold that warp's per-column sums
    const int warp = tid >> 5, lane = tid & 31;
    if (lane < S) red[warp * S + lane] = v;
    __syncthreads();
    double t = 0.0;
    if (tid < S) {
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w * S + tid];
    }
    __syncthreads();
    return t;
  }
}

// Fixed-effect rows of W'W can hold one entry per record (the mean holds all of
// them).  They are cut into segments of at most FIX_SEG entries; k_fix_seg
// computes one partial sum per (segment, column) and k_spmv adds a row's
// segment partials in order.
constexpr int FIX_SEG = 256;

template <typename T, int S>
__global__ void __launch_bounds__(NT) k_fix_seg(OpView<T> op, const int32_t* __restrict__ seg_row,
                                                const int32_t* __restrict__ seg_lo, const int32_t* __restrict__ seg_hi,
                                                const T* __restrict__ X, T* __restrict__ seg_part,
                                                const int* __restrict__ active, int ncp = S) {
  if (active && *active == 0) return;
  __shared__ T redT[NT];
  const int sg = blockIdx.x;
  constexpr int G = NT / S;
  const int tid = threadIdx.x, c = tid % S, g = tid / S;
  T acc[4] = {T(0), T(0), T(0), T(0)};
  // columns past the populated ones (ncp) are not computed
  const int32_t hi = c < ncp ? seg_hi[sg] : 0;
  int32_t j = seg_lo[sg] + g;
  for (; j + 3 * G < hi; j += 4 * G) {
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] += op.Dval[j + u * G] * X[(int64_t)op.Dcol[j + u * G] * S + c];
  }
  for (; j < hi; j += G) acc[0] += op.Dval[j] * X[(int64_t)op.Dcol[j] * S + c];
  redT[tid] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
  __syncthreads();
  if (tid < S) {
    T s = T(0);
    for (int gg = 0; gg < G; ++gg) s += redT[gg * S + tid];
    seg_part[(int64_t)sg * S + tid] = s;
  }
  (void)seg_row;
}

// Lanes of a warp over the S columns of one row: S <= 32 puts 32 / S lanes on
// each column (c = lane % S); S > 32 gives each lane CPL = S / 32 columns
// (c = lane + 32 j).
template <int S>
struct RowLayout {
  static constexpr int CPL = S > 32 ? S / 32 : 1;
};

// Random-effect row i of Y = use_D W'W X + lam [Qs X_u + scatter(Tout) +
// tshift colsum] (one warp); adds this lane's P[i] Y[i] terms to pq.
template <typename T, int S>
__device__ __forceinline__ void spmv_random_row(const OpView<T>& op, int64_t i, const T* __restrict__ X,
                                                const T* __restrict__ Tout, int tsplit,
                                                const double* __restrict__ colsum, double tshift, T lam,
                                                int use_D, T* __restrict__ Y, const T* __restrict__ P,
                                                DotAcc<T> (&pq)[RowLayout<S>::CPL], int lane) {
  const int64_t p = op.p, u = i - p;
  if constexpr (S > 32) {
    // column groups of 32; the 128-wide block holds at most 80 populated
    // columns (its tensor-core product's limit), so only its first three groups
    // are computed and the fourth is written as zero
    constexpr int CPL = S / 32;
    constexpr int NG = S == 128 ? 3 : CPL;
    T acc[CPL], qv[CPL];
#pragma unroll
    for (int j = 0; j < CPL; ++j) acc[j] = qv[j] = T(0);
    // entries in batches of 4: all the batch's row loads are issued before its
    // multiply-adds (same order of additions as one entry at a time)
    auto rowsum = [&](const int32_t* __restrict__ cidx, const T* __restrict__ val, int32_t e, int32_t e1,
                      int64_t off, T (&out)[CPL]) {
      for (; e + 3 < e1; e += 4) {
        T dv[4], xv[4][NG];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          dv[k] = val[e + k];
          const T* xr = X + (off + cidx[e + k]) * S + lane;
#pragma unroll
          for (int j = 0; j < NG; ++j) xv[k][j] = xr[32 * j];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
          for (int j = 0; j < NG; ++j) out[j] += dv[k] * xv[k][j];
      }
      for (; e < e1; ++e) {
        const T dv = val[e];
        const T* xr = X + (off + cidx[e]) * S + lane;
#pragma unroll
        for (int j = 0; j < NG; ++j) out[j] += dv * xr[32 * j];
      }
    };
    if (use_D) rowsum(op.Dcol, op.Dval, op.Dptr[i], op.Dptr[i + 1], 0, acc);
    if (op.Sptr) rowsum(op.Scol, op.Sval, op.Sptr[u], op.Sptr[u + 1], p, qv);
    if (op.Qd) {
      const int32_t k = op.ginv[u];
      if (k >= 0) {
        for (int t = 0; t < tsplit; ++t) {
          const T* tr = Tout + ((int64_t)t * op.ng + k) * S + lane;
#pragma unroll
          for (int j = 0; j < NG; ++j) qv[j] += tr[32 * j];
        }
        if (colsum) {
#pragma unroll
          for (int j = 0; j < NG; ++j) qv[j] += (T)(tshift * colsum[lane + 32 * j]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
      if (j < NG) {
        const T yv = acc[j] + lam * qv[j];
        Y[i * S + lane + 32 * j] = yv;
        if (P) pq[j].add(P[i * S + lane + 32 * j], yv);
      } else {
        Y[i * S + lane + 32 * j] = T(0);  // defined, never read
      }
    }
  } else {
    constexpr int G = 32 / S;
    const int c = lane % S, g = lane / S;
    // this lane's entries j = start + g, + G, ... in batches of 4 (loads first,
    // then the multiply-adds in the same order as one entry at a time)
    auto rowsum1 = [&](const int32_t* __restrict__ cidx, const T* __restrict__ val, int32_t j, int32_t e1,
                       int64_t off) {
      T a = T(0);
      for (; j + 3 * G < e1; j += 4 * G) {
        T dv[4], xv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          dv[k] = val[j + k * G];
          xv[k] = X[(off + cidx[j + k * G]) * S + c];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) a += dv[k] * xv[k];
      }
      for (; j < e1; j += G) a += val[j] * X[(off + cidx[j]) * S + c];
      return a;
    };
    T acc = T(0);
    if (use_D) acc = rowsum1(op.Dcol, op.Dval, op.Dptr[i] + g, op.Dptr[i + 1], 0);
    T qv = T(0);
    if (op.Sptr) qv = rowsum1(op.Scol, op.Sval, op.Sptr[u] + g, op.Sptr[u + 1], p);
#pragma unroll
    for (int off = 16; off >= S; off >>= 1) {
      acc += __shfl_xor_sync(0xffffffffu, acc, off);
      qv += __shfl_xor_sync(0xffffffffu, qv, off);
    }
    if (lane < S) {
      if (op.Qd) {
        const int32_t k = op.ginv[u];
        if (k >= 0) {
          // K-split partial sums of the dense block product, in a fixed order
          for (int t = 0; t < tsplit; ++t) qv += Tout[((int64_t)t * op.ng + k) * S + c];
          if (colsum) qv += (T)(tshift * colsum[c]);
        }
      }
      const T yv = acc + lam * qv;
      Y[i * S + c] = yv;
      if (P) pq[0].add(P[i * S + c], yv);
    }
  }
}

// Dense-block term of the genotyped rows when it is added after the sparse
// part (k_spmv run with the dense term left out, beside the block product):
// Y[p + gmap[k]] += lam (sum of the K-split partials of row k + tshift colsum),
// in a fixed order, and this block's sum_i P[i] (that term) per column into
// pq_part (thread c = tid % S keeps column c; columns >= ncp are not touched).
template <typename T, int S>
__global__ void __launch_bounds__(NT) k_dense_add(OpView<T> op, const T* __restrict__ Tout, int tsplit,
                                                  const double* __restrict__ colsum, double tshift, T lam,
                                                  T* __restrict__ Y, const T* __restrict__ P,
                                                  double* __restrict__ pq_part, const int* __restrict__ active,
                                                  int ncp) {
  if (active && *active == 0) return;
  __shared__ double red[NT];
  const int c = threadIdx.x % S;
  DotAcc<T> pq;
  const double sh = colsum ? tshift * colsum[c] : 0.0;
  const int64_t total = (int64_t)op.ng * S;
  if (c < ncp)
    for (int64_t idx = blockIdx.x * (int64_t)NT + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * NT) {
      const int64_t k = idx / S;
      T q = T(0);
      for (int t = 0; t < tsplit; ++t) q += Tout[((int64_t)t * op.ng + k) * S + c];
      q += (T)sh;
      const T d = lam * q;
      const int64_t i = op.p + op.gmap[k];
      Y[i * S + c] += d;
      if (P) pq.add(P[i * S + c], d);
    }
  const double t = block_sum_cols<S>(pq.value(), red);
  if (pq_part && threadIdx.x < S) pq_part[(int64_t)blockIdx.x * S + c] = t;
}

// Block totals per column of the pq terms left by spmv_random_row: blk[c] for
// every c < S (fixed order: lanes, then warps).
template <int S>
__device__ __forceinline__ void block_sum_row_pq(const double (&pq)[RowLayout<S>::CPL], double* red /*[NT]*/,
                                                 double* blk /*[S]*/) {
  const int tid = threadIdx.x, lane = tid & 31;
  if constexpr (S > 32) {
#pragma unroll
    for (int j = 0; j < S / 32; ++j) {
      red[tid] = pq[j];
      __syncthreads();
      if (tid < 32) {
        double t = 0.0;
        for (int w = 0; w < NT / 32; ++w) t += red[w * 32 + tid];
        blk[32 * j + tid] = t;
      }
      __syncthreads();
    }
  } else {
    const double t = block_sum_cols<S>(lane < S ? pq[0] : 0.0, red);
    if (tid < S) blk[tid] = t;
    __syncthreads();
  }
}

// Y = use_D * D X + lam * [0; Qs X_u + scatter(Tout)]; optional pq partials sum_i P[i]Y[i].
// Tout holds tsplit partial products (ng x S each).  When colsum is given the
// product was taken with the shifted block Qd - tshift, and tshift * colsum[c]
// (colsum: the column sums of the gathered block rows) is added back.
// Blocks [0, nfix) take fixed-effect rows (one block per row); the others take
// random-effect rows, one warp per row, in a grid-stride loop.
template <typename T, int S>
__global__ void __launch_bounds__(NT) k_spmv(OpView<T> op, const T* __restrict__ X,
                                             const T* __restrict__ Tout, int tsplit,
                                             const double* __restrict__ colsum, double tshift,
                                             const int32_t* __restrict__ fix_seg_ptr,
                                             const T* __restrict__ seg_part, T lam, int use_D,
                                             T* __restrict__ Y, const T* __restrict__ P,
                                             double* __restrict__ pq_part,
                                             const int* __restrict__ active, int ncp = S) {
  if (active && *active == 0) return;
  __shared__ double red[NT];
  __shared__ T redT[NT];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t p = op.p;
  const int nfix = (int)p;
  double pq = 0.0;  // this thread's share for column tid % S
  if ((int)blockIdx.x < nfix) {
    // fixed-effect row: sum its segment partials, NT / S groups in parallel,
    // groups combined in a fixed order
    const int64_t i = blockIdx.x;
    constexpr int GS = NT / S;
    const int c = tid % S, g = tid / S;
    T s = T(0);
    if (use_D && c < ncp)
      for (int32_t k = fix_seg_ptr[i] + g; k < fix_seg_ptr[i + 1]; k += GS) s += seg_part[(int64_t)k * S + c];
    redT[tid] = s;
    __syncthreads();
    if (tid >= ncp && tid < S) Y[i * S + tid] = T(0);  // defined, never read
    if (tid < ncp) {
      T t = T(0);
      for (int gg = 0; gg < GS; ++gg) t += redT[gg * S + tid];
      Y[i * S + tid] = t;
      if (P) pq = (double)P[i * S + tid] * (double)t;
    }
  } else {
    // random-effect rows, one warp per row
    DotAcc<T> pqa[RowLayout<S>::CPL];
    const int64_t nwarps = (int64_t)(gridDim.x - nfix) * (NT / 32);
    for (int64_t i = p + (int64_t)(blockIdx.x - nfix) * (NT / 32) + warp; i < op.dim; i += nwarps)
      spmv_random_row<T, S>(op, i, X, Tout, tsplit, colsum, tshift, lam, use_D, Y, P, pqa, lane);
    double pqv[RowLayout<S>::CPL];
#pragma unroll
    for (int j = 0; j < RowLayout<S>::CPL; ++j) pqv[j] = pqa[j].value();
    if (pq_part) {
      __shared__ double blk[S];
      block_sum_row_pq<S>(pqv, red, blk);
      if (tid < S) pq_part[(int64_t)blockIdx.x * S + tid] = blk[tid];
    }
    return;
  }
  // fixed-row block: thread tid < S holds p'q of its row for column tid
  if (pq_part && tid < S) pq_part[(int64_t)blockIdx.x * S + tid] = pq;
}

// r = b - Y, z = M^-1 r on random rows, partial sums of r'r, r'z (random rows) and b'b.
template <typename T, int S>
__global__ void __launch_bounds__(NT) k_init_resid(OpView<T> op, const T* __restrict__ B,
                                                   const T* __restrict__ Y, int have_Y,
                                                   T* __restrict__ R, T* __restrict__ Z,
                                                   double* __restrict__ part /*[grid][3][S]*/) {
  __shared__ double red[NT];
  DotAcc<T> arr, arz, abb;
  const int64_t total = op.dim * S;
  for (int64_t idx = blockIdx.x * (int64_t)NT + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * NT) {
    const int64_t i = idx / S;
    const T b = B[idx];
    const T r = have_Y ? b - Y[idx] : b;
    R[idx] = r;
    arr.add(r, r);
    abb.add(b, b);
    if (i >= op.p) {
      const T z = op.dinv[i - op.p] * r;
      Z[idx] = z;
      arz.add(r, z);
    }
  }
  const double rr = arr.value(), rz = arz.value(), bb = abb.value();
  const int c = threadIdx.x % S;
  double t;
  t = block_sum_cols<S>(rr, red);
  if (threadIdx.x < S) part[((int64_t)blockIdx.x * 3 + 0) * S + c] = t;
  t = block_sum_cols<S>(rz, red);
  if (threadIdx.x < S) part[((int64_t)blockIdx.x * 3 + 1) * S + c] = t;
  t = block_sum_cols<S>(bb, red);
  if (threadIdx.x < S) part[((int64_t)blockIdx.x * 3 + 2) * S + c] = t;
}

// Fixed rows: z_f = A11inv r_f and the partial r_f'z_f.  One block per fixed row,
// of NT_FIXED threads: its NT_FIXED / S groups take every (NT_FIXED / S)-th k and
// are combined in a fixed order.  The kernel is bound by the length of each
// thread's chain of loads: at p = 500, S = 128 (the 200k-animal ssGBLUP step)
// 1024-thread blocks (chains of p / 8) took the step from 65.1 to 63.7 ms against
// 256-thread blocks (chains of p / 2), and one block per 8 rows (chains of p,
// each r_k reused for four rows) made it 68.5 ms.
constexpr int NT_FIXED = 1024;

template <typename T, int S>
__global__ void __launch_bounds__(NT_FIXED) k_fixed(OpView<T> op, const T* __restrict__ R,
                                                    T* __restrict__ Z, const Col* __restrict__ col,
                                                    double* __restrict__ rz_fix /*[p][S]*/) {
  __shared__ T redT[NT_FIXED];
  const int64_t f = blockIdx.x;
  constexpr int G = NT_FIXED / S;
  const int tid = threadIdx.x, c = tid % S, g = tid / S;
  T acc = T(0);
  const int64_t kend = (col == nullptr || col[c].active) ? op.p : 0;  // inactive columns: nothing to do
  for (int64_t k = g; k < kend; k += G) acc += op.A11inv[f * op.p + k] * R[k * S + c];
  redT[tid] = acc;
  __syncthreads();
  if (tid < S) {
    T s = T(0);
    for (int gg = 0; gg < G; ++gg) s += redT[gg * S + tid];
    const bool act = col == nullptr || col[tid].active;
    if (act) Z[f * S + tid] = s;
    const T zf = act ? s : Z[f * S + tid];
    rz_fix[f * S + tid] = (double)R[f * S + tid] * (double)zf;
  }
}

// x += alpha p, r -= alpha q (active, non-skipped columns); partial sums of r'r
// and r'z over the random rows, z = Jacobi r there (computed, not stored: the
// direction update forms it again from r, so Z holds only the fixed rows' z,
// written by k_fixed, after the initial residual).  With Xlo (FP32 only) the
// iterate is a float-float pair x = Xs + Xlo: alpha p is formed exactly as a
// product and its rounding error, and added with a two-sum, so x carries about
// 48 bits although r, z, p and q stay FP32.
template <typename T, int S>
__global__ void __launch_bounds__(NT) k_update(OpView<T> op, const Col* __restrict__ col,
                                               T* __restrict__ Xs, T* __restrict__ Xlo, T* __restrict__ R,
                                               const T* __restrict__ P,
                                               const T* __restrict__ Q,
                                               double* __restrict__ part /*[grid][2][S]*/) {
  __shared__ double red[NT];
  DotAcc<T> arr, arz;
  const int c = threadIdx.x % S;
  const bool act = col[c].active != 0;
  const bool upd = act && !col[c].skip;
  const T alpha = (T)col[c].alpha;
  const int64_t total = op.dim * S;
  for (int64_t idx = blockIdx.x * (int64_t)NT + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * NT) {
    const int64_t i = idx / S;
    T r = R[idx];
    if (upd) {
      if constexpr (sizeof(T) == 4) {
        if (Xlo) {
          // the _rn intrinsics are never contracted into FMAs, which would
          // break the error-free transformations
          const float pv = P[idx];
          const float pr = __fmul_rn(alpha, pv);
          const float pe = fmaf(alpha, pv, -pr);                   // alpha p = pr + pe exactly
          const float xh = Xs[idx];
          const float sh = __fadd_rn(xh, pr);                      // two-sum: xh + pr = sh + se
          const float bv = __fsub_rn(sh, xh);
          const float se = __fadd_rn(__fsub_rn(xh, __fsub_rn(sh, bv)), __fsub_rn(pr, bv));
          const float lo = __fadd_rn(Xlo[idx], __fadd_rn(se, pe));
          const float nh = __fadd_rn(sh, lo);                      // renormalise the pair
          Xlo[idx] = __fsub_rn(lo, __fsub_rn(nh, sh));
          Xs[idx] = nh;
        } else {
          Xs[idx] += alpha * P[idx];
        }
      } else {
        Xs[idx] += alpha * P[idx];
      }
      r -= alpha * Q[idx];
      R[idx] = r;
    }
    arr.add(r, r);
    if (i >= op.p) arz.add(r, op.dinv[i - op.p] * r);
  }
  const double rr = arr.value(), rz = arz.value();
  double t = block_sum_cols<S>(rr, red);
  if (threadIdx.x < S) part[((int64_t)blockIdx.x * 2 + 0) * S + c] = t;
  t = block_sum_cols<S>(rz, red);
  if (threadIdx.x < S) part[((int64_t)blockIdx.x * 2 + 1) * S + c] = t;
}

// p = z + beta p (active columns); z = Z on the fixed rows (k_fixed), Jacobi r on
// the random rows (the same product k_update sums).
template <typename T, int S>
__global__ void __launch_bounds__(NT) k_pupdate(int64_t dim, int64_t nfix, const T* __restrict__ dinv,
                                                const Col* __restrict__ col, const T* __restrict__ R,
                                                const T* __restrict__ Z, T* __restrict__ P) {
  const int c = threadIdx.x % S;
  if (!col[c].active) return;
  const T beta = (T)col[c].beta;
  const int64_t total = dim * S;
  for (int64_t idx = blockIdx.x * (int64_t)NT + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * NT) {
    const int64_t i = idx / S;
    const T z = i < nfix ? Z[idx] : dinv[i - nfix] * R[idx];
    P[idx] = z + beta * P[idx];
  }
}

// Sum of part[b * stride + c] over b < nblk for every column c < S, by all
// threads of the block in a fixed order (deterministic); result in red[c].
template <int S>
__device__ __forceinline__ void col_sums(const double* __restrict__ part, int nblk, int64_t stride,
                                         double* red /*[blockDim]*/) {
  const int t = threadIdx.x;
  const int G = blockDim.x / S;
  const int c = t % S, g = t / S;
  // 16 independent partial sums per thread keep 16 loads in flight; they are
  // combined in a fixed order, so the total does not depend on timing
  constexpr int U = 16;
  double v[U];
#pragma unroll
  for (int u = 0; u < U; ++u) v[u] = 0.0;
  if (g < G) {
    int b = g;
    for (; b + (U - 1) * G < nblk; b += U * G) {
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] += part[(int64_t)(b + u * G) * stride + c];
    }
    for (; b < nblk; b += G) v[0] += part[(int64_t)b * stride + c];
  }
#pragma unroll
  for (int w = U / 2; w > 0; w >>= 1)
#pragma unroll
    for (int u = 0; u < w; ++u) v[u] += v[u + w];
  red[t] = v[0];
  __syncthreads();
  if (t < S) {
    double a = 0.0;
    for (int k = 0; k < G; ++k) a += red[k * S + t];
    red[t] = a;  // safe: red[t] for t < S is only read by thread t itself above
  }
  __syncthreads();
}

// Scalar step after the initial residual: rz, b norm, convergence of x0.
template <int S>
__global__ void k_scalar_init(Col* col, int ncols, const double* part, int nblk,
                              const double* rz_fix, int64_t p, int abs_tol, int* active_count) {
  __shared__ double red[NTS];
  __shared__ double sums[3][S];
  for (int j = 0; j < 3; ++j) {
    col_sums<S>(part + (int64_t)j * S, nblk, 3 * S, red);
    if (threadIdx.x < S) sums[j][threadIdx.x] = red[threadIdx.x];
    __syncthreads();
  }
  col_sums<S>(rz_fix, (int)p, S, red);
  const int c = threadIdx.x;
  int act = 0;
  if (c < S) {
    const double rr = sums[0][c], rz = sums[1][c] + (p > 0 ? red[c] : 0.0), bb = sums[2][c];
    Col s{};
    s.rz = rz;
    s.rr = rr;
    s.bnorm2 = bb;
    s.beta = 0.0;
    s.active = c < ncols ? 1 : 0;
    s.status = c < ncols ? COL_RUNNING : COL_CONVERGED;
    // MatrixFreePCG returns at once when ||r0|| < 1e-20 (matrix_free_pcg.h:31)
    if (c < ncols && abs_tol && sqrt(rr) < 1e-20) { s.active = 0; s.status = COL_CONVERGED; }
    col[c] = s;
    act = s.active;
  }
  const int n_act = __syncthreads_count(act);
  if (c == 0) *active_count = n_act;
}

// alpha = rz / p'Ap, breakdown handling (pcg_solver.h:482-498).
template <int S>
__global__ void k_scalar_alpha(Col* col, const double* pq_part, int nblk) {
  __shared__ double red[NTS];
  col_sums<S>(pq_part, nblk, S, red);
  const int c = threadIdx.x;
  if (c >= S) return;
  Col s = col[c];
  s.skip = 0;
  if (s.active) {
    const double pq = red[c];
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
  col[c] = s;
}

// After the update: convergence test on the recursive residual, beta.
template <int S>
__global__ void k_scalar_beta(Col* col, const double* part, int nblk, const double* rz_fix,
                              int64_t p, const double* tol_col, int abs_tol, int maxit,
                              int* active_count) {
  __shared__ double red[NTS];
  __shared__ double sums[3][S];
  for (int j = 0; j < 2; ++j) {
    col_sums<S>(part + (int64_t)j * S, nblk, 2 * S, red);
    if (threadIdx.x < S) sums[j][threadIdx.x] = red[threadIdx.x];
    __syncthreads();
  }
  col_sums<S>(rz_fix, (int)p, S, red);
  const int c = threadIdx.x;
  int act = 0;
  if (c < S) {
    Col s = col[c];
    if (s.active) {
      const double rr = sums[0][c];
      const double rz = sums[1][c] + (p > 0 ? red[c] : 0.0);
      s.rr = rr;
      if (s.skip) {
        s.beta = 0.0;
        s.rz = rz;
      } else {
        s.iters += 1;
        const double bn = s.bnorm2 > 0 ? sqrt(s.bnorm2) : 1.0;
        const double res = sqrt(rr);
        const double tol = tol_col[c];
        const bool conv = abs_tol ? (res < tol) : (res / bn < tol);
        if (conv) {
          s.active = 0;
          s.status = COL_CONVERGED;
        } else if (!isfinite(rr) || !isfinite(rz)) {
          s.active = 0;
          s.status = COL_NONFINITE;
        } else if (s.iters >= maxit) {
          s.active = 0;
          s.status = COL_MAXIT;
        } else {
          s.beta = rz / s.rz;
          s.rz = rz;
        }
      }
    }
    col[c] = s;
    act = s.active;
  }
  const int n_act = __syncthreads_count(act);
  if (c == 0) *active_count = n_act;
}

// Per-column forms of the two scalar steps of every iteration: one block of
// NTC threads per column sums that column's block partials (in a fixed order:
// strided per thread, then a tree), then thread 0 updates the column.  With
// eight vector blocks per SM the single-block forms above spent ~80 us per
// call reading ~10^5 partials through one SM.
constexpr int NTC = 256;

__device__ __forceinline__ double col_total_c(const double* __restrict__ part, int nblk, int64_t stride, int c,
                                              double* red /*[NTC]*/) {
  double a = 0.0;
  for (int b = threadIdx.x; b < nblk; b += NTC) a += part[(int64_t)b * stride + c];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int o = NTC / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double t = red[0];
  __syncthreads();
  return t;
}

// alpha = rz / p'Ap per column (grid = S blocks), breakdown handling as k_scalar_alpha.
template <int S>
__global__ void __launch_bounds__(NTC) k_scalar_alpha_c(Col* col, const double* pq_part, int nblk) {
  __shared__ double red[NTC];
  const int c = blockIdx.x;
  if (!col[c].active) return;  // uniform over the block
  const double pq = col_total_c(pq_part, nblk, S, c, red);
  if (threadIdx.x != 0) return;
  Col s = col[c];
  s.skip = 0;
  if (s.active) {
    s.pq = pq;
    if (fabs(pq) < 1e-300) {
      if (!s.restarted) {
        s.restarted = 1;
        s.skip = 1;
      } else {
        s.active = 0;
        s.status = COL_BREAKDOWN;
      }
    } else {
      s.alpha = s.rz / pq;
    }
  }
  col[c] = s;
}

// The convergence test and beta per column (grid = S blocks), as k_scalar_beta;
// the block that finishes last counts the active columns into *active_count and
// resets the arrival counter *done (zero before the first launch).
template <int S>
__global__ void __launch_bounds__(NTC) k_scalar_beta_c(Col* col, const double* part, int nblk,
                                                       const double* rz_fix, int64_t p, const double* tol_col,
                                                       int abs_tol, int maxit, int* active_count,
                                                       unsigned* done) {
  __shared__ double red[NTC];
  __shared__ int last;
  const int c = blockIdx.x;
  // an inactive column's partials are not read (uniform over the block)
  const bool was_active = col[c].active != 0;
  const double rr = was_active ? col_total_c(part, nblk, 2 * S, c, red) : 0.0;
  const double rzr = was_active ? col_total_c(part + S, nblk, 2 * S, c, red) : 0.0;
  const double rzf = (was_active && p > 0) ? col_total_c(rz_fix, (int)p, S, c, red) : 0.0;
  if (threadIdx.x == 0) {
    Col s = col[c];
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
        const double tol = tol_col[c];
        const bool conv = abs_tol ? (res < tol) : (res / bn < tol);
        if (conv) {
          s.active = 0;
          s.status = COL_CONVERGED;
        } else if (!isfinite(rr) || !isfinite(rz)) {
          s.active = 0;
          s.status = COL_NONFINITE;
        } else if (s.iters >= maxit) {
          s.active = 0;
          s.status = COL_MAXIT;
        } else {
          s.beta = rz / s.rz;
          s.rz = rz;
        }
      }
    }
    col[c] = s;
    __threadfence();
    last = atomicAdd(done, 1u) == (unsigned)(S - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    int n_act = 0;
    for (int k = 0; k < S; ++k) n_act += __ldcg(&col[k].active);
    *active_count = n_act;
    *done = 0u;
  }
}


// Partial sums of squares per column (interleaved layout).
template <int S>
__global__ void __launch_bounds__(NT) k_colnorm2(const double* __restrict__ V, int64_t dim,
                                                 double* __restrict__ part) {
  __shared__ double red[NT];
  double acc = 0;
  const int64_t total = dim * S;
  for (int64_t idx = blockIdx.x * (int64_t)NT + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * NT)
    acc += V[idx] * V[idx];
  const double t = block_sum_cols<S>(acc, red);
  if (threadIdx.x < S) part[(int64_t)blockIdx.x * S + threadIdx.x] = t;
}

// Record loop: e = y - (X b + Z u) for column 0, partial sums of e'e.
__global__ void k_resid_records(int64_t n_rec, int64_t p, const double* __restrict__ y,
                                const int32_t* __restrict__ aid, int64_t q,
                                const int32_t* __restrict__ xp, const int32_t* __restrict__ xc,
                                const double* __restrict__ xv, const double* __restrict__ sol,
                                double* __restrict__ e, double* __restrict__ part);

}  // namespace sv
}  // namespace cbx
