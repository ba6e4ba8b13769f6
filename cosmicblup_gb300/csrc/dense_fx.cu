// FP64-accurate dense block product on the tensor cores by exact fixed-point
// digits (an Ozaki-style split), for the refinement residuals of the
// mixed-precision PCG: T[i][c] = sum_k A[i][k] v[k][c], A = hi + lo (the FP32
// planes of Qd - shift), v the gathered FP64 columns.
//
// This replaces, for the FP64 residual b - A x of every refinement, the
// CUDA-core float-float product (which is FP32-issue-bound), i.e. the FP64
// dense product of DenseMatrixAdapter / SplitMatrixAdapter (reference
// src/core/matrix_adapter.h:125-127, 252-278) inside PCGSolver::solve.
//
// Scaling: row i of A by 2^(47 - e_i), e_i = 3 + ilogb(max_k |hi_ik|), column c
// of v by 2^(47 - f_c), f_c = 3 + ilogb(max_k |v_kc|); both are rounded to
// integers F with |F| < 2^45 (an error of about 2^-44 of the row / column
// maximum).  Each F is cut into six balanced base-256 digits d_1..d_6 (d_1 the
// most significant, -128 <= d <= 127, exact in f16; |d_1| <= 32 since |F| < 2^45)
// by adding 128 to every digit position and reading the bytes.  Digit products
// d_s(A) d_t(v) are exact integers of at most 2^14; the pairs with s + t = w share
// one FP32 accumulator ("class" w = 2..8, 26 pairs; the pairs with s + t >= 9
// weigh at most 2^-50 of the row and column scales per term and are dropped).  A
// class takes at most 6 pairs, so the tensor core's FP32 sums stay exact integers
// (< 2^24) over chunks of 128 K elements; each chunk is flushed into two exact
// int64 totals per output,
//   I_hi += C_2 2^16 + C_3 2^8 + C_4,   I_lo += C_5 2^24 + C_6 2^16 + C_7 2^8 + C_8,
// and T = 2^(e_i + f_c - 62) (I_hi 2^32 + I_lo), rounded once to FP64 per
// K-split partial.  The partials are summed in a fixed order.
//
// One persistent CTA per SM takes an equal share of the (128-row tile, 32-element
// K step) space, as the 3xTF32 product does.  Warp roles:
//   0      TMA loads of the hi and lo tiles (SWIZZLE_128B FP32)
//   1      TMEM owner, MMA issuer (kind::f16, M = 128, N = (6 - s) nc per A digit)
//   2      bulk loads of the column digits (prepared per call in global memory)
//   3-6    converters: hi/lo rows -> six f16 digit planes of the A tile
//   7-14   epilogue: chunk flush (two warps per TMEM lane quadrant, 16 columns each)
#include <algorithm>
#include <cmath>
#include "handle.h"
#include "dense_tc.h"
#include "tma.cuh"

namespace cbx {
namespace dfx {

inline unsigned blocks_for(int64_t n, int threads, int cap) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cap, (n + threads - 1) / threads));
}

constexpr int KB = 32;          // K elements per step (one 128-byte FP32 tile row)
constexpr int NDIG = 6;         // digits per operand
constexpr int NCLS = 7;         // accumulator classes (digit pairs s + t = 2 .. 8)
constexpr int CHUNK = 4;        // K steps per exact FP32 chunk (128 elements)
constexpr int NCMAX = 32;       // columns per product (TMEM class stride nc = 16 or 32)
constexpr int THREADS = 480;
constexpr int NR = 3, NO = 2;   // raw (hi, lo) stages and operand (digit) stages
constexpr int TILE_F32 = 128 * KB * 4;               // 16 KB
constexpr int RAW_BYTES = 2 * TILE_F32;              // hi + lo
constexpr int PLANE_BYTES = 128 * KB * 2;            // one f16 digit plane of the A tile: 8 KB
constexpr int ADIG_BYTES = NDIG * PLANE_BYTES;       // 48 KB
constexpr int BDIG_MAX = NDIG * NCMAX * KB * 2;      // 12 KB
constexpr int OP_BYTES = ADIG_BYTES + BDIG_MAX;
constexpr int OFF_RAW = 0;
constexpr int OFF_OP = NR * RAW_BYTES;
constexpr int OFF_BAR = OFF_OP + NO * OP_BYTES;
constexpr int SMEM = OFF_BAR + 256 + 1024;
static_assert(SMEM <= 232448, "shared memory budget");
static_assert(RAW_BYTES % 1024 == 0 && OFF_OP % 1024 == 0, "SWIZZLE_128B tiles need 1024-byte alignment");
constexpr uint32_t TMEM_COLS = 512;                  // 2 buffers x 7 classes x nc <= 448
constexpr int64_t DIGIT_BIAS = 0x808080808080LL;     // 128 in each of the six digit bytes

struct Bars {
  uint64_t raw_full[NR], raw_empty[NR], op_full[NO], op_empty[NO];
  uint64_t acc_full[2], acc_empty[2], drain;
  uint32_t tmem;
  int abort;
};

__device__ __forceinline__ uint32_t hadd2u(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("add.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
// 2^n as a float / double (n in the normal range)
__device__ __forceinline__ float pow2f(int n) { return __int_as_float((n + 127) << 23); }
__device__ __forceinline__ double pow2d(int n) { return __longlong_as_double((long long)(n + 1023) << 52); }

// (hi + lo) * sc rounded to an integer F (|F| < 2^45 when |hi sc| < 2^45), returned as
// G = F + DIGIT_BIAS in two words.  All steps are exact FP32 operations but the
// roundings of h0 (when |hi sc| < 2^23) and of lo sc, each at most half a unit.
__device__ __forceinline__ void fixed_point(float hi, float lo, float sc, uint32_t& glo, uint32_t& ghi) {
  const float hs = hi * sc;
  const float h1 = floorf(hs * 0x1p-23f);                        // |h1| < 2^22, exact
  const float h0 = fmaf(h1, -0x1p23f, hs);                       // in [0, 2^23]
  const int i0 = __float_as_int(__fadd_rn(h0, 0x1p23f)) - 0x4B000000;          // round(h0)
  const int i1 = __float_as_int(__fadd_rn(h1, 12582912.0f)) - 0x4B400000;      // h1
  const int il = __float_as_int(__fadd_rn(lo * sc, 12582912.0f)) - 0x4B400000;  // round(lo sc)
  const long long F = ((long long)i1 << 23) + (long long)(i0 + il);
  const unsigned long long G = (unsigned long long)(F + DIGIT_BIAS);
  glo = (uint32_t)G;
  ghi = (uint32_t)(G >> 32);
}
// digit of byte j (0 = least significant) of two elements' G as an f16 pair
// (element a in the low half): byte - 128, exact
__device__ __forceinline__ uint32_t digit_pair(uint32_t ga, uint32_t gb, uint32_t j) {
  const uint32_t u = __byte_perm(ga, gb, j | ((j + 4) << 4));
  const uint32_t v = __byte_perm(u, 0x64646464u, 0x4140);  // f16 1024 + byte in each half
  return hadd2u(v, 0xE480E480u);                           // - 1152
}
// canonical K-major no-swizzle offset of (row r, k) in a tile of 32 K elements (f16)
__host__ __device__ __forceinline__ uint32_t cm_off(int r, int k) {
  return (uint32_t)((r >> 3) * 512 + (r & 7) * 16 + (k >> 3) * 128 + (k & 7) * 2);
}

__global__ void __launch_bounds__(THREADS, 1)
    k_dense_fx(const __grid_constant__ CUtensorMap tmHi, const __grid_constant__ CUtensorMap tmLo,
               const uint16_t* __restrict__ Bd, const int32_t* __restrict__ rowexp, const int32_t* __restrict__ cexp,
               int ng, int ksteps, int total, int per, int nslot, int nc, double* __restrict__ part,
               const int* active, int* status) {
  if (active && *active == 0) return;
  extern __shared__ uint8_t dsm_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsm_raw) + 1023) & ~uintptr_t(1023));
  Bars* bars = reinterpret_cast<Bars*>(smem + OFF_BAR);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bbytes = (uint32_t)(NDIG * nc * KB * 2);
  if (tid == 0) {
    for (int i = 0; i < NR; ++i) {
      mbar_init(&bars->raw_full[i], 1);
      mbar_init(&bars->raw_empty[i], 128);
    }
    for (int i = 0; i < NO; ++i) {
      mbar_init(&bars->op_full[i], 129);
      mbar_init(&bars->op_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&bars->acc_full[i], 1);
      mbar_init(&bars->acc_empty[i], 8);
    }
    mbar_init(&bars->drain, 1);
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    tmem_alloc(&bars->tmem, TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = bars->tmem;
  volatile int* abort_flag = &bars->abort;
  auto fail = [&]() {
    bars->abort = 1;
    atomicExch(status, DEV_TIMEOUT);
  };
  const int seg_begin = (int)blockIdx.x * per;
  const int seg_end = min(total, seg_begin + per);

  if (warp == 0) {
    // ---------------- TMA: hi and lo tiles ----------------
    if (lane == 0) {
      uint32_t g = 0;
      bool ok = true;
      for (int pos = seg_begin; pos < seg_end && ok;) {
        const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
        pos += k1 - k0;
        for (int k = k0; k < k1; ++k, ++g) {
          const uint32_t r = g % NR;
          if (!mbar_wait(&bars->raw_empty[r], ((g / NR) & 1) ^ 1, abort_flag)) { ok = false; break; }
          const uint32_t dst = smem_addr(smem + OFF_RAW + r * RAW_BYTES);
          mbar_expect_tx(&bars->raw_full[r], RAW_BYTES);
          tma_load_2d(dst, &tmHi, k * KB, mt * 128, &bars->raw_full[r]);
          tma_load_2d(dst + TILE_F32, &tmLo, k * KB, mt * 128, &bars->raw_full[r]);
        }
      }
      if (!ok) fail();
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t g = 0, c = 0;
      bool ok = true;
      for (int pos = seg_begin; pos < seg_end && ok;) {
        const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
        pos += k1 - k0;
        uint32_t b = 0;
        for (int k = k0; k < k1; ++k, ++g) {
          const int ci = (k - k0) % CHUNK;
          if (ci == 0) {
            b = c & 1;
            if (!mbar_wait(&bars->acc_empty[b], ((c >> 1) & 1) ^ 1, abort_flag)) { ok = false; break; }
            tc_fence_after();
          }
          const uint32_t o = g % NO;
          if (!mbar_wait(&bars->op_full[o], (g / NO) & 1, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t op = smem_addr(smem + OFF_OP + o * OP_BYTES);
          const uint32_t d = tmem + b * (NCLS * nc);
          const uint32_t plane_b = (uint32_t)(nc * KB * 2);  // bytes of one column-digit plane
#pragma unroll
          for (int kh = 0; kh < 2; ++kh) {
            const uint32_t acc0 = (ci == 0 && kh == 0) ? 0u : 1u;  // 0: the chunk's first K half
            const uint64_t dB = sdesc_noswizzle(op + ADIG_BYTES + kh * 256, 128, 512);
            // A digit pl against column digits 0 .. min(5, 6 - pl): classes pl .. pl + n - 1.
            // Digit 0 opens classes 0..5 of a chunk and the pair (1, 5) opens class 6.
            umma_f16(d, sdesc_noswizzle(op + kh * 256, 128, 512), dB, idesc_f16_f32(128, 6 * nc), acc0);
            const uint64_t dA1 = sdesc_noswizzle(op + PLANE_BYTES + kh * 256, 128, 512);
            umma_f16(d + nc, dA1, dB, idesc_f16_f32(128, 5 * nc), 1u);
            umma_f16(d + 6 * nc, dA1, sdesc_noswizzle(op + ADIG_BYTES + 5 * plane_b + kh * 256, 128, 512),
                     idesc_f16_f32(128, nc), acc0);
#pragma unroll
            for (int pl = 2; pl < NDIG; ++pl) {
              const uint64_t dA = sdesc_noswizzle(op + pl * PLANE_BYTES + kh * 256, 128, 512);
              umma_f16(d + pl * nc, dA, dB, idesc_f16_f32(128, (NCLS - pl) * nc), 1u);
            }
          }
          umma_commit(&bars->op_empty[o]);
          if (ci == CHUNK - 1 || k == k1 - 1) {
            umma_commit(&bars->acc_full[b]);
            ++c;
          }
        }
      }
      if (!ok) fail();
      umma_commit(&bars->drain);
      const uint64_t t0 = global_ns();
      while (!mbar_try(&bars->drain, 0) && global_ns() - t0 < kWaitLimitNs) {}
    }
    __syncwarp();
  } else if (warp == 2) {
    // ---------------- column digits: bulk copies ----------------
    if (lane == 0) {
      uint32_t g = 0;
      bool ok = true;
      for (int pos = seg_begin; pos < seg_end && ok;) {
        const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
        pos += k1 - k0;
        for (int k = k0; k < k1; ++k, ++g) {
          const uint32_t o = g % NO;
          if (!mbar_wait(&bars->op_empty[o], ((g / NO) & 1) ^ 1, abort_flag)) { ok = false; break; }
          mbar_expect_tx(&bars->op_full[o], bbytes);
          bulk_load(smem_addr(smem + OFF_OP + o * OP_BYTES + ADIG_BYTES),
                    reinterpret_cast<const uint8_t*>(Bd) + (size_t)k * bbytes, bbytes, &bars->op_full[o]);
        }
      }
      if (!ok) fail();
    }
    __syncwarp();
  } else if (warp < 7) {
    // ---------------- converters: one tile row per thread ----------------
    const int row = tid - 96;
    uint32_t g = 0;
    bool ok = true;
    for (int pos = seg_begin; pos < seg_end && ok;) {
      const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
      pos += k1 - k0;
      const int gr = mt * 128 + row;
      const float sc = pow2f(47 - (gr < ng ? rowexp[gr] : 0));
      for (int k = k0; k < k1; ++k, ++g) {
        const uint32_t r = g % NR, o = g % NO;
        if (!mbar_wait(&bars->raw_full[r], (g / NR) & 1, abort_flag)) { ok = false; break; }
        if (!mbar_wait(&bars->op_empty[o], ((g / NO) & 1) ^ 1, abort_flag)) { ok = false; break; }
        const uint8_t* rh = smem + OFF_RAW + r * RAW_BYTES + row * 128;
        const uint8_t* rl = rh + TILE_F32;
        const uint32_t ob = smem_addr(smem + OFF_OP + o * OP_BYTES) + cm_off(row, 0);
#pragma unroll
        for (int kg = 0; kg < 4; ++kg) {
          uint32_t gl[8], gh[8];
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            const int ch = 2 * kg + hh;  // 16-byte chunk of the swizzled 128-byte row
            const float4 a = *reinterpret_cast<const float4*>(rh + ((ch ^ (row & 7)) << 4));
            const float4 l = *reinterpret_cast<const float4*>(rl + ((ch ^ (row & 7)) << 4));
            fixed_point(a.x, l.x, sc, gl[4 * hh + 0], gh[4 * hh + 0]);
            fixed_point(a.y, l.y, sc, gl[4 * hh + 1], gh[4 * hh + 1]);
            fixed_point(a.z, l.z, sc, gl[4 * hh + 2], gh[4 * hh + 2]);
            fixed_point(a.w, l.w, sc, gl[4 * hh + 3], gh[4 * hh + 3]);
          }
#pragma unroll
          for (int pl = 0; pl < NDIG; ++pl) {
            const int j = 5 - pl;  // digit pl is byte 5 - pl of G
            uint32_t w[4];
#pragma unroll
            for (int e = 0; e < 4; ++e)
              w[e] = j < 4 ? digit_pair(gl[2 * e], gl[2 * e + 1], j) : digit_pair(gh[2 * e], gh[2 * e + 1], j - 4);
            st_shared_v4(ob + pl * PLANE_BYTES + kg * 128, w[0], w[1], w[2], w[3]);
          }
        }
        fence_async_smem();
        mbar_arrive(&bars->op_full[o]);
        mbar_arrive(&bars->raw_empty[r]);
      }
    }
    if (!ok) fail();
  } else {
    // ---------------- epilogue ----------------
    const int q = warp & 3;
    const int j0 = ((warp - 7) >> 2) * 16;  // this warp's 16 columns
    const bool mine = j0 < nc;
    uint32_t c = 0;
    bool ok = true;
    for (int pos = seg_begin; pos < seg_end && ok;) {
      const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
      pos += k1 - k0;
      const int ks = (int)blockIdx.x - (mt * ksteps) / per;  // this CTA's partial slot for the tile
      long long Ihi[16], Ilo[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) Ihi[j] = Ilo[j] = 0;
      const int nch = (k1 - k0 + CHUNK - 1) / CHUNK;
      for (int ch = 0; ch < nch; ++ch, ++c) {
        const uint32_t b = c & 1;
        if (!mbar_wait_idle(&bars->acc_full[b], (c >> 1) & 1, abort_flag, 32)) { ok = false; break; }
        tc_fence_after();
        if (mine) {
          const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + b * (NCLS * nc) + j0;
#pragma unroll
          for (int ci = 0; ci < NCLS; ++ci) {
            uint32_t rr[16];
            tmem_ld16(ta + ci * nc, rr);
            tmem_ld_wait();
            const int sh = ci < 3 ? (2 - ci) * 8 : (6 - ci) * 8;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const long long v = (long long)__float2int_rn(__uint_as_float(rr[j])) << sh;
              if (ci < 3) Ihi[j] += v;
              else Ilo[j] += v;
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars->acc_empty[b]);
      }
      if (!ok) break;
      const int row = mt * 128 + q * 32 + lane;
      if (mine && row < ng) {
        const int e = rowexp[row];
        double* dst = part + ((size_t)ks * ng + row) * NCMAX + j0;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const double t = fma((double)Ihi[j], 0x1p32, (double)Ilo[j]);
          const int n = e + cexp[j0 + j] - 62;
          dst[j] = (n > -1000 && n < 1000) ? t * pow2d(n) : ldexp(t, n);
        }
        if (k1 == ksteps) {
          // the tile ends here: its later slots hold nothing
          for (int z = ks + 1; z < nslot; ++z) {
            double* zd = part + ((size_t)z * ng + row) * NCMAX + j0;
#pragma unroll
            for (int j = 0; j < 16; ++j) zd[j] = 0.0;
          }
        }
      }
    }
    if (!ok) fail();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, TMEM_COLS);
}

// e_i = 3 + ilogb(max_k |hi_ik|) (0 for a zero row), clamped so that 2^(47 - e)
// stays a normal float.
__global__ void k_fx_rowexp(const float* __restrict__ qh, int64_t ng, int64_t ld, int32_t* __restrict__ rowexp) {
  __shared__ float red[256];
  const int64_t i = blockIdx.x;
  float m = 0.0f;
  for (int64_t k = threadIdx.x; k < ld; k += blockDim.x) m = fmaxf(m, fabsf(qh[i * ld + k]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) rowexp[i] = red[0] > 0.0f ? min(170, max(-80, ilogbf(red[0]) + 3)) : 0;
}

// f_c = 3 + ilogb(max_k |v_kc|) for c < ncols, 0 otherwise (and for a zero column)
__global__ void k_fx_colexp(const double* __restrict__ X, int xs, int64_t p, const int32_t* __restrict__ gmap,
                            int64_t ng, int ncols, int32_t* __restrict__ cexp) {
  __shared__ double red[256];
  const int c = blockIdx.x;
  double m = 0.0;
  if (c < ncols)
    for (int64_t k = threadIdx.x; k < ng; k += blockDim.x) m = fmax(m, fabs(X[(p + gmap[k]) * xs + c]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) cexp[c] = red[0] > 0.0 ? min(1000, max(-1000, ilogb(red[0]) + 3)) : 0;
}

// Column digits in the K-step blocks the product loads: block k (6 nc 64 bytes)
// holds digit plane t (t = 0 most significant) of columns 0 .. nc - 1 at t nc 64,
// element (c, kk) at cm_off(c, kk).  One thread per (K step, column, 8 K elements).
__global__ void k_fx_vdigits(const double* __restrict__ X, int xs, int64_t p, const int32_t* __restrict__ gmap,
                             int64_t ng, int ncols, int nc, int ksteps, const int32_t* __restrict__ cexp,
                             uint16_t* __restrict__ Bd) {
  const int64_t total = (int64_t)ksteps * nc * 4;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int kg = (int)(idx & 3);
    const int c = (int)((idx >> 2) % nc);
    const int ks = (int)(idx / (4 * nc));
    const double sc = c < ncols ? pow2d(47 - cexp[c]) : 0.0;
    uint32_t gl[8], gh[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int64_t k = (int64_t)ks * KB + kg * 8 + e;
      const double v = (c < ncols && k < ng) ? X[(p + gmap[k]) * xs + c] : 0.0;
      const long long F = __double2ll_rn(v * sc);
      const unsigned long long G = (unsigned long long)(F + DIGIT_BIAS);
      gl[e] = (uint32_t)G;
      gh[e] = (uint32_t)(G >> 32);
    }
    uint8_t* blk = reinterpret_cast<uint8_t*>(Bd) + (size_t)ks * (NDIG * nc * KB * 2);
#pragma unroll
    for (int pl = 0; pl < NDIG; ++pl) {
      const int j = 5 - pl;
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 4; ++e)
        w[e] = j < 4 ? digit_pair(gl[2 * e], gl[2 * e + 1], j) : digit_pair(gh[2 * e], gh[2 * e + 1], j - 4);
      *reinterpret_cast<uint4*>(blk + pl * nc * KB * 2 + cm_off(c, kg * 8)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// Tout[i * os + c] = sum of the partial slots in slot order (c < ncols)
__global__ void k_fx_reduce(const double* __restrict__ part, int nslot, int64_t ng, int ncols,
                            double* __restrict__ Tout, int os, const int* active) {
  if (active && *active == 0) return;
  const int64_t total = ng * ncols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / ncols;
    const int c = (int)(idx - i * ncols);
    double s = 0.0;
    for (int z = 0; z < nslot; ++z) s += part[((size_t)z * ng + i) * NCMAX + c];
    Tout[i * os + c] = s;
  }
}

}  // namespace dfx

void fx_row_scales(cbx_handle* h, const float* qh, int64_t ng, int64_t ld, int32_t* rowexp) {
  dfx::k_fx_rowexp<<<(unsigned)ng, 256, 0, h->stream>>>(qh, ng, ld, rowexp);
  h->launched("k_fx_rowexp");
}

void fx_product(cbx_handle* h, const float* qh, const float* ql, const int32_t* rowexp, int64_t ng, int64_t ld,
                const double* X, int xs, int64_t p, const int32_t* gmap, int ncols, DevBuf<uint16_t>& bdig,
                DevBuf<int32_t>& cexp, DevBuf<double>& part, double* Tout, int os, const int* active) {
  CBX_REQUIRE(ncols >= 1 && ncols <= dfx::NCMAX, CBX_ERR_ARG, "fx_product takes 1 to 32 columns");
  CBX_REQUIRE(ld % 4 == 0 && ng > 0 && ng <= INT32_MAX, CBX_ERR_ARG, "bad block shape");
  cudaStream_t s = h->stream;
  const int nc = ncols <= 16 ? 16 : 32;
  const int ksteps = (int)((ld + dfx::KB - 1) / dfx::KB);
  const int mtiles = (int)((ng + 127) / 128);
  const int total = mtiles * ksteps;
  int grid = 0, per = 0;
  const int nslot = dense_tc_stream_k(ng, ld, h->num_sms, &grid, &per);
  bdig.resize((size_t)ksteps * dfx::NDIG * nc * dfx::KB);
  cexp.resize(dfx::NCMAX);
  part.resize((size_t)nslot * ng * dfx::NCMAX);
  dfx::k_fx_colexp<<<nc, 256, 0, s>>>(X, xs, p, gmap, ng, ncols, cexp.p);
  h->launched("k_fx_colexp");
  dfx::k_fx_vdigits<<<dfx::blocks_for((int64_t)ksteps * nc * 4, 256, 4 * h->num_sms), 256, 0, s>>>(
      X, xs, p, gmap, ng, ncols, nc, ksteps, cexp.p, bdig.p);
  h->launched("k_fx_vdigits");
  const CUtensorMap mh = make_map_f32(qh, ld, ng, 128);
  const CUtensorMap ml = make_map_f32(ql, ld, ng, 128);
  ensure_smem((const void*)dfx::k_dense_fx, dfx::SMEM, h->device);
  dfx::k_dense_fx<<<grid, dfx::THREADS, dfx::SMEM, s>>>(mh, ml, bdig.p, rowexp, cexp.p, (int)ng, ksteps, total, per,
                                                       nslot, nc, part.p, active, h->status.p);
  h->launched("k_dense_fx");
  dfx::k_fx_reduce<<<dfx::blocks_for(ng * ncols, 256, 8 * h->num_sms), 256, 0, s>>>(part.p, nslot, ng, ncols, Tout, os,
                                                                            active);
  h->launched("k_fx_reduce");
}

}  // namespace cbx
