// Genomic relationship matrix from PLINK BED on sm_103a tensor cores.
//
// Replaces GrmBuilder::compute(const PlinkReader&) for VanRaden (algorithm 1),
// reference src/core/grm_builder.cpp:63-405.
//
// The reference forms Z (n x m, FP64) with Z_ij = x_ij - mu_j for observed
// calls and 0 for missing ones, then G = Z Z^T / sum_2pq (FP64 GEMM, :351).
// Here the same quantity is computed in integer arithmetic on the f16 tensor
// cores and rounded once at the end.  XX and L are exact; Q uses mu_j^2
// rounded to a multiple of 2^-45, so |G - G_exact| <= n_valid 2^-46 / sum_2pq
// (plus the final rounding) -- below the FP64 GEMM rounding of the reference
// for realistic SNP counts:
//
//   (Z Z^T)_ik = XX_ik - L_ik 2^-29 + Q_ik 2^-45, with
//   XX_ik = sum_j x_ij x_kj                               (integer cross-products)
//   L_ik  = sum_j (x_ij o_kj + o_ij x_kj) a_j,  a_j = mu_j 2^29 (exact, < 2^30)
//   Q_ik  = sum_j o_ij o_kj e_j,                e_j = round(a_j^2 / 2^13) (< 2^47)
//
// o_ij = 1 for an observed call.  mu_j is a float >= 2^-6 (MAF >= 0.01), so
// a_j is an exact integer.  a_j and e_j are split into balanced base-4096
// digits (|digit| <= 2048, exactly representable in f16), so every product
// the tensor core forms is an exact small integer.  Partial sums stay below
// 2^24 within 2048-SNP chunks (FP32-exact); each chunk is flushed into exact
// int64 totals in shared memory while the other TMEM buffer accumulates.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include <cuda_fp16.h>
#include "handle.h"

namespace cbx {
namespace grm {

constexpr int TILE_M = 128;   // samples per tile row block (= TMEM lanes)
constexpr int TILE_N = 32;    // samples per tile column block
constexpr int KSTEP = 32;     // SNPs per operand stage
constexpr int NSTAGE = 3;     // operand stages
constexpr int NRAW = 4;       // raw 2-bit stages
constexpr int CHUNK_STEPS = 64;  // 2048 SNPs per exact FP32 chunk
constexpr int NVAR = 11;      // B-side operand variants
constexpr int NDIG = 7;       // digits per SNP (3 for a_j, 4 for e_j)
constexpr int THREADS = 448;  // 14 warps: MMA, loader, 8 producers, 4 epilogue
constexpr int NPROD = 256;    // producer threads

constexpr int A_TILE_BYTES = TILE_M * KSTEP * 2;                   // 8192
constexpr int B_VAR_BYTES = TILE_N * KSTEP * 2;                    // 2048
constexpr int STAGE_BYTES = 2 * A_TILE_BYTES + NVAR * B_VAR_BYTES; // 38912
constexpr int RAW_A = TILE_M * (KSTEP / 4);                        // 1024
constexpr int RAW_B = TILE_N * (KSTEP / 4);                        // 256
constexpr int RAW_D = NDIG * KSTEP * 2;                            // 448
constexpr int RAW_BYTES = 1792;
constexpr int OFF_STAGE = 0;
constexpr int OFF_RAW = OFF_STAGE + NSTAGE * STAGE_BYTES;          // 116736
constexpr int OFF_XX = OFF_RAW + NRAW * RAW_BYTES;                 // 123904
constexpr int OFF_L = OFF_XX + TILE_N * TILE_M * 4;                // 140288
constexpr int OFF_Q = OFF_L + TILE_N * TILE_M * 8;                 // 173056
constexpr int OFF_BAR = OFF_Q + TILE_N * TILE_M * 8;               // 205824
constexpr int SMEM_BYTES = OFF_BAR + 256;                          // 206080
static_assert(SMEM_BYTES <= 232448, "shared memory budget");

struct Args {
  const uint8_t* xt;    // sample-major 2-bit genotypes, n_pad rows x row_bytes
  const uint16_t* dig;  // f16 digits, [Kp/32][NDIG][32]
  const int2* tiles;    // (row block, column block) per tile
  int ntiles;
  int nsteps;           // Kp / KSTEP
  int64_t row_bytes;    // Kp / 4
  int n;
  double s2pq;
  double* G;            // n x n
  int32_t* xx;          // n x n or null
  int* status;
};

struct Bars {
  uint64_t op_full[NSTAGE];
  uint64_t op_empty[NSTAGE];
  uint64_t raw_full[NRAW];
  uint64_t raw_empty[NRAW];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ void fail(Bars* b, int* status) {
  b->abort = 1;
  atomicExch(status, DEV_TIMEOUT);
}

__device__ __forceinline__ void st_shared_v2(uint32_t addr, uint32_t a, uint32_t b) {
  asm volatile("st.shared.v2.b32 [%0], {%1,%2};" ::"r"(addr), "r"(a), "r"(b) : "memory");
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c,
                                             uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(a), "r"(b), "r"(c),
               "r"(d)
               : "memory");
}

// One BED byte (4 codes, first SNP in the low bits) -> f16 pairs of the
// allele counts x (code 00 -> 2, 10 -> 1, 01 / 11 -> 0) and of the observed
// mask o (code 01 -> 0, else 1): x01 / o01 hold SNPs 0 and 1 (SNP 0 in the low
// half), x23 / o23 SNPs 2 and 3.  Byte permutes pick each f16's high byte from
// a 4-entry table indexed by the code (the low bytes are zero), so the decode
// touches no shared memory.
__device__ __forceinline__ void decode_byte(uint32_t b, uint32_t& x01, uint32_t& x23, uint32_t& o01,
                                            uint32_t& o23) {
  constexpr uint32_t kX = 0x003C0040u;  // high bytes of 2.0, 0, 1.0, 0 by code
  constexpr uint32_t kO = 0x3C3C003Cu;  // high bytes of 1.0, 0, 1.0, 1.0 by code
  const uint32_t s01 = 0x0404u | ((b & 3u) << 4) | (((b >> 2) & 3u) << 12);
  const uint32_t s23 = 0x0404u | (((b >> 4) & 3u) << 4) | (((b >> 6) & 3u) << 12);
  x01 = __byte_perm(kX, 0u, s01);
  x23 = __byte_perm(kX, 0u, s23);
  o01 = __byte_perm(kO, 0u, s01);
  o23 = __byte_perm(kO, 0u, s23);
}

__device__ __forceinline__ uint32_t hmul2u(uint32_t a, uint32_t b) {
  __half2 r = __hmul2(*reinterpret_cast<__half2*>(&a), *reinterpret_cast<__half2*>(&b));
  return *reinterpret_cast<uint32_t*>(&r);
}

__global__ void __launch_bounds__(THREADS, 1) k_grm_tc(Args args) {
  extern __shared__ __align__(1024) uint8_t smem[];
  Bars* bars = reinterpret_cast<Bars*>(smem + OFF_BAR);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;

  if (tid == 0) {
    for (int i = 0; i < NSTAGE; ++i) {
      mbar_init(&bars->op_full[i], NPROD);
      mbar_init(&bars->op_empty[i], 1);
    }
    for (int i = 0; i < NRAW; ++i) {
      mbar_init(&bars->raw_full[i], 32);
      mbar_init(&bars->raw_empty[i], NPROD);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&bars->acc_full[i], 1);
      mbar_init(&bars->acc_empty[i], 4);
    }
    mbar_init(&bars->drain, 1);
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    tmem_alloc(&bars->tmem_base, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = bars->tmem_base;
  volatile int* abort_flag = &bars->abort;
  const int nsteps = args.nsteps;
  const int nchunks = (nsteps + CHUNK_STEPS - 1) / CHUNK_STEPS;

  if (warp == 0) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t ID128 = idesc_f16_f32(128, 128);
      constexpr uint32_t ID96 = idesc_f16_f32(128, 96);
      uint32_t g = 0, c = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < args.ntiles && ok; t += gridDim.x) {
        for (int s = 0; s < nsteps && ok; ++s, ++g) {
          const int sc = s % CHUNK_STEPS;
          const uint32_t b = c & 1;
          if (sc == 0) {
            if (!mbar_wait(&bars->acc_empty[b], ((c >> 1) & 1) ^ 1, abort_flag)) { ok = false; break; }
            tc_fence_after();
          }
          const uint32_t slot = g % NSTAGE;
          if (!mbar_wait(&bars->op_full[slot], (g / NSTAGE) & 1, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t st = smem_addr(smem + OFF_STAGE + slot * STAGE_BYTES);
          const uint32_t aX = st, aO = st + A_TILE_BYTES, bB = st + 2 * A_TILE_BYTES;
          const uint32_t tb = tmem_base + b * 256;
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const uint32_t acc = (sc > 0 || ks > 0) ? 1u : 0u;
            const uint32_t ko = ks * 256;  // two 8-element core matrices along K
            umma_f16(tb + 0, sdesc_noswizzle(aX + ko, 128, 512),
                     sdesc_noswizzle(bB + 0 * B_VAR_BYTES + ko, 128, 512), ID128, acc);
            umma_f16(tb + 32, sdesc_noswizzle(aO + ko, 128, 512),
                     sdesc_noswizzle(bB + 4 * B_VAR_BYTES + ko, 128, 512), ID96, 1u);
            umma_f16(tb + 128, sdesc_noswizzle(aO + ko, 128, 512),
                     sdesc_noswizzle(bB + 7 * B_VAR_BYTES + ko, 128, 512), ID128, acc);
          }
          umma_commit(&bars->op_empty[slot]);
          if (sc == CHUNK_STEPS - 1 || s == nsteps - 1) {
            umma_commit(&bars->acc_full[b]);
            ++c;
          }
        }
      }
      if (!ok) fail(bars, args.status);
      // make sure no MMA is in flight before TMEM is released
      umma_commit(&bars->drain);
      if (!mbar_wait(&bars->drain, 0, abort_flag)) {
        // abort already set; the final wait below is bounded by time only
        const uint64_t t0 = global_ns();
        while (!mbar_try(&bars->drain, 0) && global_ns() - t0 < kWaitLimitNs) {}
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- raw loader (cp.async) ----------------
    uint32_t g = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < args.ntiles && ok; t += gridDim.x) {
      const int2 tl = args.tiles[t];
      const uint8_t* rowA = args.xt + (int64_t)tl.x * TILE_M * args.row_bytes;
      const uint8_t* rowB = args.xt + (int64_t)tl.y * TILE_N * args.row_bytes;
      for (int s = 0; s < nsteps; ++s, ++g) {
        const uint32_t slot = g % NRAW;
        if (!mbar_wait(&bars->raw_empty[slot], ((g / NRAW) & 1) ^ 1, abort_flag)) { ok = false; break; }
        uint8_t* raw = smem + OFF_RAW + slot * RAW_BYTES;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = lane + 32 * q;
          cp_async_8(raw + r * 8, rowA + (int64_t)r * args.row_bytes + s * 8);
        }
        cp_async_8(raw + RAW_A + lane * 8, rowB + (int64_t)lane * args.row_bytes + s * 8);
        if (lane < RAW_D / 16)
          cp_async_16(raw + RAW_A + RAW_B + lane * 16,
                      args.dig + (int64_t)s * NDIG * KSTEP + lane * 8);
        cp_async_arrive(&bars->raw_full[slot]);
      }
    }
    if (!ok) fail(bars, args.status);
    cp_async_wait_all();
  } else if (warp < 2 + NPROD / 32) {
    // ---------------- producers: 2-bit codes -> f16 operand tiles ----------------
    // Eight warps: A side, thread = (row, half of the 32 SNPs); B side, thread =
    // (row, k-group of 8 SNPs, half of it).  Every warp's 16-byte (A) and 8-byte
    // (B) stores cover whole 128-byte lines.
    const int pt = tid - 64;
    uint32_t g = 0;
    bool ok = true;
    const int arow = pt >> 1, ahalf = pt & 1;         // A-side row, SNPs 16*ahalf .. +15
    const int unit = pt >> 1, bhalf = pt & 1;
    const int br = unit & 31;                         // B-side row
    const int bkg = unit >> 5;                        // B-side k-group (8 SNPs)
    for (int t = blockIdx.x; t < args.ntiles && ok; t += gridDim.x) {
      for (int s = 0; s < nsteps; ++s, ++g) {
        const uint32_t rslot = g % NRAW, oslot = g % NSTAGE;
        if (!mbar_wait(&bars->raw_full[rslot], (g / NRAW) & 1, abort_flag)) { ok = false; break; }
        if (!mbar_wait(&bars->op_empty[oslot], ((g / NSTAGE) & 1) ^ 1, abort_flag)) { ok = false; break; }
        const uint8_t* raw = smem + OFF_RAW + rslot * RAW_BYTES;
        const uint32_t st = smem_addr(smem + OFF_STAGE + oslot * STAGE_BYTES);
        // A side: row arow, SNPs 16*ahalf .. 16*ahalf+15 (k-groups 2*ahalf, 2*ahalf+1)
        {
          const uint32_t word = *reinterpret_cast<const uint32_t*>(raw + arow * 8 + ahalf * 4);
          const uint32_t base = (arow >> 3) * 512 + (arow & 7) * 16;
#pragma unroll
          for (int kk = 0; kk < 2; ++kk) {
            const int kg = 2 * ahalf + kk;
            const uint32_t b0 = (word >> (16 * kk)) & 0xFF;
            const uint32_t b1 = (word >> (16 * kk + 8)) & 0xFF;
            uint32_t x0, x1, x2, x3, o0, o1, o2, o3;
            decode_byte(b0, x0, x1, o0, o1);
            decode_byte(b1, x2, x3, o2, o3);
            st_shared_v4(st + base + kg * 128, x0, x1, x2, x3);
            st_shared_v4(st + A_TILE_BYTES + base + kg * 128, o0, o1, o2, o3);
          }
        }
        // B side: row br, SNPs 8*bkg + 4*bhalf .. +3, 11 variants
        {
          const uint32_t b = raw[RAW_A + br * 8 + 2 * bkg + bhalf];
          uint32_t X[2], O[2];
          decode_byte(b, X[0], X[1], O[0], O[1]);
          const uint8_t* dg = raw + RAW_A + RAW_B + bkg * 16 + bhalf * 8;
          const uint32_t vbase =
              st + 2 * A_TILE_BYTES + (br >> 3) * 512 + (br & 7) * 16 + bkg * 128 + bhalf * 8;
          st_shared_v2(vbase, X[0], X[1]);  // variant 0: X
#pragma unroll
          for (int d = 0; d < NDIG; ++d) {
            const uint2 dv = *reinterpret_cast<const uint2*>(dg + d * 64);
            if (d < 3) {
              // variants 1..3: O*d, variants 4..6: X*d
              st_shared_v2(vbase + (1 + d) * B_VAR_BYTES, hmul2u(O[0], dv.x), hmul2u(O[1], dv.y));
              st_shared_v2(vbase + (4 + d) * B_VAR_BYTES, hmul2u(X[0], dv.x), hmul2u(X[1], dv.y));
            } else {
              // variants 7..10: O*e
              st_shared_v2(vbase + (4 + d) * B_VAR_BYTES, hmul2u(O[0], dv.x), hmul2u(O[1], dv.y));
            }
          }
        }
        mbar_arrive(&bars->raw_empty[rslot]);
        fence_async_smem();
        mbar_arrive(&bars->op_full[oslot]);
      }
    }
    if (!ok) fail(bars, args.status);
  } else {
    // ---------------- epilogue: exact chunk flush + final write ----------------
    const int q = warp & 3;
    const int row = q * 32 + lane;
    int32_t* XX = reinterpret_cast<int32_t*>(smem + OFF_XX);
    int64_t* LT = reinterpret_cast<int64_t*>(smem + OFF_L);
    double* QT = reinterpret_cast<double*>(smem + OFF_Q);
    uint32_t c = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < args.ntiles && ok; t += gridDim.x) {
      const int2 tl = args.tiles[t];
      for (int ch = 0; ch < nchunks; ++ch, ++c) {
        const uint32_t b = c & 1;
        if (!mbar_wait_idle(&bars->acc_full[b], (c >> 1) & 1, abort_flag, 1000)) { ok = false; break; }
        tc_fence_after();
        const uint32_t ta = tmem_base + (uint32_t(q * 32) << 16) + b * 256;
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
          uint32_t vx[16], l0[16], l1[16], l2[16];
          tmem_ld16(ta + 0 + 16 * h, vx);
          tmem_ld16(ta + 32 + 16 * h, l0);
          tmem_ld16(ta + 64 + 16 * h, l1);
          tmem_ld16(ta + 96 + 16 * h, l2);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = 16 * h + j;
            const int32_t xi = __float2int_rn(__uint_as_float(vx[j]));
            const int64_t L = (int64_t)__float2int_rn(__uint_as_float(l0[j])) +
                              ((int64_t)__float2int_rn(__uint_as_float(l1[j])) << 12) +
                              ((int64_t)__float2int_rn(__uint_as_float(l2[j])) << 24);
            if (ch == 0) {
              XX[col * TILE_M + row] = xi;
              LT[col * TILE_M + row] = L;
            } else {
              XX[col * TILE_M + row] += xi;
              LT[col * TILE_M + row] += L;
            }
          }
          uint32_t q0[16], q1[16], q2[16], q3[16];
          tmem_ld16(ta + 128 + 16 * h, q0);
          tmem_ld16(ta + 160 + 16 * h, q1);
          tmem_ld16(ta + 192 + 16 * h, q2);
          tmem_ld16(ta + 224 + 16 * h, q3);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = 16 * h + j;
            const int64_t Q = (int64_t)__float2int_rn(__uint_as_float(q0[j])) +
                              ((int64_t)__float2int_rn(__uint_as_float(q1[j])) << 12) +
                              ((int64_t)__float2int_rn(__uint_as_float(q2[j])) << 24) +
                              ((int64_t)__float2int_rn(__uint_as_float(q3[j])) << 36);
            if (ch == 0) QT[col * TILE_M + row] = (double)Q;
            else QT[col * TILE_M + row] += (double)Q;
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars->acc_empty[b]);
      }
      if (!ok) break;
      // final write of this tile (both triangles)
      const int gi = tl.x * TILE_M + row;
      if (gi < args.n) {
        for (int col = 0; col < TILE_N; ++col) {
          const int gk = tl.y * TILE_N + col;
          if (gk >= args.n) break;
          const int32_t xi = XX[col * TILE_M + row];
          const int64_t xl = (int64_t)xi * (int64_t(1) << 29) - LT[col * TILE_M + row];
          const double graw = (double)xl * 0x1p-29 + QT[col * TILE_M + row] * 0x1p-45;
          const double gv = args.s2pq > 0 ? graw / args.s2pq : graw;
          args.G[(int64_t)gi * args.n + gk] = gv;
          args.G[(int64_t)gk * args.n + gi] = gv;
          if (args.xx) {
            args.xx[(int64_t)gi * args.n + gk] = xi;
            args.xx[(int64_t)gk * args.n + gi] = xi;
          }
        }
      }
    }
    if (!ok) fail(bars, args.status);
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem_base, 512);
}

// Per-SNP tallies of 2-bit codes over the first n samples (codes beyond n ignored).
__global__ void k_snp_counts(const uint8_t* __restrict__ payload, int64_t n, int64_t m,
                             int64_t bps, int32_t* n_obs, int32_t* sum_x, int32_t* n_hom1,
                             int32_t* n_het, int32_t* n_hom2) {
  const int64_t j = blockIdx.x;
  if (j >= m) return;
  const uint8_t* row = payload + j * bps;
  int hom1 = 0, het = 0, hom2 = 0;
  for (int64_t b = threadIdx.x; b < bps; b += blockDim.x) {
    const uint32_t v = row[b];
    const int64_t left = n - 4 * b;
    const uint32_t mask = left >= 4 ? 0x55u : (0x55u >> (2 * (4 - left)));
    const uint32_t lo = v & 0x55u, hi = (v >> 1) & 0x55u;
    hom1 += __popc(~lo & ~hi & mask);
    het += __popc(~lo & hi & mask);
    hom2 += __popc(lo & hi & mask);
  }
  __shared__ int red[3][32];
  for (int off = 16; off > 0; off >>= 1) {
    hom1 += __shfl_down_sync(0xffffffffu, hom1, off);
    het += __shfl_down_sync(0xffffffffu, het, off);
    hom2 += __shfl_down_sync(0xffffffffu, hom2, off);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { red[0][w] = hom1; red[1][w] = het; red[2][w] = hom2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0, b2 = 0, c = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { a += red[0][i]; b2 += red[1][i]; c += red[2][i]; }
    if (n_obs) n_obs[j] = a + b2 + c;
    if (sum_x) sum_x[j] = 2 * a + b2;
    if (n_hom1) n_hom1[j] = a;
    if (n_het) n_het[j] = b2;
    if (n_hom2) n_hom2[j] = c;
  }
}

// Transpose the valid SNPs into sample-major 2-bit rows: xt[i][k/4] holds SNP k of
// sample i at bits 2*(k%4).  Samples >= n and SNP columns >= K are code 01 (missing).
__global__ void k_repack(const uint8_t* __restrict__ payload, int64_t n, int64_t bps,
                         const int32_t* __restrict__ valid_idx, int64_t K, int64_t row_bytes,
                         uint8_t* __restrict__ xt) {
  __shared__ uint8_t raw[64][33];
  const int kb = blockIdx.x, ib = blockIdx.y, t = threadIdx.x;
  for (int idx = t; idx < 64 * 32; idx += 128) {
    const int sl = idx >> 5, byte = idx & 31;
    const int64_t k = (int64_t)kb * 64 + sl;
    const int64_t sb = (int64_t)ib * 32 + byte;
    uint8_t v = 0x55;
    if (k < K && sb < bps) v = payload[(int64_t)valid_idx[k] * bps + sb];
    raw[sl][byte] = v;
  }
  __syncthreads();
  const int64_t i = (int64_t)ib * 128 + t;
  uint32_t out[4] = {0, 0, 0, 0};
#pragma unroll 4
  for (int s = 0; s < 64; ++s) {
    uint32_t code = (raw[s][t >> 2] >> (2 * (t & 3))) & 3u;
    if (i >= n) code = 1;
    out[s >> 4] |= code << (2 * (s & 15));
  }
  uint4* dst = reinterpret_cast<uint4*>(xt + i * row_bytes + (int64_t)kb * 16);
  *dst = make_uint4(out[0], out[1], out[2], out[3]);
}

static uint16_t half_bits(int v) {
  __half h = __float2half_rn(static_cast<float>(v));
  return __half_as_ushort(h);
}

static inline int64_t balanced12(int64_t v) { return ((v + 2048) & 4095) - 2048; }

}  // namespace grm
}  // namespace cbx

using namespace cbx;

static const uint8_t* check_bed_bytes(const uint8_t* bed, int64_t bed_bytes, int64_t n, int64_t m) {
  CBX_REQUIRE(bed != nullptr, CBX_ERR_ARG, "bed is null");
  CBX_REQUIRE(n > 0 && m > 0, CBX_ERR_ARG, "Empty dataset provided to GrmBuilder");
  CBX_REQUIRE(n < (int64_t(1) << 31) && m < (int64_t(1) << 31), CBX_ERR_ARG, "n or m too large");
  CBX_REQUIRE(bed_bytes >= 3, CBX_ERR_FORMAT, "Invalid .bed file (too small)");
  CBX_REQUIRE(bed[0] == 0x6C && bed[1] == 0x1B, CBX_ERR_FORMAT, "Invalid .bed file magic number");
  CBX_REQUIRE(bed[2] == 0x01, CBX_ERR_FORMAT, "Only SNP-major mode (0x01) .bed files are supported");
  const int64_t bps = (n + 3) / 4;
  CBX_REQUIRE(bed_bytes >= 3 + m * bps, CBX_ERR_FORMAT,
              ".bed file is truncated: " + std::to_string(bed_bytes) + " < " +
                  std::to_string(3 + m * bps) + " bytes");
  return bed + 3;
}

extern "C" int cbx_bed_snp_counts(cbx_handle* h, const uint8_t* bed, int64_t bed_bytes, int64_t n,
                                  int64_t m, int32_t* n_obs, int32_t* sum_x, int32_t* n_hom1,
                                  int32_t* n_het, int32_t* n_hom2) {
  return cbx_guard(h, [&] {
    const uint8_t* payload = check_bed_bytes(bed, bed_bytes, n, m);
    CBX_CUDA(cudaSetDevice(h->device));
    const int64_t bps = (n + 3) / 4;
    DevBuf<uint8_t> d_bed;
    d_bed.resize(m * bps);
    CBX_CUDA(cudaMemcpyAsync(d_bed.p, payload, m * bps, cudaMemcpyHostToDevice, h->stream));
    DevBuf<int32_t> cnt;
    cnt.resize(5 * m);
    grm::k_snp_counts<<<(unsigned)m, 128, 0, h->stream>>>(d_bed.p, n, m, bps, cnt.p, cnt.p + m,
                                                          cnt.p + 2 * m, cnt.p + 3 * m, cnt.p + 4 * m);
    h->launched("k_snp_counts");
    int32_t* outs[5] = {n_obs, sum_x, n_hom1, n_het, n_hom2};
    for (int i = 0; i < 5; ++i)
      if (outs[i])
        CBX_CUDA(cudaMemcpyAsync(outs[i], cnt.p + i * m, m * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                 h->stream));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
  });
}

extern "C" int cbx_grm_bed(cbx_handle* h, const uint8_t* bed, int64_t bed_bytes, int64_t n, int64_t m,
                           float min_maf, int algorithm, int64_t block_size, double* G,
                           int32_t* xx_counts, float* allele_freqs, double* sum2pq,
                           int64_t* n_valid) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(algorithm == 1, CBX_ERR_UNSUPPORTED,
                "GPU GRM implements algorithm 1 (VanRaden) only; got " + std::to_string(algorithm));
    CBX_REQUIRE(block_size > 0, CBX_ERR_ARG, "block_size must be positive");
    const uint8_t* payload = check_bed_bytes(bed, bed_bytes, n, m);
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const int64_t bps = (n + 3) / 4;

    // 1. per-SNP integer tallies on the device
    DevBuf<uint8_t> d_bed;
    d_bed.resize(m * bps);
    CBX_CUDA(cudaMemcpyAsync(d_bed.p, payload, m * bps, cudaMemcpyHostToDevice, s));
    DevBuf<int32_t> cnt;
    cnt.resize(2 * m);
    grm::k_snp_counts<<<(unsigned)m, 128, 0, s>>>(d_bed.p, n, m, bps, cnt.p, cnt.p + m, nullptr,
                                                  nullptr, nullptr);
    h->launched("k_snp_counts");
    std::vector<int32_t> n_obs(m), sum_x(m);
    CBX_CUDA(cudaMemcpyAsync(n_obs.data(), cnt.p, m * 4, cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaMemcpyAsync(sum_x.data(), cnt.p + m, m * 4, cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));

    // 2. host: validity, float mean / 2pq, blocked sum 2pq (grm_builder.cpp:219-277,353)
    std::vector<int32_t> valid_idx;
    std::vector<float> mean;
    valid_idx.reserve(m);
    double total_sum_2pq = 0.0;
    const double thr = static_cast<double>(min_maf);
    for (int64_t start = 0; start < m; start += block_size) {
      const int64_t end = std::min(start + block_size, m);
      double block_sum = 0.0;
      for (int64_t j = start; j < end; ++j) {
        if (allele_freqs) allele_freqs[j] = -1.0f;
        if (n_obs[j] == 0) continue;
        const double freq = (double)sum_x[j] / (2.0 * n_obs[j]);
        const double maf = std::min(freq, 1.0 - freq);
        if (maf < thr || std::abs(maf) < 1e-8) continue;
        const float two_pq = (float)(1.0f * 2.0 * freq * (1.0 - freq));
        if (allele_freqs) allele_freqs[j] = (float)freq;
        mean.push_back((float)(freq * 2.0));
        valid_idx.push_back((int32_t)j);
        block_sum += two_pq;
      }
      total_sum_2pq += block_sum;
    }
    const int64_t K = (int64_t)valid_idx.size();
    if (sum2pq) *sum2pq = total_sum_2pq;
    if (n_valid) *n_valid = K;

    h->G.resize(n * n);
    h->G_n = n;
    if (K == 0) {
      // no usable SNP: the reference leaves G at zero
      h->G.zero(s);
      if (G) CBX_CUDA(cudaMemsetAsync(h->G.p, 0, n * n * sizeof(double), s));
      if (G) std::memset(G, 0, n * n * sizeof(double));
      if (xx_counts) std::memset(xx_counts, 0, n * n * sizeof(int32_t));
      CBX_CUDA(cudaStreamSynchronize(s));
      return;
    }
    // L stays an exact int64 below 2^53 for up to 2^21 SNPs
    CBX_REQUIRE(K <= 2000000, CBX_ERR_UNSUPPORTED, "more than 2e6 valid SNPs");

    // 3. digits of a_j = mean_j * 2^29 and e_j = round(a_j^2 / 2^13)
    const int64_t Kp = (K + 63) / 64 * 64;
    const int64_t nsteps = Kp / grm::KSTEP;
    std::vector<uint16_t> dig(Kp * grm::NDIG, 0);
    for (int64_t k = 0; k < K; ++k) {
      const double mu = (double)mean[k];
      const double ad = mu * 536870912.0;  // 2^29
      const int64_t a = (int64_t)ad;
      CBX_REQUIRE((double)a == ad && a > 0 && a < (int64_t(1) << 30), CBX_ERR_ARG,
                  "allele mean outside the exact-integer range (MAF filter below 2^-7?)");
      int64_t d[7];
      int64_t r = a;
      d[0] = grm::balanced12(r); r = (r - d[0]) >> 12;
      d[1] = grm::balanced12(r); r = (r - d[1]) >> 12;
      d[2] = r;
      const uint64_t a2 = (uint64_t)a * (uint64_t)a;
      int64_t e = (int64_t)((a2 + (uint64_t(1) << 12)) >> 13);
      d[3] = grm::balanced12(e); e = (e - d[3]) >> 12;
      d[4] = grm::balanced12(e); e = (e - d[4]) >> 12;
      d[5] = grm::balanced12(e); e = (e - d[5]) >> 12;
      d[6] = e;
      CBX_REQUIRE(d[2] >= 0 && d[2] <= 2048 && d[6] >= 0 && d[6] <= 2048, CBX_ERR_ARG,
                  "digit range check failed");
      const int64_t step = k / grm::KSTEP, lane = k % grm::KSTEP;
      for (int q = 0; q < grm::NDIG; ++q)
        dig[(step * grm::NDIG + q) * grm::KSTEP + lane] = grm::half_bits((int)d[q]);
    }

    // 4. upload tables, repack to sample-major 2-bit rows
    const int64_t n_pad = (n + 127) / 128 * 128;
    const int64_t row_bytes = Kp / 4;
    DevBuf<int32_t> d_valid;
    d_valid.resize(K);
    CBX_CUDA(cudaMemcpyAsync(d_valid.p, valid_idx.data(), K * 4, cudaMemcpyHostToDevice, s));
    DevBuf<uint16_t> d_dig;
    d_dig.resize(dig.size());
    CBX_CUDA(cudaMemcpyAsync(d_dig.p, dig.data(), dig.size() * 2, cudaMemcpyHostToDevice, s));
    DevBuf<uint8_t> d_xt;
    d_xt.resize(n_pad * row_bytes);
    grm::k_repack<<<dim3((unsigned)(Kp / 64), (unsigned)(n_pad / 128)), 128, 0, s>>>(
        d_bed.p, n, bps, d_valid.p, K, row_bytes, d_xt.p);
    h->launched("k_repack");

    // 5. tiles of the upper triangle (128-row x 32-column blocks)
    const int nib = (int)(n_pad / 128), njb = (int)(n_pad / 32);
    std::vector<int2> tiles;
    for (int ib = 0; ib < nib; ++ib)
      for (int jb = 4 * ib; jb < njb; ++jb) tiles.push_back(make_int2(ib, jb));
    DevBuf<int2> d_tiles;
    d_tiles.resize(tiles.size());
    CBX_CUDA(cudaMemcpyAsync(d_tiles.p, tiles.data(), tiles.size() * sizeof(int2),
                             cudaMemcpyHostToDevice, s));
    DevBuf<int32_t> d_xx;
    if (xx_counts) d_xx.resize(n * n);

    grm::Args args;
    args.xt = d_xt.p;
    args.dig = d_dig.p;
    args.tiles = d_tiles.p;
    args.ntiles = (int)tiles.size();
    args.nsteps = (int)nsteps;
    args.row_bytes = row_bytes;
    args.n = (int)n;
    args.s2pq = total_sum_2pq;
    args.G = h->G.p;
    args.xx = xx_counts ? d_xx.p : nullptr;
    args.status = h->status.p;
    CBX_CUDA(cudaFuncSetAttribute(grm::k_grm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  grm::SMEM_BYTES));
    const int grid = std::min<int>(h->num_sms, args.ntiles);
    cbx_handle::ProfRec pr{};
    if (h->prof_on) {
      CBX_CUDA(cudaEventCreate(&pr.a));
      CBX_CUDA(cudaEventCreate(&pr.b));
      CBX_CUDA(cudaEventRecord(pr.a, s));
    }
    grm::k_grm_tc<<<grid, grm::THREADS, grm::SMEM_BYTES, s>>>(args);
    h->launched("k_grm_tc");
    if (h->prof_on) {
      CBX_CUDA(cudaEventRecord(pr.b, s));
      pr.bucket = 2;
      // algorithmic integer work 2 n^2 K (the full square of X X^T)
      pr.bytes = 2.0 * (double)n * (double)n * (double)K;
      h->prof.push_back(pr);
    }
    h->check_status("cbx_grm_bed");
    if (G) CBX_CUDA(cudaMemcpyAsync(G, h->G.p, n * n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (xx_counts)
      CBX_CUDA(cudaMemcpyAsync(xx_counts, d_xx.p, n * n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
  });
}
