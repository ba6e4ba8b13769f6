// BF16 dense block product for the FP32 PCG bulk (optional, CBX_BF16=1):
//   Tpart[ks][i][c] = sum_{k in split ks} Qbf[i][k] (Vhi[c][k] + Vlo[c][k])
// with Qbf = bf16(Qd - shift), read at half the bytes of the FP32 block, and the
// gathered vectors as bf16 hi + lo rows (16 significant bits).  The block's
// rounding (2^-9 per entry) perturbs the inner operator, so each refinement
// removes less of the residual (about 1e-3 of it on a scaled single-step problem
// with an exact inner solve, against 1e-7 for the FP32 block); the FP64-accurate
// refinement residuals are unchanged, so the solution is the same to the stopping
// tolerance.
//
// A plain TMA -> tcgen05 pipeline (kind::f16, bf16 operands, FP32 accumulation
// in TMEM): one MMA with N = 2 nc forms A [B_hi | B_lo] per 16 K elements, the
// epilogue adds the two halves.  One persistent CTA per SM over the (128-row
// tile, 64-element K step) space as the 3xTF32 product (stream-K; each tile's
// partial sums go to fixed slots summed in slot order by k_spmv).  Warp roles:
//   0     TMA producer (SWIZZLE_128B bf16 tiles of Qbf and of the vector rows)
//   1     TMEM owner and MMA issuer
//   2-5   epilogue (TMEM -> partial sums in global memory)
#include <cuda.h>
#include <cuda_bf16.h>
#include <algorithm>
#include "handle.h"
#include "dense_tc.h"
#include "tma.cuh"

namespace cbx {
namespace dbf {

constexpr int KB = 64;                 // bf16 elements per 128-byte tile row
constexpr int A_BYTES = 128 * 128;     // 16 KB
constexpr int THREADS = 192;
constexpr uint32_t TMEM_ALLOC = 512;   // two accumulators of 2 NCM <= 160 columns

template <int S, int NCM = S>
struct Layout {
  static constexpr int B_BYTES = 2 * NCM * 128;          // hi rows, then lo rows
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int NSTAGE = std::min(12, (227 * 1024 - 1280) / STAGE);
  static_assert(STAGE % 1024 == 0, "stages must stay 1024-byte aligned for SWIZZLE_128B");
  static constexpr int OFF_BAR = NSTAGE * STAGE;
  static constexpr int SMEM = OFF_BAR + 256 + 1024;
  static_assert(4 * NCM <= (int)TMEM_ALLOC, "tensor memory budget");
};

struct Bars {
  uint64_t full[12], empty[12];
  uint64_t acc_full[2], acc_empty[2], drain;
  uint32_t tmem;
  int abort;
};

// kind::f16 instruction descriptor: A, B bf16, D f32, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

template <int S, int NCM = S>
__global__ void __launch_bounds__(THREADS, 1)
    k_dense_bf16(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int ng,
                 int ksteps, int total, int per, int nslot, float* __restrict__ Tpart, const int* active,
                 int* status, int nc) {
  if (active && *active == 0) return;
  using LY = Layout<S, NCM>;
  constexpr int NSTAGE = LY::NSTAGE;
  extern __shared__ uint8_t dsm_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsm_raw) + 1023) & ~uintptr_t(1023));
  Bars* bars = reinterpret_cast<Bars*>(smem + LY::OFF_BAR);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int i = 0; i < NSTAGE; ++i) {
      mbar_init(&bars->full[i], 1);
      mbar_init(&bars->empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&bars->acc_full[i], 1);
      mbar_init(&bars->acc_empty[i], 4);
    }
    mbar_init(&bars->drain, 1);
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    tmem_alloc(&bars->tmem, TMEM_ALLOC);
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
  const int seg_end = min(total, (int)blockIdx.x * per + per);

  if (warp == 0) {
    if (lane == 0) {
      uint32_t g = 0;
      bool ok = true;
      for (int pos = blockIdx.x * per; pos < seg_end && ok;) {
        const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
        pos += k1 - k0;
        for (int k = k0; k < k1; ++k, ++g) {
          const uint32_t s = g % NSTAGE;
          if (!mbar_wait(&bars->empty[s], ((g / NSTAGE) & 1) ^ 1, abort_flag)) { ok = false; break; }
          uint8_t* st = smem + s * LY::STAGE;
          mbar_expect_tx(&bars->full[s], A_BYTES + 2 * nc * 128);
          tma_load_2d(smem_addr(st), &tmA, k * KB, mt * 128, &bars->full[s]);
          tma_load_2d(smem_addr(st + A_BYTES), &tmB, k * KB, 0, &bars->full[s]);
        }
      }
      if (!ok) fail();
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t ID = idesc_bf16(128, 2 * nc);
      uint32_t g = 0, c = 0;
      bool ok = true;
      for (int pos = blockIdx.x * per; pos < seg_end && ok; ++c) {
        const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
        pos += k1 - k0;
        const uint32_t b = c & 1;
        if (!mbar_wait(&bars->acc_empty[b], ((c >> 1) & 1) ^ 1, abort_flag)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tmem + b * 2 * NCM;
        for (int k = k0; k < k1; ++k, ++g) {
          const uint32_t s = g % NSTAGE;
          if (!mbar_wait(&bars->full[s], (g / NSTAGE) & 1, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t st = smem_addr(smem + s * LY::STAGE);
          const uint64_t dA = sdesc_sw128(st);
          const uint64_t dB = sdesc_sw128(st + A_BYTES);  // 2 nc rows: B_hi then B_lo
#pragma unroll
          for (int j = 0; j < 4; ++j)  // four K slices of 16 bf16 (32 bytes) per 128-byte row
            umma_f16(d, dA + 2 * j, dB + 2 * j, ID, (k == k0 && j == 0) ? 0u : 1u);
          umma_commit(&bars->empty[s]);
        }
        if (!ok) break;
        umma_commit(&bars->acc_full[b]);
      }
      if (!ok) fail();
      umma_commit(&bars->drain);
      const uint64_t t0 = global_ns();
      while (!mbar_try(&bars->drain, 0) && global_ns() - t0 < kWaitLimitNs) {}
    }
    __syncwarp();
  } else {
    // epilogue: TMEM lane quadrant (warp % 4), one output row per thread
    const int q = warp & 3;
    uint32_t c = 0;
    bool ok = true;
    for (int pos = blockIdx.x * per; pos < seg_end && ok; ++c) {
      const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
      pos += k1 - k0;
      const int ks = (int)blockIdx.x - (mt * ksteps) / per;
      const uint32_t b = c & 1;
      if (!mbar_wait_idle(&bars->acc_full[b], (c >> 1) & 1, abort_flag, 64)) { ok = false; break; }
      tc_fence_after();
      // columns [0, nc): A B_hi; [nc, 2 nc): A B_lo; stored as read, nc .. S - 1 zero
      const uint32_t ta = tmem + (uint32_t(q * 32) << 16) + b * 2 * NCM;
      const int row = mt * 128 + q * 32 + lane;
      float4* dst = reinterpret_cast<float4*>(Tpart + ((int64_t)ks * ng + (row < ng ? row : 0)) * S);
#pragma unroll
      for (int j0 = 0; j0 < NCM; j0 += 16) {
        if (j0 < nc) {
          uint32_t r1[16], r2[16];
          tmem_ld16(ta + j0, r1);
          tmem_ld16(ta + nc + j0, r2);
          tmem_ld_wait();
          if (row < ng) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
              dst[j0 / 4 + j] = make_float4(__uint_as_float(r1[4 * j]) + __uint_as_float(r2[4 * j]),
                                            __uint_as_float(r1[4 * j + 1]) + __uint_as_float(r2[4 * j + 1]),
                                            __uint_as_float(r1[4 * j + 2]) + __uint_as_float(r2[4 * j + 2]),
                                            __uint_as_float(r1[4 * j + 3]) + __uint_as_float(r2[4 * j + 3]));
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars->acc_empty[b]);
      if (row < ng) {
        for (int j = nc / 4; j < S / 4; ++j) dst[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k1 == ksteps) {
          for (int z = ks + 1; z < nslot; ++z) {
            float4* zd = reinterpret_cast<float4*>(Tpart + ((int64_t)z * ng + row) * S);
            for (int j = 0; j < S / 4; ++j) zd[j] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
      }
    }
    if (!ok) fail();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, TMEM_ALLOC);
}

// Vhl[c][k] = bf16(v), Vhl[nc + c][k] = bf16(v - bf16(v)) for the first ncols of the
// S gathered FP32 rows of Vt (rows ncols .. nc - 1 zero)
__global__ void k_vt_bf16(const float* __restrict__ Vt, int64_t ld, int ncols, int nc, uint16_t* __restrict__ Vhl) {
  const int64_t total = (int64_t)nc * ld;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / ld;
    const float v = c < ncols ? Vt[idx] : 0.0f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
    Vhl[idx] = __bfloat16_as_ushort(hi);
    Vhl[idx + (int64_t)nc * ld] = __bfloat16_as_ushort(lo);
  }
}

// Qbf = bf16(Q - shift) of the FP64 block (ng x ld row-major); the row padding
// (columns ng .. ld - 1) stays zero
__global__ void k_block_bf16(const double* __restrict__ Q, int64_t ng, int64_t ld, double shift,
                             uint16_t* __restrict__ Qbf) {
  const int64_t n = ng * ld;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    Qbf[i] = i % ld < ng ? __bfloat16_as_ushort(__double2bfloat16(Q[i] - shift)) : (uint16_t)0;
}

}  // namespace dbf

void dense_bf_block(cbx_handle* h, const double* Qd64, int64_t ng, int64_t ld, double shift, uint16_t* Qbf) {
  dbf::k_block_bf16<<<8 * h->num_sms, 256, 0, h->stream>>>(Qd64, ng, ld, shift, Qbf);
  h->launched("k_block_bf16");
}

int dense_bf(cbx_handle* h, const uint16_t* Qbf, int64_t ng, int64_t ld, const float* Vt, int S, uint16_t* Vhl,
             float* Tpart, const int* active, int ncols) {
  CBX_REQUIRE(S == 16 || S == 32 || S == 64 || S == 128, CBX_ERR_ARG, "dense_bf supports 16 to 128 columns");
  const int ncm = S == 128 ? 80 : S;
  const int nc = std::min(ncm, std::max(16, (ncols + 15) / 16 * 16));
  CBX_REQUIRE(ncols <= nc, CBX_ERR_ARG, "too many populated columns for the bf16 block product");
  CBX_REQUIRE(ld % 8 == 0, CBX_ERR_ARG, "bf16 rows must be 16-byte multiples (pitch % 8 == 0)");
  cudaStream_t s = h->stream;
  dbf::k_vt_bf16<<<4 * h->num_sms, 256, 0, s>>>(Vt, ld, ncols, nc, Vhl);
  h->launched("k_vt_bf16");
  const CUtensorMap ma = make_map_bf16(Qbf, ld, ng, 128);
  const CUtensorMap mb = make_map_bf16(Vhl, ld, 2 * nc, 2 * nc);
  int grid = 0, per = 0;
  const int nslot = dense_bf_stream_k(ng, ld, h->num_sms, &grid, &per);
  const int ksteps = (int)((ld + dbf::KB - 1) / dbf::KB);
  const int total = (int)((ng + 127) / 128) * ksteps;
#define CBX_BF(SS, NN)                                                                                         \
  do {                                                                                                         \
    constexpr int SM = dbf::Layout<SS, NN>::SMEM;                                                              \
    ensure_smem((const void*)dbf::k_dense_bf16<SS, NN>, SM, h->device);                                        \
    dbf::k_dense_bf16<SS, NN><<<grid, dbf::THREADS, SM, s>>>(ma, mb, (int)ng, ksteps, total, per, nslot, Tpart, \
                                                             active, h->status.p, nc);                         \
  } while (0)
  switch (S) {
    case 16: CBX_BF(16, 16); break;
    case 32: CBX_BF(32, 32); break;
    case 64: CBX_BF(64, 64); break;
    default: CBX_BF(128, 80); break;
  }
#undef CBX_BF
  h->launched("k_dense_bf16");
  return nslot;
}

}  // namespace cbx
