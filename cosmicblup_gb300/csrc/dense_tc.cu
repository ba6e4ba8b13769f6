// Dense block product on the tensor cores for the FP32 PCG bulk:
//   Tpart[ks][i][c] = sum_{k in split ks} Qd[i][k] * Vt[c][k]      (S = 16, 32 or 64 columns)
// with 3xTF32 splitting (hi*hi + hi*lo + lo*hi, FP32 accumulation in TMEM),
// which keeps FP32-level accuracy on the tf32 tensor path.  The tf32 MMA reads
// an FP32 operand as its 19 high bits (the 13 low mantissa bits are dropped),
// so the staged tiles serve as the hi parts unchanged; the converter warps
// only write the lo parts (a - hi, exact in FP32).  One MMA with N = 2S
// forms A_hi [B_hi | B_lo]; a second (N = S) adds A_lo B_hi into the upper
// half, and the epilogue sums the two halves.
//
// This replaces, for probe blocks, the CUDA-core product of DenseMatrixAdapter /
// SplitMatrixAdapter (reference src/core/matrix_adapter.h:125-127, 252-278)
// applied to every probe of AdaptiveTraceEstimator.  One persistent CTA per SM
// takes an equal contiguous share of the (128-row tile, K step) space (a
// stream-K split: a tile is cut where a CTA's share ends, so every SM gets the
// same number of K steps and a tile has at most a few partial sums):
//   warp 0  TMA producer (SWIZZLE_128B tiles of Qd and Vt),
//   warp 1  TMEM owner and MMA issuer (kind::tf32, M = 128, N = 2S and S),
//   warps 2-5 write the tf32 lo parts of each staged tile to shared memory,
//   warps 6-9 epilogue (TMEM -> partial sums in global memory).
// Each tile's partial sums go to fixed slots (the CTA's rank among those
// covering the tile; the CTA finishing a tile zeroes its unused slots) and are
// summed in slot order by the consumer (k_spmv), so the result is
// deterministic.
#include <cuda.h>
#include <algorithm>
#include <vector>
#include "handle.h"
#include "dense_tc.h"
#include "tma.cuh"

namespace cbx {
namespace dtc {

constexpr int KB = 32;                 // FP32 elements per 128-byte row of a tile
constexpr int A_BYTES = 128 * KB * 4;  // 16 KB
constexpr int THREADS = 320;
constexpr uint32_t TMEM_ALLOC = 512;

// S: the output row stride (the solver's block width); NCM: the most populated
// columns one launch multiplies (S, or 80 for the 128-wide block, whose TMEM
// budget holds two 2 x 80-column accumulators beside the A_lo stages).
template <int S, int NCM = S>
struct Layout {
  static constexpr int B_BYTES = NCM * KB * 4;           // NCM rows of 128 bytes
  // stage: the Qd tile (its tf32 lo part goes to TMEM), then the vector tile
  // as B_hi rows followed by B_lo rows (one N = 2 nc descriptor covers both)
  static constexpr int OFF_B = A_BYTES;
  static constexpr int STAGE = A_BYTES + 2 * B_BYTES;
  static constexpr int NSTAGE = (227 * 1024 - 1280) / STAGE;  // as deep as shared memory allows
  static_assert(STAGE % 1024 == 0, "stages must stay 1024-byte aligned for SWIZZLE_128B");
  static constexpr int OFF_BAR = NSTAGE * STAGE;
  static constexpr int SMEM = OFF_BAR + 256 + 1024;     // + alignment slack
  // TMEM: two accumulator buffers of 2 NCM columns, then 32 columns (one K step
  // of tf32 lo values) per stage
  static constexpr uint32_t ALO_COL = 4 * NCM;
  static_assert(ALO_COL + 32 * NSTAGE <= TMEM_ALLOC, "tensor memory budget");
  static_assert(NSTAGE <= 12, "barrier arrays");
};

struct Bars {
  uint64_t full[12], conv[12], empty[12];
  uint64_t acc_full[2], acc_empty[2], drain;
  uint32_t tmem;
  int abort;
};

__device__ __forceinline__ void umma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__host__ __device__ constexpr uint32_t idesc_tf32(uint32_t M, uint32_t N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

// D[tmem] (+)= A[tmem] * B[smem]^T, kind::tf32 (A: 128 lanes = rows, one
// column per K element)
__device__ __forceinline__ void umma_tf32_ts(uint32_t d, uint32_t a_tmem, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// 32 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
      "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]),
      "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]),
      "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// lo = a - hi with hi = a's 13 low mantissa bits cleared (the tf32 value the
// MMA reads); exact in FP32
__device__ __forceinline__ float4 lo4(const float4& v) {
  const float* p = reinterpret_cast<const float*>(&v);
  float4 lo;
  float* q = reinterpret_cast<float*>(&lo);
#pragma unroll
  for (int e = 0; e < 4; ++e) q[e] = p[e] - __uint_as_float(__float_as_uint(p[e]) & 0xFFFFE000u);
  return lo;
}

template <int S, int NCM = S>
__global__ void __launch_bounds__(THREADS, 1)
    k_dense_tf32(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int ng,
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
      mbar_init(&bars->conv[i], 128);
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

  if (warp == 0) {
    if (lane == 0) {
      uint32_t g = 0;
      bool ok = true;
      const int seg_end = min(total, (int)blockIdx.x * per + per);
      for (int pos = blockIdx.x * per; pos < seg_end && ok;) {
        const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
        pos += k1 - k0;
        for (int k = k0; k < k1; ++k, ++g) {
          const uint32_t s = g % NSTAGE;
          if (!mbar_wait(&bars->empty[s], ((g / NSTAGE) & 1) ^ 1, abort_flag)) { ok = false; break; }
          uint8_t* st = smem + s * LY::STAGE;
          mbar_expect_tx(&bars->full[s], A_BYTES + nc * KB * 4);
          tma_load_2d(smem_addr(st), &tmA, k * KB, mt * 128, &bars->full[s]);
          tma_load_2d(smem_addr(st + LY::OFF_B), &tmB, k * KB, 0, &bars->full[s]);
        }
      }
      if (!ok) fail();
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // N = 2 nc for [B_hi; B_lo] and nc for B_hi (nc populated columns, a multiple of 16)
      const uint32_t ID2 = idesc_tf32(128, 2 * nc), ID1 = idesc_tf32(128, nc);
      uint32_t g = 0, c = 0;
      bool ok = true;
      const int seg_end = min(total, (int)blockIdx.x * per + per);
      for (int pos = blockIdx.x * per; pos < seg_end && ok; ++c) {
        const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
        pos += k1 - k0;
        const uint32_t b = c & 1;
        if (!mbar_wait(&bars->acc_empty[b], ((c >> 1) & 1) ^ 1, abort_flag)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tmem + b * 2 * NCM;
        for (int k = k0; k < k1; ++k, ++g) {
          const uint32_t s = g % NSTAGE;
          if (!mbar_wait(&bars->conv[s], (g / NSTAGE) & 1, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t st = smem_addr(smem + s * LY::STAGE);
          const uint64_t dA = sdesc_sw128(st);
          const uint32_t aLo = tmem + LY::ALO_COL + 32 * s;   // A_lo of this stage in TMEM
          const uint64_t dB = sdesc_sw128(st + LY::OFF_B);  // N = 2 nc rows: B_hi then B_lo
#pragma unroll
          for (int j = 0; j < 4; ++j) {  // four K slices of 8 tf32 (32 bytes) per 128-byte row
            const uint32_t first = (k == k0 && j == 0) ? 0u : 1u;
            umma_tf32(d, dA + 2 * j, dB + 2 * j, ID2, first);        // [A B_hi | A B_lo]
            umma_tf32_ts(d + nc, aLo + 8 * j, dB + 2 * j, ID1, 1u);  // upper half += A_lo B_hi
          }
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
  } else if (warp < 6) {
    // converters: the tf32 lo part of the Qd tile into TMEM (each warp its
    // lane quadrant: thread = one row of 32 K elements), the lo part of the
    // vector tile into shared memory after its hi rows
    const int t = tid - 64;
    const int row = (warp & 3) * 32 + lane;
    uint32_t g = 0;
    bool ok = true;
    const int seg_end = min(total, (int)blockIdx.x * per + per);
    for (int pos = blockIdx.x * per; pos < seg_end && ok;) {
      const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
      pos += k1 - k0;
      for (int k = k0; k < k1; ++k, ++g) {
        const uint32_t s = g % NSTAGE;
        if (!mbar_wait(&bars->full[s], (g / NSTAGE) & 1, abort_flag)) { ok = false; break; }
        uint8_t* st = smem + s * LY::STAGE;
        // row `row` of the SWIZZLE_128B tile: 16-byte chunk c at (c ^ (row & 7)) * 16
        const uint8_t* arow = st + row * 128;
        uint32_t lo[32];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const float4 v = *reinterpret_cast<const float4*>(arow + ((c ^ (row & 7)) << 4));
          const float4 l = lo4(v);
          lo[4 * c] = __float_as_uint(l.x);
          lo[4 * c + 1] = __float_as_uint(l.y);
          lo[4 * c + 2] = __float_as_uint(l.z);
          lo[4 * c + 3] = __float_as_uint(l.w);
        }
        tmem_st32(tmem + (uint32_t((warp & 3) * 32) << 16) + LY::ALO_COL + 32 * s, lo);
        const float4* B = reinterpret_cast<const float4*>(st + LY::OFF_B);
        float4* Bl = reinterpret_cast<float4*>(st + LY::OFF_B + nc * KB * 4);
        for (int i = t; i < nc * KB / 4; i += 128) Bl[i] = lo4(B[i]);
        tmem_st_wait();
        fence_async_smem();
        tc_fence_before();
        mbar_arrive(&bars->conv[s]);
      }
    }
    if (!ok) fail();
  } else {
    // epilogue: TMEM lane quadrant (warp % 4), one output row per thread
    const int q = warp & 3;
    uint32_t c = 0;
    bool ok = true;
    const int seg_end = min(total, (int)blockIdx.x * per + per);
    for (int pos = blockIdx.x * per; pos < seg_end && ok; ++c) {
      const int mt = pos / ksteps, k0 = pos - mt * ksteps, k1 = min(ksteps, k0 + (seg_end - pos));
      pos += k1 - k0;
      // slot: this CTA's rank among the CTAs that cover the tile
      const int ks = (int)blockIdx.x - (mt * ksteps) / per;
      const uint32_t b = c & 1;
      if (!mbar_wait_idle(&bars->acc_full[b], (c >> 1) & 1, abort_flag, 64)) { ok = false; break; }
      tc_fence_after();
      // columns [0, nc): A B_hi; [nc, 2 nc): A B_lo + A_lo B_hi; nc <= NCM.  Each
      // 16-column group is stored as it is read; columns nc .. S - 1 are zero.
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
          // the tile ends here: its slots after this one hold nothing
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

}  // namespace dtc

// Stream-K split of the (tile, K step) space: CTA b takes steps [b per,
// (b + 1) per).  Returns the number of partial slots a tile can need (the
// consumer's split count); per and grid are chosen so that it stays <= 8.
static int stream_k(int64_t ng, int64_t ld, int num_sms, int* grid_out, int* per_out) {
  const int mtiles = (int)((ng + 127) / 128);
  const int ksteps = (int)((ld + dtc::KB - 1) / dtc::KB);
  const int total = mtiles * ksteps;
  int grid = std::max(1, std::min(num_sms, total));
  int per = (total + grid - 1) / grid;
  per = std::max(per, (ksteps + 6) / 7);   // at most 8 CTAs on any tile
  grid = (total + per - 1) / per;
  int nslot = 1;
  for (int t = 0; t < mtiles; ++t) {
    const int first = (t * ksteps) / per, last = ((t + 1) * ksteps - 1) / per;
    nslot = std::max(nslot, last - first + 1);
  }
  if (grid_out) *grid_out = grid;
  if (per_out) *per_out = per;
  return nslot;
}

int dense_tc_ksplit(int64_t ng, int64_t ld, int num_sms) { return stream_k(ng, ld, num_sms, nullptr, nullptr); }
// bf16 tiles are 64 elements wide: the same split over ld / 2
int dense_bf_stream_k(int64_t ng, int64_t ld, int num_sms, int* grid, int* per) {
  return stream_k(ng, (ld + 1) / 2, num_sms, grid, per);
}
int dense_tc_stream_k(int64_t ng, int64_t ld, int num_sms, int* grid, int* per) {
  return stream_k(ng, ld, num_sms, grid, per);
}

void dense_tc(cbx_handle* h, const float* Qd, int64_t ng, int64_t ld, const float* Vt, int S, int ksplit, float* Tpart,
              const int* active, int ncols) {
  CBX_REQUIRE(S == 16 || S == 32 || S == 64 || S == 128, CBX_ERR_ARG, "dense_tc supports 16, 32, 64 or 128 columns");
  // the MMAs and the lo conversion run on the populated columns, rounded up
  // to the MMA granularity of 16; the output's other columns are written as 0
  const int nc = std::min(S, std::max(16, (ncols + 15) / 16 * 16));
  CBX_REQUIRE(S != 128 || nc <= 80, CBX_ERR_ARG, "the 128-wide block product takes at most 80 populated columns");
  CBX_REQUIRE(ld % 4 == 0, CBX_ERR_ARG, "row pitch must be a multiple of 4");
  const CUtensorMap ma = make_map_f32(Qd, ld, ng, 128);
  const CUtensorMap mb = make_map_f32(Vt, ld, S, nc);
  const int ksteps = (int)((ld + dtc::KB - 1) / dtc::KB);
  const int mtiles = (int)((ng + 127) / 128);
  const int total = mtiles * ksteps;
  int grid = 0, per = 0;
  const int nslot = stream_k(ng, ld, h->num_sms, &grid, &per);
  CBX_REQUIRE(nslot == ksplit, CBX_ERR_ARG, "partial slot count does not match dense_tc_ksplit");
  if (S == 128) {
    constexpr int SM = dtc::Layout<128, 80>::SMEM;
    ensure_smem((const void*)dtc::k_dense_tf32<128, 80>, SM, h->device);
    dtc::k_dense_tf32<128, 80><<<grid, dtc::THREADS, SM, h->stream>>>(ma, mb, (int)ng, ksteps, total, per, nslot,
                                                                      Tpart, active, h->status.p, nc);
  } else if (S == 64) {
    constexpr int SM = dtc::Layout<64>::SMEM;
    ensure_smem((const void*)dtc::k_dense_tf32<64>, SM, h->device);
    dtc::k_dense_tf32<64><<<grid, dtc::THREADS, SM, h->stream>>>(ma, mb, (int)ng, ksteps, total, per, nslot, Tpart,
                                                                 active, h->status.p, nc);
  } else if (S == 32) {
    constexpr int SM = dtc::Layout<32>::SMEM;
    ensure_smem((const void*)dtc::k_dense_tf32<32>, SM, h->device);
    dtc::k_dense_tf32<32><<<grid, dtc::THREADS, SM, h->stream>>>(ma, mb, (int)ng, ksteps, total, per, nslot, Tpart,
                                                                 active, h->status.p, nc);
  } else {
    constexpr int SM = dtc::Layout<16>::SMEM;
    ensure_smem((const void*)dtc::k_dense_tf32<16>, SM, h->device);
    dtc::k_dense_tf32<16><<<grid, dtc::THREADS, SM, h->stream>>>(ma, mb, (int)ng, ksteps, total, per, nslot, Tpart,
                                                                 active, h->status.p, nc);
  }
  h->launched("k_dense_tf32");
}

}  // namespace cbx
