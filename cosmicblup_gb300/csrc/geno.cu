// Genotype matrix-free products from PLINK BED on the device.
//
// Replaces PlinkReader's RHE / PCG support (reference src/core/plink_reader.cpp):
//   computeStats  (:186-237)  per-SNP mean of the observed calls, p = mean / 2,
//                             var = 2p(1-p), inv_std = 1/sqrt(var), or 0 when
//                             var < 1e-9 or no call is observed;
//   multiply_Z_v  (:239-293)  y = Z v, every term (x - mean_j) v_j inv_std_j rounded
//                             to float first, as the reference's per-SNP val_map is;
//   multiply_Zt_v (:341-392)  y_j = (sum_obs x_ij v_i - mean_j sum_obs v_i) inv_std_j;
// and the SNP-effect back-solve of the result writer (src/solve/result_writer.cpp:
// 565-623, the --bfile branch): q = G^-1 u_g, effect_j = ((Z^T q)_j / inv_std_j) /
// total_2pq with total_2pq = the sum of var over SNPs with var >= 1e-9.
//
// The sums are exact.  The FP64 input vector is scaled by a power of two 2^s, chosen
// so that the sum of its magnitudes stays below 2^61, and rounded to int64.  The
// device adds int64 values modulo 2^64, so neither the order of the additions nor
// that of the atomics changes a bit of the result, and partial sums may wrap; the
// totals fit and are scaled back once.  The only rounding is the conversion of each
// input, at most 2^-(s+1) per term: the total error is below n 2^-62 sum|v|, far
// below that of the reference's sequential FP64 sums.
//
// Codes (2 bits, first sample in the low bits): 00 -> x = 2, 01 -> missing,
// 10 -> x = 1, 11 -> x = 0.  With lo / hi the two bits and k = lo + hi, every
// observed call has x = 2 - k (a missing call has k = 1).  So one SNP needs a single
// dense sum S = sum_i k_i v_i plus M = the sum of v over its missing calls, taken
// from a sparse list built once:
//   sum_obs x v = 2T - S - M,   sum_obs v = T - M,
// with T the sum of v over all samples.  Z v needs, per SNP j, w0_j for every
// sample, k (w2_j - w0_j) and, where both bits are set, w3_j - 2 w2_j + w0_j (w_c =
// the float term of code c, which is not linear in x); a missing call then receives
// w2_j, which the sample-major missing list takes back out.  Missing calls are rare
// in genotype data: the dense passes cost a few integer operations per code, the
// sparse ones one gather per missing call.
//
// The k-weighted sums run on the integer multiply path instead of as masked adds.
// For one 32-bit word of 16 codes, kw = (w & 0x55..) + ((w >> 1) & 0x55..) holds the
// k_t in 2-bit fields, and with a_t = kw >> 2t (so that k_t = a_t - 4 a_{t+1}, a_16 = 0)
//   sum_t k_t v_t = sum_t a_t (v_t - 4 v_{t-1})      (v_{-1} = 0),
// one 32 x 64-bit multiply-add per code against u_t = v_t - 4 v_{t-1}, precomputed per
// 16-sample word; modulo 2^64 it is two multiply-adds (the low word widening, the high
// word 32-bit).  Z v telescopes over the accumulators instead: P_t = sum_j a_t(j) d_j
// gives sum_j k_t(j) d_j = P_t - 4 P_{t+1}.
//
// Layout: the payload is copied once into rows of `pitch` bytes (a multiple of 16,
// the padding bytes zero).  Samples at or beyond n get v = 0 (Z^T v) or are dropped
// (Z v), so the padding codes never reach a result; the missing lists hold calls of
// samples below n only.
#include <algorithm>
#include <cmath>
#include <vector>
#include <cublas_v2.h>
#include "dense.h"
#include "handle.h"
#include "pcg.h"
#include "tune.h"

namespace cbx {
namespace geno {

constexpr int ZT_THREADS = 256;   // one SNP row per thread
constexpr int Z_THREADS = 256;    // 16 samples (one 32-bit word) per thread
constexpr int Z_MAX_ROWS = 2048;  // SNP rows per CTA (48 KB of deltas in shared memory)
constexpr int PREP_THREADS = 1024;

// Deterministic block sum of a double (fixed shuffle tree, then warp 0 over the warps).
__device__ double block_sum_f64(double a, double* red) {
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = a;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

__device__ unsigned long long block_sum_u64(unsigned long long a, unsigned long long* red) {
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = a;
  __syncthreads();
  unsigned long long r = 0;
  if (w == 0) {
    r = l < (int)(blockDim.x >> 5) ? red[l] : 0ull;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

// Scale exponent for a sum of magnitudes S: S 2^s < 2^61.
__device__ int fix_exponent(double S) {
  if (!(S > 0.0)) return 0;
  int e = 0;
  frexp(S, &e);  // S = f 2^e, 0.5 <= f < 1
  return 61 - e;
}

// computeStats for one SNP row per block (plink_reader.cpp:192-236).
// Also counts the SNP's missing calls (miss_cnt) for the sparse missing lists.
__global__ void k_geno_stats(const uint8_t* __restrict__ bed, int64_t pitch, int64_t n, int64_t m,
                             double* __restrict__ mean, double* __restrict__ inv_std,
                             double* __restrict__ var2pq, int32_t* __restrict__ miss_cnt) {
  const int64_t j = blockIdx.x;
  if (j >= m) return;
  const uint32_t* row = reinterpret_cast<const uint32_t*>(bed + j * pitch);
  const int64_t nw = (n + 15) / 16;
  int hom1 = 0, het = 0, hom2 = 0, miss = 0;
  for (int64_t t = threadIdx.x; t < nw; t += blockDim.x) {
    const uint32_t v = row[t];
    const int64_t valid = n - 16 * t;  // >= 1
    const uint32_t mask = valid >= 16 ? 0x55555555u : (0x55555555u >> (2 * (16 - valid)));
    const uint32_t lo = v & 0x55555555u, hi = (v >> 1) & 0x55555555u;
    hom1 += __popc(~lo & ~hi & mask);
    het += __popc(~lo & hi & mask);
    hom2 += __popc(lo & hi & mask);
    miss += __popc(lo & ~hi & mask);
  }
  for (int o = 16; o > 0; o >>= 1) {
    hom1 += __shfl_down_sync(0xffffffffu, hom1, o);
    het += __shfl_down_sync(0xffffffffu, het, o);
    hom2 += __shfl_down_sync(0xffffffffu, hom2, o);
    miss += __shfl_down_sync(0xffffffffu, miss, o);
  }
  __shared__ int red[4][32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { red[0][w] = hom1; red[1][w] = het; red[2][w] = hom2; red[3][w] = miss; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  int a = 0, b = 0, c = 0, d = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
    a += red[0][i]; b += red[1][i]; c += red[2][i]; d += red[3][i];
  }
  miss_cnt[j] = d;
  const int count = a + b + c;
  double mu = 0.0, is = 0.0, v2 = 0.0;
  if (count > 0) {
    // the reference sums the float codes 2, 1, 0 in double: an exact integer
    mu = __ddiv_rn((double)(2 * a + b), (double)count);
    const double p = __ddiv_rn(mu, 2.0);
    const double var = __dmul_rn(__dmul_rn(2.0, p), __dsub_rn(1.0, p));
    if (!(var < 1e-9)) {
      is = __ddiv_rn(1.0, __dsqrt_rn(var));
      v2 = var;
    }
  }
  mean[j] = mu;
  inv_std[j] = is;
  var2pq[j] = v2;
}

// total_2pq of the back-solve (result_writer.cpp:604-609): one block, fixed order.
__global__ void __launch_bounds__(PREP_THREADS) k_geno_total(const double* __restrict__ var2pq, int64_t m,
                                                            double* __restrict__ out) {
  __shared__ double red[32];
  double a = 0.0;
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) a += var2pq[j];
  a = block_sum_f64(a, red);
  if (threadIdx.x == 0) *out = a;
}

// Exclusive prefix sum of len int32 counts into ptr[0..len] (one block, fixed order).
__global__ void __launch_bounds__(PREP_THREADS) k_geno_scan(const int32_t* __restrict__ cnt, int64_t len,
                                                           int64_t* __restrict__ ptr) {
  __shared__ long long part[PREP_THREADS];
  const int t = threadIdx.x;
  const int64_t seg = (len + PREP_THREADS - 1) / PREP_THREADS;
  const int64_t lo = std::min<int64_t>(len, t * seg), hi = std::min<int64_t>(len, lo + seg);
  long long sum = 0;
  for (int64_t i = lo; i < hi; ++i) sum += cnt[i];
  part[t] = sum;
  __syncthreads();
  if (t == 0) {
    long long run = 0;
    for (int i = 0; i < PREP_THREADS; ++i) {
      const long long x = part[i];
      part[i] = run;
      run += x;
    }
    ptr[len] = run;
  }
  __syncthreads();
  long long run = part[t];
  for (int64_t i = lo; i < hi; ++i) {
    ptr[i] = run;
    run += cnt[i];
  }
}

// SNP-major missing list: one warp per SNP writes the sample indices of its missing
// calls (increasing) at snp_list[ptr[j]..] and counts them per sample.
__global__ void k_geno_miss_fill(const uint8_t* __restrict__ bed, int64_t pitch, int64_t n, int64_t m,
                                 const int64_t* __restrict__ ptr, int32_t* __restrict__ snp_list,
                                 int32_t* __restrict__ samp_cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= m) return;
  const uint32_t* row = reinterpret_cast<const uint32_t*>(bed + j * pitch);
  const int64_t nw = (n + 15) / 16;
  int64_t base = ptr[j];
  for (int64_t w0 = 0; w0 < nw; w0 += 32) {
    const int64_t t = w0 + lane;
    uint32_t bits = 0;
    if (t < nw) {
      const uint32_t v = row[t];
      const int64_t valid = n - 16 * t;
      const uint32_t mask = valid >= 16 ? 0x55555555u : (0x55555555u >> (2 * (16 - valid)));
      bits = v & ~(v >> 1) & mask;  // code 01
    }
    const int c = __popc(bits);
    int incl = c;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    int64_t pos = base + incl - c;
    while (bits) {
      const int b = __ffs(bits) - 1;
      const int32_t i = (int32_t)(16 * t + (b >> 1));
      snp_list[pos++] = i;
      atomicAdd(samp_cnt + i, 1);
      bits &= bits - 1;
    }
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
}

// Sample-major copy of the missing list (the order within a sample is free: the
// corrections it feeds are exact integer sums).
__global__ void k_geno_miss_transpose(const int64_t* __restrict__ ptr, const int32_t* __restrict__ snp_list,
                                      int64_t m, const int64_t* __restrict__ samp_ptr,
                                      int32_t* __restrict__ samp_fill, int32_t* __restrict__ samp_list) {
  const int lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= m) return;
  for (int64_t k = ptr[j] + lane; k < ptr[j + 1]; k += 32) {
    const int32_t i = snp_list[k];
    const int pos = atomicAdd(samp_fill + i, 1);
    samp_list[samp_ptr[i] + pos] = (int32_t)j;
  }
}

// M_j = sum of V over SNP j's missing calls, into acc[m + j] (one warp per SNP).
__global__ void k_geno_miss_zt(const int64_t* __restrict__ ptr, const int32_t* __restrict__ snp_list, int64_t m,
                               const long long* __restrict__ V, unsigned long long* __restrict__ acc) {
  const int lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= m) return;
  unsigned long long s = 0;
  for (int64_t k = ptr[j] + lane; k < ptr[j + 1]; k += 32) s += (unsigned long long)V[snp_list[k]];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) acc[m + j] = s;
}

// Takes the missing calls' spurious terms back out of Z v: acc[i] -= sum of D[3j + 2]
// over the SNPs j where sample i is missing (one warp per sample).
__global__ void k_geno_miss_z(const int64_t* __restrict__ samp_ptr, const int32_t* __restrict__ samp_list,
                              int64_t n, const long long* __restrict__ D, unsigned long long* __restrict__ acc) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= n) return;
  unsigned long long s = 0;
  for (int64_t k = samp_ptr[i] + lane; k < samp_ptr[i + 1]; k += 32)
    s += (unsigned long long)D[3 * (int64_t)samp_list[k] + 2];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) acc[i] -= s;
}

// v (n, FP64) -> V (n_pad, int64 at scale 2^s) and U_i = V_i - 4 V_{i-1} within each
// 16-sample word (V_{i-1} = 0 at a word's first sample); meta[0] = s, meta[1] = T = sum V.
__global__ void __launch_bounds__(PREP_THREADS) k_geno_vprep(const double* __restrict__ v, int64_t n,
                                                            int64_t n_pad, long long* __restrict__ V,
                                                            long long* __restrict__ U,
                                                            long long* __restrict__ meta, int* status) {
  __shared__ double red[32];
  __shared__ unsigned long long redu[32];
  __shared__ int s_sh;
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) a += fabs(v[i]);
  a = block_sum_f64(a, red);
  if (threadIdx.x == 0) {
    int s = 0;
    if (!isfinite(a)) atomicExch(status, DEV_NONFINITE);
    else s = fix_exponent(a);
    s_sh = s;
    meta[0] = s;
  }
  __syncthreads();
  const int s = s_sh;
  unsigned long long t = 0;
  for (int64_t i = threadIdx.x; i < n_pad; i += blockDim.x) {
    const long long x = i < n ? __double2ll_rn(ldexp(v[i], s)) : 0ll;
    const long long xp = (i % 16) && i - 1 < n ? __double2ll_rn(ldexp(v[i - 1], s)) : 0ll;
    V[i] = x;
    U[i] = (long long)((unsigned long long)x - 4ull * (unsigned long long)xp);
    t += (unsigned long long)x;
  }
  t = block_sum_u64(t, redu);
  if (threadIdx.x == 0) meta[1] = (long long)t;
}

// Per-SNP float terms of multiply_Z_v (plink_reader.cpp:258-270) -> int64 values
// at scale 2^s: D[3j..3j+2] = (W2 - W0 per unit of k, W3 - 2 W2 + W0 where both bits
// are set, W2 = the spurious term of a missing call); meta[0] = s, meta[1] =
// C = sum_j W0_j (added to every sample).  w (3m floats) is scratch.
__global__ void __launch_bounds__(PREP_THREADS) k_geno_zprep(const double* __restrict__ v,
                                                            const double* __restrict__ mean,
                                                            const double* __restrict__ inv_std, int64_t m,
                                                            float* __restrict__ w, long long* __restrict__ D,
                                                            long long* __restrict__ meta, int* status) {
  __shared__ double red[32];
  __shared__ unsigned long long redu[32];
  __shared__ int s_sh;
  double a = 0.0;
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
    float w0 = 0.f, w2 = 0.f, w3 = 0.f;
    const double is = inv_std[j];
    if (is != 0.0) {
      const double mu = mean[j];
      const double weight = __dmul_rn(v[j], is);
      w0 = __double2float_rn(__dmul_rn(__dsub_rn(2.0, mu), weight));
      w2 = __double2float_rn(__dmul_rn(__dsub_rn(1.0, mu), weight));
      w3 = __double2float_rn(__dmul_rn(__dsub_rn(0.0, mu), weight));
    }
    w[3 * j] = w0;
    w[3 * j + 1] = w2;
    w[3 * j + 2] = w3;
    a += (double)fmaxf(fabsf(w0), fmaxf(fabsf(w2), fabsf(w3)));
  }
  a = block_sum_f64(a, red);
  if (threadIdx.x == 0) {
    int s = 0;
    if (!isfinite(a)) atomicExch(status, DEV_NONFINITE);
    else s = fix_exponent(a);
    s_sh = s;
    meta[0] = s;
  }
  __syncthreads();
  const int s = s_sh;
  unsigned long long c = 0;
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
    const long long W0 = __double2ll_rn(ldexp((double)w[3 * j], s));
    const long long W2 = __double2ll_rn(ldexp((double)w[3 * j + 1], s));
    const long long W3 = __double2ll_rn(ldexp((double)w[3 * j + 2], s));
    D[3 * j] = W2 - W0;
    D[3 * j + 1] = W3 - 2 * W2 + W0;
    D[3 * j + 2] = W2;
    c += (unsigned long long)W0;
  }
  c = block_sum_u64(c, redu);
  if (threadIdx.x == 0) meta[1] = (long long)c;
}

// sum_t k_t V_t for one 32-bit word of 16 codes against u = U of its 16 samples
// (the telescoped form above): lo accumulates the low words' 64-bit products, hi
// the high words' products modulo 2^32.
__device__ __forceinline__ void kdot16(uint32_t w, const uint2* __restrict__ u, unsigned long long& lo,
                                       uint32_t& hi) {
  const uint32_t kw = (w & 0x55555555u) + ((w >> 1) & 0x55555555u);
#pragma unroll
  for (int t = 0; t < 16; ++t) {
    const uint32_t at = kw >> (2 * t);
    const uint2 x = u[t];
    lo += (unsigned long long)at * x.x;
    hi += at * x.y;
  }
}

// Z^T v: one SNP row per thread over a chunk of CHUNK samples (2,048 to 8,192, a
// tuned launch shape).  The chunk's U sits in shared memory and is read as
// broadcasts; each thread streams its own row 16 bytes (64 samples) at a time.
// acc[row] += S (64-bit atomics).
template <int CHUNK>
__global__ void __launch_bounds__(ZT_THREADS) k_geno_zt(const uint8_t* __restrict__ bed, int64_t pitch,
                                                       int64_t m, const long long* __restrict__ U,
                                                       unsigned long long* __restrict__ acc) {
  __shared__ __align__(16) long long su[CHUNK];
  const int64_t c0 = (int64_t)blockIdx.y * CHUNK;
  const int len = (int)std::min<int64_t>(CHUNK, 4 * pitch - c0);  // multiple of 64
  for (int i = threadIdx.x; i < len; i += ZT_THREADS) su[i] = U[c0 + i];
  __syncthreads();
  const int64_t row = (int64_t)blockIdx.x * ZT_THREADS + threadIdx.x;
  if (row >= m) return;
  const uint4* p = reinterpret_cast<const uint4*>(bed + row * pitch + c0 / 4);
  const uint2* u = reinterpret_cast<const uint2*>(su);
  unsigned long long lo = 0;
  uint32_t hi = 0;
  const int nv = len / 64;  // 16-byte words of this row in the chunk
  for (int k = 0; k < nv; ++k) {
    const uint4 a = __ldg(p + k);
    kdot16(a.x, u + 64 * k, lo, hi);
    kdot16(a.y, u + 64 * k + 16, lo, hi);
    kdot16(a.z, u + 64 * k + 32, lo, hi);
    kdot16(a.w, u + 64 * k + 48, lo, hi);
  }
  atomicAdd(acc + row, lo + ((unsigned long long)hi << 32));
}

// Z v: 16 samples per thread (one 32-bit word per row, 128 coalesced bytes per
// warp), looping over a chunk of SNP rows whose values sit in shared memory.
// Per sample t: P_t = sum_j (kw_j >> 2t) D[3j] (telescoped, split into a 64-bit low
// and a 32-bit high accumulator) and Q_t = sum of D[3j+1] where both bits are set;
// acc[t] += P_t - 4 P_{t+1} + Q_t (64-bit atomics, one word per sample of n_pad).
__global__ void __launch_bounds__(Z_THREADS) k_geno_z(const uint8_t* __restrict__ bed, int64_t pitch,
                                                     int64_t m, int rows_per_cta,
                                                     const long long* __restrict__ D,
                                                     unsigned long long* __restrict__ acc) {
  extern __shared__ __align__(16) long long sd[];
  const int64_t r0 = (int64_t)blockIdx.y * rows_per_cta;
  const int nr = (int)std::min<int64_t>(rows_per_cta, m - r0);
  for (int i = threadIdx.x; i < 3 * nr; i += Z_THREADS) sd[i] = D[3 * r0 + i];
  __syncthreads();
  const int64_t byte_off = ((int64_t)blockIdx.x * Z_THREADS + threadIdx.x) * 4;
  if (byte_off >= pitch) return;
  const uint8_t* p = bed + r0 * pitch + byte_off;
  unsigned long long P[16], Q[16];
  uint32_t H[16];
#pragma unroll
  for (int t = 0; t < 16; ++t) { P[t] = 0; Q[t] = 0; H[t] = 0; }
#pragma unroll 2
  for (int r = 0; r < nr; ++r) {
    const uint32_t w = __ldg(reinterpret_cast<const uint32_t*>(p + (int64_t)r * pitch));
    const unsigned long long d1 = (unsigned long long)sd[3 * r];
    const unsigned long long d2 = (unsigned long long)sd[3 * r + 1];
    const uint32_t d1l = (uint32_t)d1, d1h = (uint32_t)(d1 >> 32);
    const uint32_t kw = (w & 0x55555555u) + ((w >> 1) & 0x55555555u);
    const uint32_t both = w & (w >> 1);
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const uint32_t at = kw >> (2 * t);
      P[t] += (unsigned long long)at * d1l;
      H[t] += at * d1h;
      if (both & (1u << (2 * t))) Q[t] += d2;
    }
  }
  const int64_t i0 = byte_off * 4;
#pragma unroll
  for (int t = 0; t < 16; ++t) {
    const unsigned long long pt = P[t] + ((unsigned long long)H[t] << 32);
    const unsigned long long pn = t < 15 ? P[t + 1] + ((unsigned long long)H[t + 1] << 32) : 0ull;
    atomicAdd(acc + i0 + t, pt - 4ull * pn + Q[t]);
  }
}

// multiply_Zt_v's last step (plink_reader.cpp:387) and, when effect != null, the
// back-solve's effect / frequency (result_writer.cpp:614-620).
__global__ void k_geno_zt_fin(const unsigned long long* __restrict__ acc, const long long* __restrict__ meta,
                              const double* __restrict__ mean, const double* __restrict__ inv_std,
                              int64_t m, const double* __restrict__ total_2pq, double* __restrict__ y,
                              double* __restrict__ effect, double* __restrict__ freq) {
  const int s = (int)meta[0];
  const unsigned long long T = (unsigned long long)meta[1];
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long S = acc[j], miss = acc[m + j];
    const long long A = (long long)(2ull * T - S - miss);
    const long long B = (long long)(T - miss);
    const double is = inv_std[j];
    double r = 0.0;
    if (is != 0.0) {
      const double sum_xv = ldexp(__ll2double_rn(A), -s);
      const double sum_v_obs = ldexp(__ll2double_rn(B), -s);
      r = __dmul_rn(__dsub_rn(sum_xv, __dmul_rn(mean[j], sum_v_obs)), is);
    }
    if (y) y[j] = r;
    if (effect) {
      const double t2 = *total_2pq;
      effect[j] = (is > 0.0 && t2 > 0.0) ? __ddiv_rn(__ddiv_rn(r, is), t2) : 0.0;
      freq[j] = __ddiv_rn(mean[j], 2.0);
    }
  }
}

__global__ void k_geno_z_fin(const unsigned long long* __restrict__ acc, const long long* __restrict__ meta,
                             int64_t n, double* __restrict__ y) {
  const int s = (int)meta[0];
  const unsigned long long C = (unsigned long long)meta[1];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = ldexp(__ll2double_rn((long long)(C + acc[i])), -s);
}

struct State {
  DevBuf<uint8_t> bed;      // m x pitch
  int64_t n = 0, m = 0, pitch = 0;
  DevBuf<double> stats;     // mean (m), inv_std (m), var2pq (m), total_2pq (1)
  DevBuf<long long> fixv;   // fixed-point V and U (2 n_pad) or per-SNP values (3m)
  DevBuf<float> wterm;      // float terms of Z v (3m)
  DevBuf<long long> meta;   // s, T or C
  DevBuf<unsigned long long> acc;
  DevBuf<double> vin, vout, q;
  // missing calls: SNP-major (miss_ptr m + 1, miss_snp) and sample-major (samp_ptr
  // n + 1, miss_samp) lists of the other index
  int64_t nmiss = 0;
  DevBuf<int64_t> miss_ptr, samp_ptr;
  DevBuf<int32_t> miss_snp, miss_samp;
  double* mean() const { return stats.p; }
  double* inv_std() const { return stats.p + m; }
  double* var2pq() const { return stats.p + 2 * m; }
  double* total() const { return stats.p + 3 * m; }
  int64_t n_pad() const { return 4 * pitch; }
};

State& state(cbx_handle* h) {
  CBX_REQUIRE(h->geno_slot, CBX_ERR_STATE, "call cbx_geno_attach first");
  return *static_cast<State*>(h->geno_slot.get());
}

template <typename F>
void timed(cbx_handle* h, int bucket, double bytes, F&& launch) {
  cbx_handle::ProfRec pr{};
  if (h->prof_on) {
    CBX_CUDA(cudaEventCreate(&pr.a));
    CBX_CUDA(cudaEventCreate(&pr.b));
    CBX_CUDA(cudaEventRecord(pr.a, h->stream));
  }
  launch();
  if (h->prof_on) {
    CBX_CUDA(cudaEventRecord(pr.b, h->stream));
    pr.bucket = bucket;
    pr.bytes = bytes;
    h->prof.push_back(pr);
  }
}

// y (m) = Z^T v for a device vector v (n).  With effect != null also the
// back-solve's effect and frequency columns.
void zt_device(cbx_handle* h, State& g, const double* v, double* y, double* effect, double* freq) {
  cudaStream_t s = h->stream;
  const int64_t n_pad = g.n_pad();
  g.fixv.resize(std::max<int64_t>(2 * n_pad, 3 * g.m));
  g.meta.resize(2);
  g.acc.resize(std::max<int64_t>(2 * g.m, n_pad));
  CBX_CUDA(cudaMemsetAsync(g.acc.p + g.m, 0, g.m * sizeof(unsigned long long), s));
  long long* V = g.fixv.p;
  long long* U = g.fixv.p + n_pad;
  k_geno_vprep<<<1, PREP_THREADS, 0, s>>>(v, g.n, n_pad, V, U, g.meta.p, h->status.p);
  h->launched("k_geno_vprep");
  // algorithmic bytes: the payload once, v once per SNP block of the grid, one row result
  const double bytes = (double)g.m * (double)((g.n + 3) / 4) + 8.0 * (double)g.n + 8.0 * (double)g.m;
  const unsigned gx = (unsigned)((g.m + ZT_THREADS - 1) / ZT_THREADS);
  // samples per CTA: 4,096 (default), 2,048 or 8,192; exact integer sums, so every
  // shape gives the same bits (the accumulator is zeroed before each run)
  auto zt = [&](int c) {
    CBX_CUDA(cudaMemsetAsync(g.acc.p, 0, g.m * sizeof(unsigned long long), s));
    const int chunk = c == 1 ? 2048 : (c == 2 ? 8192 : 4096);
    const dim3 grid(gx, (unsigned)((n_pad + chunk - 1) / chunk));
    if (c == 1) k_geno_zt<2048><<<grid, ZT_THREADS, 0, s>>>(g.bed.p, g.pitch, g.m, U, g.acc.p);
    else if (c == 2) k_geno_zt<8192><<<grid, ZT_THREADS, 0, s>>>(g.bed.p, g.pitch, g.m, U, g.acc.p);
    else k_geno_zt<4096><<<grid, ZT_THREADS, 0, s>>>(g.bed.p, g.pitch, g.m, U, g.acc.p);
    h->launched("k_geno_zt");
  };
  const int choice = tune::choose(h, tune::GENO_ZT, tune::size_class(g.n), tune::size_class(g.m), 1, 3, zt);
  timed(h, 3, bytes, [&] { zt(choice); });
  if (g.nmiss > 0) {
    k_geno_miss_zt<<<(unsigned)((g.m + 7) / 8), 256, 0, s>>>(g.miss_ptr.p, g.miss_snp.p, g.m, V, g.acc.p);
    h->launched("k_geno_miss_zt");
  }
  k_geno_zt_fin<<<gridn(g.m, 256, 4 * h->num_sms), 256, 0, s>>>(g.acc.p, g.meta.p, g.mean(), g.inv_std(), g.m,
                                                                g.total(), y, effect, freq);
  h->launched("k_geno_zt_fin");
}

// y (n) = Z v for a device vector v (m).
void z_device(cbx_handle* h, State& g, const double* v, double* y) {
  cudaStream_t s = h->stream;
  const int64_t n_pad = g.n_pad();
  g.fixv.resize(std::max<int64_t>(2 * n_pad, 3 * g.m));
  g.wterm.resize(3 * g.m);
  g.meta.resize(2);
  g.acc.resize(std::max<int64_t>(2 * g.m, n_pad));
  k_geno_zprep<<<1, PREP_THREADS, 0, s>>>(v, g.mean(), g.inv_std(), g.m, g.wterm.p, g.fixv.p, g.meta.p,
                                          h->status.p);
  h->launched("k_geno_zprep");
  const int gx = (int)((g.pitch + 4 * Z_THREADS - 1) / (4 * Z_THREADS));
  const double bytes = (double)g.m * (double)((g.n + 3) / 4) + 8.0 * (double)g.m + 8.0 * (double)g.n;
  // about 4 (default), 2 or 8 CTAs per SM, at most Z_MAX_ROWS SNP rows each; exact
  // integer sums, so every shape gives the same bits (the accumulator is zeroed
  // before each run)
  auto zk = [&](int c) {
    CBX_CUDA(cudaMemsetAsync(g.acc.p, 0, n_pad * sizeof(unsigned long long), s));
    const int per_sm = c == 1 ? 2 : (c == 2 ? 8 : 4);
    int64_t gy = std::max<int64_t>(1, (per_sm * (int64_t)h->num_sms + gx - 1) / gx);
    int64_t rows = std::min<int64_t>((g.m + gy - 1) / gy, Z_MAX_ROWS);
    gy = (g.m + rows - 1) / rows;
    CBX_REQUIRE(gy <= 65535, CBX_ERR_ARG, "too many SNPs for the Z v grid");
    const int smem = (int)(3 * rows * sizeof(long long));
    k_geno_z<<<dim3((unsigned)gx, (unsigned)gy), Z_THREADS, smem, s>>>(g.bed.p, g.pitch, g.m, (int)rows, g.fixv.p,
                                                                      g.acc.p);
    h->launched("k_geno_z");
  };
  const int choice = tune::choose(h, tune::GENO_Z, tune::size_class(g.n), tune::size_class(g.m), 1, 3, zk);
  timed(h, 4, bytes, [&] { zk(choice); });
  if (g.nmiss > 0) {
    k_geno_miss_z<<<(unsigned)((g.n + 7) / 8), 256, 0, s>>>(g.samp_ptr.p, g.miss_samp.p, g.n, g.fixv.p, g.acc.p);
    h->launched("k_geno_miss_z");
  }
  k_geno_z_fin<<<gridn(g.n, 256, 4 * h->num_sms), 256, 0, s>>>(g.acc.p, g.meta.p, g.n, y);
  h->launched("k_geno_z_fin");
}

}  // namespace geno
}  // namespace cbx

using namespace cbx;

extern "C" int cbx_geno_attach(cbx_handle* h, const uint8_t* bed, int64_t bed_bytes, int64_t n, int64_t m,
                               double* means, double* inv_stds) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(bed != nullptr, CBX_ERR_ARG, "bed is null");
    CBX_REQUIRE(n > 0 && m > 0, CBX_ERR_ARG, "empty genotype matrix");
    CBX_REQUIRE(n < (int64_t(1) << 31) && m < (int64_t(1) << 31), CBX_ERR_ARG, "n or m too large");
    CBX_REQUIRE(bed_bytes >= 3, CBX_ERR_FORMAT, "Invalid .bed file (too small)");
    CBX_REQUIRE(bed[0] == 0x6C && bed[1] == 0x1B, CBX_ERR_FORMAT, "Invalid .bed file magic number");
    CBX_REQUIRE(bed[2] == 0x01, CBX_ERR_FORMAT, "Only SNP-major mode (0x01) .bed files are supported");
    const int64_t bps = (n + 3) / 4;
    CBX_REQUIRE(bed_bytes >= 3 + m * bps, CBX_ERR_FORMAT,
                ".bed file is truncated: " + std::to_string(bed_bytes) + " < " + std::to_string(3 + m * bps) +
                    " bytes");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    auto g = std::make_shared<geno::State>();
    g->n = n;
    g->m = m;
    g->pitch = (bps + 15) / 16 * 16;
    g->bed.resize(m * g->pitch);
    g->bed.zero(s);
    CBX_CUDA(cudaMemcpy2DAsync(g->bed.p, g->pitch, bed + 3, bps, bps, m, cudaMemcpyHostToDevice, s));
    g->stats.resize(3 * m + 1);
    DevBuf<int32_t> cnt;
    cnt.resize(std::max(m, n));
    geno::k_geno_stats<<<(unsigned)m, 128, 0, s>>>(g->bed.p, g->pitch, n, m, g->mean(), g->inv_std(),
                                                    g->var2pq(), cnt.p);
    h->launched("k_geno_stats");
    geno::k_geno_total<<<1, geno::PREP_THREADS, 0, s>>>(g->var2pq(), m, g->total());
    h->launched("k_geno_total");
    // sparse missing lists
    g->miss_ptr.resize(m + 1);
    geno::k_geno_scan<<<1, geno::PREP_THREADS, 0, s>>>(cnt.p, m, g->miss_ptr.p);
    h->launched("k_geno_scan");
    CBX_CUDA(cudaMemcpyAsync(&g->nmiss, g->miss_ptr.p + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    if (g->nmiss > 0) {
      g->miss_snp.resize(g->nmiss);
      g->miss_samp.resize(g->nmiss);
      g->samp_ptr.resize(n + 1);
      CBX_CUDA(cudaMemsetAsync(cnt.p, 0, n * sizeof(int32_t), s));
      geno::k_geno_miss_fill<<<(unsigned)((m + 7) / 8), 256, 0, s>>>(g->bed.p, g->pitch, n, m, g->miss_ptr.p,
                                                                     g->miss_snp.p, cnt.p);
      h->launched("k_geno_miss_fill");
      geno::k_geno_scan<<<1, geno::PREP_THREADS, 0, s>>>(cnt.p, n, g->samp_ptr.p);
      h->launched("k_geno_scan");
      CBX_CUDA(cudaMemsetAsync(cnt.p, 0, n * sizeof(int32_t), s));
      geno::k_geno_miss_transpose<<<(unsigned)((m + 7) / 8), 256, 0, s>>>(g->miss_ptr.p, g->miss_snp.p, m,
                                                                          g->samp_ptr.p, cnt.p, g->miss_samp.p);
      h->launched("k_geno_miss_transpose");
    }
    if (means) CBX_CUDA(cudaMemcpyAsync(means, g->mean(), m * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (inv_stds)
      CBX_CUDA(cudaMemcpyAsync(inv_stds, g->inv_std(), m * sizeof(double), cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    h->geno_slot = g;
  });
}

extern "C" int cbx_geno_zt_v(cbx_handle* h, int32_t nvec, const double* v, double* y) {
  return cbx_guard(h, [&] {
    geno::State& g = geno::state(h);
    CBX_REQUIRE(nvec > 0 && v && y, CBX_ERR_ARG, "bad vectors");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    g.vin.resize(g.n);
    g.vout.resize(g.m);
    for (int c = 0; c < nvec; ++c) {
      CBX_CUDA(cudaMemcpyAsync(g.vin.p, v + (int64_t)c * g.n, g.n * sizeof(double), cudaMemcpyHostToDevice, s));
      geno::zt_device(h, g, g.vin.p, g.vout.p, nullptr, nullptr);
      CBX_CUDA(cudaMemcpyAsync(y + (int64_t)c * g.m, g.vout.p, g.m * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    h->check_status("cbx_geno_zt_v");
  });
}

extern "C" int cbx_geno_z_v(cbx_handle* h, int32_t nvec, const double* v, double* y) {
  return cbx_guard(h, [&] {
    geno::State& g = geno::state(h);
    CBX_REQUIRE(nvec > 0 && v && y, CBX_ERR_ARG, "bad vectors");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    g.vin.resize(g.m);
    g.vout.resize(g.n);
    for (int c = 0; c < nvec; ++c) {
      CBX_CUDA(cudaMemcpyAsync(g.vin.p, v + (int64_t)c * g.m, g.m * sizeof(double), cudaMemcpyHostToDevice, s));
      geno::z_device(h, g, g.vin.p, g.vout.p);
      CBX_CUDA(cudaMemcpyAsync(y + (int64_t)c * g.n, g.vout.p, g.n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    h->check_status("cbx_geno_z_v");
  });
}

extern "C" int cbx_snp_effects(cbx_handle* h, const double* u_g, int64_t n_g, const double* Ginv,
                               double* effect, double* freq, double* total_2pq) {
  return cbx_guard(h, [&] {
    geno::State& g = geno::state(h);
    CBX_REQUIRE(u_g && effect, CBX_ERR_ARG, "bad vectors");
    CBX_REQUIRE(n_g == g.n, CBX_ERR_ARG,
                "u_g has " + std::to_string(n_g) + " entries; the genotypes have " + std::to_string(g.n) +
                    " samples");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    g.vin.resize(n_g);
    g.q.resize(n_g);
    g.vout.resize(2 * g.m);
    CBX_CUDA(cudaMemcpyAsync(g.vin.p, u_g, n_g * sizeof(double), cudaMemcpyHostToDevice, s));
    // q = G^-1 u_g (DenseMatrixAdapter::operator*, FP64)
    DevBuf<double> gtmp;
    const double* gd = nullptr;
    if (Ginv) {
      gtmp.resize((size_t)n_g * n_g);
      CBX_CUDA(cudaMemcpyAsync(gtmp.p, Ginv, (size_t)n_g * n_g * sizeof(double), cudaMemcpyHostToDevice, s));
      gd = gtmp.p;
    } else if (h->Ginv.p && h->Ginv_n == n_g) {
      gd = h->Ginv.p;
    }
    if (gd) {
      Libs& L = libs(h);
      const double one = 1.0, zero = 0.0;
      CBX_BLAS(cublasDgemv(L.blas, CUBLAS_OP_T, (int)n_g, (int)n_g, &one, gd, (int)n_g, g.vin.p, 1, &zero,
                           g.q.p, 1));
    } else {
      CBX_REQUIRE(h->mme && h->mme->has_dense && !h->mme->has_sparse && h->mme->q == n_g, CBX_ERR_STATE,
                  "Could not locate Ginv for back-solving (pass Ginv, or call cbx_invert_psd / "
                  "cbx_mme_set_qinv_dense with a dense inverse of order n)");
      qinv_apply(h, 1, g.vin.p, g.q.p);
    }
    geno::zt_device(h, g, g.q.p, nullptr, g.vout.p, g.vout.p + g.m);
    CBX_CUDA(cudaMemcpyAsync(effect, g.vout.p, g.m * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (freq) CBX_CUDA(cudaMemcpyAsync(freq, g.vout.p + g.m, g.m * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (total_2pq) CBX_CUDA(cudaMemcpyAsync(total_2pq, g.total(), sizeof(double), cudaMemcpyDeviceToHost, s));
    h->check_status("cbx_snp_effects");
  });
}
