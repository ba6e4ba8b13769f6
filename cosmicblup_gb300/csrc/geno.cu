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
// 10 -> x = 1, 11 -> x = 0.  With lo / hi the two bits, x = (1 - lo)(2 - hi) and
// missing = lo (1 - hi), so one SNP needs three masked sums, S_lo = sum_{lo} v,
// S_hi = sum_{hi} v and S_both = sum_{lo and hi} v:
//   sum_obs x v = 2T - 2 S_lo - S_hi + S_both,   sum_obs v = T - S_lo + S_both,
// with T the sum of v over all samples.  In the same way Z v adds, for SNP j, w0_j to
// every sample, plus -w0_j where lo is set, w2_j - w0_j where hi is set and
// w0_j - w2_j + w3_j where both are set (w_c = the float term of code c).
//
// Layout: the payload is copied once into rows of `pitch` bytes (a multiple of 16,
// the padding bytes zero).  Samples at or beyond n get v = 0 (Z^T v) or are dropped
// (Z v), so the padding codes never reach a result.
#include <algorithm>
#include <cmath>
#include <vector>
#include <cublas_v2.h>
#include "dense.h"
#include "handle.h"
#include "pcg.h"

namespace cbx {
namespace geno {

constexpr int ZT_THREADS = 256;   // one SNP row per thread
constexpr int ZT_CHUNK = 4096;    // samples per CTA (32 KB of fixed-point v in shared memory)
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
__global__ void k_geno_stats(const uint8_t* __restrict__ bed, int64_t pitch, int64_t n, int64_t m,
                             double* __restrict__ mean, double* __restrict__ inv_std,
                             double* __restrict__ var2pq) {
  const int64_t j = blockIdx.x;
  if (j >= m) return;
  const uint32_t* row = reinterpret_cast<const uint32_t*>(bed + j * pitch);
  const int64_t nw = (n + 15) / 16;
  int hom1 = 0, het = 0, hom2 = 0;
  for (int64_t t = threadIdx.x; t < nw; t += blockDim.x) {
    const uint32_t v = row[t];
    const int64_t valid = n - 16 * t;  // >= 1
    const uint32_t mask = valid >= 16 ? 0x55555555u : (0x55555555u >> (2 * (16 - valid)));
    const uint32_t lo = v & 0x55555555u, hi = (v >> 1) & 0x55555555u;
    hom1 += __popc(~lo & ~hi & mask);
    het += __popc(~lo & hi & mask);
    hom2 += __popc(lo & hi & mask);
  }
  for (int o = 16; o > 0; o >>= 1) {
    hom1 += __shfl_down_sync(0xffffffffu, hom1, o);
    het += __shfl_down_sync(0xffffffffu, het, o);
    hom2 += __shfl_down_sync(0xffffffffu, hom2, o);
  }
  __shared__ int red[3][32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { red[0][w] = hom1; red[1][w] = het; red[2][w] = hom2; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  int a = 0, b = 0, c = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { a += red[0][i]; b += red[1][i]; c += red[2][i]; }
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

// v (n, FP64) -> V (n_pad, int64 at scale 2^s); meta[0] = s, meta[1] = T = sum V.
__global__ void __launch_bounds__(PREP_THREADS) k_geno_vprep(const double* __restrict__ v, int64_t n,
                                                            int64_t n_pad, long long* __restrict__ V,
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
    V[i] = x;
    t += (unsigned long long)x;
  }
  t = block_sum_u64(t, redu);
  if (threadIdx.x == 0) meta[1] = (long long)t;
}

// Per-SNP float terms of multiply_Z_v (plink_reader.cpp:258-270) -> int64 deltas
// D[3j..3j+2] = (-W0, W2 - W0, W0 - W2 + W3) at scale 2^s; meta[0] = s, meta[1] =
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
    D[3 * j] = -W0;
    D[3 * j + 1] = W2 - W0;
    D[3 * j + 2] = W0 - W2 + W3;
    c += (unsigned long long)W0;
  }
  c = block_sum_u64(c, redu);
  if (threadIdx.x == 0) meta[1] = (long long)c;
}

// Masked sums of one 32-bit word (16 codes) against 16 fixed-point values.
__device__ __forceinline__ void masked16(uint32_t w, const long long* __restrict__ v,
                                         unsigned long long& s_lo, unsigned long long& s_hi,
                                         unsigned long long& s_both) {
  const uint32_t both = w & (w >> 1);
#pragma unroll
  for (int t = 0; t < 16; t += 2) {
    const longlong2 x = *reinterpret_cast<const longlong2*>(v + t);
    if ((w >> (2 * t)) & 1u) s_lo += (unsigned long long)x.x;
    if ((w >> (2 * t + 1)) & 1u) s_hi += (unsigned long long)x.x;
    if ((both >> (2 * t)) & 1u) s_both += (unsigned long long)x.x;
    if ((w >> (2 * t + 2)) & 1u) s_lo += (unsigned long long)x.y;
    if ((w >> (2 * t + 3)) & 1u) s_hi += (unsigned long long)x.y;
    if ((both >> (2 * t + 2)) & 1u) s_both += (unsigned long long)x.y;
  }
}

// Z^T v: one SNP row per thread over a chunk of ZT_CHUNK samples.  The chunk's
// fixed-point v sits in shared memory and is read as broadcasts; each thread
// streams its own row 32 bytes (128 samples) at a time.  acc = (S_lo, S_hi,
// S_both) per row, 3m words, added with 64-bit atomics.
__global__ void __launch_bounds__(ZT_THREADS) k_geno_zt(const uint8_t* __restrict__ bed, int64_t pitch,
                                                       int64_t m, const long long* __restrict__ V,
                                                       unsigned long long* __restrict__ acc) {
  __shared__ __align__(16) long long sv[ZT_CHUNK];
  const int64_t c0 = (int64_t)blockIdx.y * ZT_CHUNK;
  const int len = (int)std::min<int64_t>(ZT_CHUNK, 4 * pitch - c0);  // multiple of 64
  for (int i = threadIdx.x; i < len; i += ZT_THREADS) sv[i] = V[c0 + i];
  __syncthreads();
  const int64_t row = (int64_t)blockIdx.x * ZT_THREADS + threadIdx.x;
  if (row >= m) return;
  const uint4* p = reinterpret_cast<const uint4*>(bed + row * pitch + c0 / 4);
  unsigned long long s_lo = 0, s_hi = 0, s_both = 0;
  const int nv = len / 64;  // 16-byte words of this row in the chunk
  int k = 0;
  for (; k + 1 < nv; k += 2) {
    const uint4 a = __ldg(p + k);
    const uint4 b = __ldg(p + k + 1);
    const long long* v = sv + 64 * k;
    masked16(a.x, v, s_lo, s_hi, s_both);
    masked16(a.y, v + 16, s_lo, s_hi, s_both);
    masked16(a.z, v + 32, s_lo, s_hi, s_both);
    masked16(a.w, v + 48, s_lo, s_hi, s_both);
    masked16(b.x, v + 64, s_lo, s_hi, s_both);
    masked16(b.y, v + 80, s_lo, s_hi, s_both);
    masked16(b.z, v + 96, s_lo, s_hi, s_both);
    masked16(b.w, v + 112, s_lo, s_hi, s_both);
  }
  if (k < nv) {
    const uint4 a = __ldg(p + k);
    const long long* v = sv + 64 * k;
    masked16(a.x, v, s_lo, s_hi, s_both);
    masked16(a.y, v + 16, s_lo, s_hi, s_both);
    masked16(a.z, v + 32, s_lo, s_hi, s_both);
    masked16(a.w, v + 48, s_lo, s_hi, s_both);
  }
  atomicAdd(acc + row, s_lo);
  atomicAdd(acc + m + row, s_hi);
  atomicAdd(acc + 2 * m + row, s_both);
}

// Z v: 16 samples per thread (one 32-bit word per row, 128 coalesced bytes per
// warp), looping over a chunk of SNP rows whose deltas sit in shared memory.
// acc: one word per sample (n_pad), added with 64-bit atomics.
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
  unsigned long long a[16];
#pragma unroll
  for (int t = 0; t < 16; ++t) a[t] = 0;
#pragma unroll 2
  for (int r = 0; r < nr; ++r) {
    const uint32_t w = __ldg(reinterpret_cast<const uint32_t*>(p + (int64_t)r * pitch));
    const unsigned long long d_lo = (unsigned long long)sd[3 * r];
    const unsigned long long d_hi = (unsigned long long)sd[3 * r + 1];
    const unsigned long long d_both = (unsigned long long)sd[3 * r + 2];
    const uint32_t both = w & (w >> 1);
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      if ((w >> (2 * t)) & 1u) a[t] += d_lo;
      if ((w >> (2 * t + 1)) & 1u) a[t] += d_hi;
      if ((both >> (2 * t)) & 1u) a[t] += d_both;
    }
  }
  const int64_t i0 = byte_off * 4;
#pragma unroll
  for (int t = 0; t < 16; ++t) atomicAdd(acc + i0 + t, a[t]);
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
    const unsigned long long slo = acc[j], shi = acc[m + j], sboth = acc[2 * m + j];
    const long long A = (long long)(2ull * T - 2ull * slo - shi + sboth);
    const long long B = (long long)(T - slo + sboth);
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
  DevBuf<long long> fixv;   // fixed-point v (n_pad) or deltas (3m)
  DevBuf<float> wterm;      // float terms of Z v (3m)
  DevBuf<long long> meta;   // s, T or C
  DevBuf<unsigned long long> acc;
  DevBuf<double> vin, vout, q;
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
  g.fixv.resize(std::max<int64_t>(n_pad, 3 * g.m));
  g.meta.resize(2);
  g.acc.resize(3 * g.m);
  g.acc.zero(s);
  k_geno_vprep<<<1, PREP_THREADS, 0, s>>>(v, g.n, n_pad, g.fixv.p, g.meta.p, h->status.p);
  h->launched("k_geno_vprep");
  const dim3 grid((unsigned)((g.m + ZT_THREADS - 1) / ZT_THREADS), (unsigned)((n_pad + ZT_CHUNK - 1) / ZT_CHUNK));
  // algorithmic bytes: the payload once, v once per SNP block of the grid, one row result
  const double bytes = (double)g.m * (double)((g.n + 3) / 4) + 8.0 * (double)g.n + 8.0 * (double)g.m;
  timed(h, 3, bytes, [&] {
    k_geno_zt<<<grid, ZT_THREADS, 0, s>>>(g.bed.p, g.pitch, g.m, g.fixv.p, g.acc.p);
    h->launched("k_geno_zt");
  });
  k_geno_zt_fin<<<gridn(g.m, 256, 4 * h->num_sms), 256, 0, s>>>(g.acc.p, g.meta.p, g.mean(), g.inv_std(), g.m,
                                                                g.total(), y, effect, freq);
  h->launched("k_geno_zt_fin");
}

// y (n) = Z v for a device vector v (m).
void z_device(cbx_handle* h, State& g, const double* v, double* y) {
  cudaStream_t s = h->stream;
  const int64_t n_pad = g.n_pad();
  g.fixv.resize(std::max<int64_t>(n_pad, 3 * g.m));
  g.wterm.resize(3 * g.m);
  g.meta.resize(2);
  g.acc.resize(n_pad);
  g.acc.zero(s);
  k_geno_zprep<<<1, PREP_THREADS, 0, s>>>(v, g.mean(), g.inv_std(), g.m, g.wterm.p, g.fixv.p, g.meta.p,
                                          h->status.p);
  h->launched("k_geno_zprep");
  const int gx = (int)((g.pitch + 4 * Z_THREADS - 1) / (4 * Z_THREADS));
  // about four CTAs per SM, at most Z_MAX_ROWS rows each
  int64_t gy = std::max<int64_t>(1, (4 * (int64_t)h->num_sms + gx - 1) / gx);
  int64_t rows = (g.m + gy - 1) / gy;
  rows = std::min<int64_t>(rows, Z_MAX_ROWS);
  gy = (g.m + rows - 1) / rows;
  const int smem = (int)(3 * rows * sizeof(long long));
  const double bytes = (double)g.m * (double)((g.n + 3) / 4) + 8.0 * (double)g.m + 8.0 * (double)g.n;
  timed(h, 4, bytes, [&] {
    k_geno_z<<<dim3((unsigned)gx, (unsigned)gy), Z_THREADS, smem, s>>>(g.bed.p, g.pitch, g.m, (int)rows,
                                                                      g.fixv.p, g.acc.p);
    h->launched("k_geno_z");
  });
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
    geno::k_geno_stats<<<(unsigned)m, 128, 0, s>>>(g->bed.p, g->pitch, n, m, g->mean(), g->inv_std(),
                                                    g->var2pq());
    h->launched("k_geno_stats");
    geno::k_geno_total<<<1, geno::PREP_THREADS, 0, s>>>(g->var2pq(), m, g->total());
    h->launched("k_geno_total");
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
