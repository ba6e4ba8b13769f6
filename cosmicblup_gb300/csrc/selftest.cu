// Self-test entry points (not part of include/cbx.h): a single tcgen05 MMA on
// known small integers, using exactly the shared-memory layout, descriptors and
// TMEM read-back of the GRM kernel.  Used by the GPU tests to localise layout
// errors.  All accesses stay inside one 16 KB shared-memory tile set.
#include <cuda_fp16.h>
#include <vector>
#include "dense_tc.h"
#include "handle.h"
#include "solver.cuh"

namespace cbx {
namespace selftest {

// A: 128 x 32, B: 32 x 32 (both K-major, no swizzle, 8x16B core matrices,
// LBO = 128 B along K, SBO = 512 B between 8-row groups).  D = A B^T (f32).
__global__ void __launch_bounds__(128, 1) k_umma_probe(const float* A, const float* B, float* D,
                                                       int* status) {
  __shared__ __align__(1024) uint8_t sa[128 * 32 * 2];
  __shared__ __align__(1024) uint8_t sb[32 * 32 * 2];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  // row t of A: 32 halves in 4 core matrices along K
  for (int kg = 0; kg < 4; ++kg)
    for (int e = 0; e < 8; ++e) {
      __half v = __float2half_rn(A[t * 32 + kg * 8 + e]);
      *reinterpret_cast<__half*>(sa + (t >> 3) * 512 + kg * 128 + (t & 7) * 16 + e * 2) = v;
    }
  if (t < 32)
    for (int kg = 0; kg < 4; ++kg)
      for (int e = 0; e < 8; ++e) {
        __half v = __float2half_rn(B[t * 32 + kg * 8 + e]);
        *reinterpret_cast<__half*>(sb + (t >> 3) * 512 + kg * 128 + (t & 7) * 16 + e * 2) = v;
      }
  if (t == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();
  if (warp == 0) {
    tmem_alloc(&tbase, 32);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = tbase;
  volatile int abort_flag = 0;
  if (t == 0) {
    const uint32_t a = smem_addr(sa), b = smem_addr(sb);
    for (int ks = 0; ks < 2; ++ks)
      umma_f16(tm, sdesc_noswizzle(a + ks * 256, 128, 512), sdesc_noswizzle(b + ks * 256, 128, 512),
               idesc_f16_f32(128, 32), ks > 0 ? 1u : 0u);
    umma_commit(&bar);
  }
  __syncwarp();
  if (!mbar_wait(&bar, 0, &abort_flag)) atomicExch(status, DEV_TIMEOUT);
  tc_fence_after();
  uint32_t r0[16], r1[16];
  const uint32_t ta = tm + (uint32_t(warp * 32) << 16);
  tmem_ld16(ta, r0);
  tmem_ld16(ta + 16, r1);
  tmem_ld_wait();
  for (int j = 0; j < 16; ++j) {
    D[t * 32 + j] = __uint_as_float(r0[j]);
    D[t * 32 + 16 + j] = __uint_as_float(r1[j]);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tm, 32);
}

// The bounded mbarrier wait of the pipelined kernels, on a barrier that no
// thread ever arrives at: every thread's wait gives up after limit_ns and
// thread 0 records DEV_TIMEOUT in the status word.  Nothing else is in flight
// (no TMA copy, no MMA, no TMEM), so the kernel returns normally and the
// context stays usable.
__global__ void k_wait_probe(int* status, uint64_t limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  volatile int abort_flag = 0;
  const bool ok = mbar_wait_for(&bar, 0, &abort_flag, limit_ns);
  if (__syncthreads_count(ok ? 0 : 1) > 0 && threadIdx.x == 0) atomicExch(status, DEV_TIMEOUT);
}

}  // namespace selftest
}  // namespace cbx

// Runs k_wait_probe with the given limit (1 us .. 1 s) and returns its status:
// CBX_ERR_TIMEOUT when the wait gave up, as every bounded wait of the library
// reports it.  *elapsed_ms receives the kernel's run time.
extern "C" int cbx_selftest_wait_timeout(cbx_handle* h, int64_t limit_ns, double* elapsed_ms) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(limit_ns >= 1000 && limit_ns <= 1000000000, CBX_ERR_ARG, "limit must be 1 us .. 1 s");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaEvent_t a, b;
    CBX_CUDA(cudaEventCreate(&a));
    CBX_CUDA(cudaEventCreate(&b));
    CBX_CUDA(cudaEventRecord(a, h->stream));
    cbx::selftest::k_wait_probe<<<1, 128, 0, h->stream>>>(h->status.p, (uint64_t)limit_ns);
    h->launched("k_wait_probe");
    CBX_CUDA(cudaEventRecord(b, h->stream));
    CBX_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    CBX_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (elapsed_ms) *elapsed_ms = ms;
    h->check_status("k_wait_probe");
  });
}

extern "C" int cbx_selftest_umma(cbx_handle* h, const float* A, const float* B, float* D) {
  return cbx_guard(h, [&] {
    CBX_CUDA(cudaSetDevice(h->device));
    cbx::DevBuf<float> dA, dB, dD;
    dA.resize(128 * 32);
    dB.resize(32 * 32);
    dD.resize(128 * 32);
    CBX_CUDA(cudaMemcpyAsync(dA.p, A, 128 * 32 * 4, cudaMemcpyHostToDevice, h->stream));
    CBX_CUDA(cudaMemcpyAsync(dB.p, B, 32 * 32 * 4, cudaMemcpyHostToDevice, h->stream));
    cbx::selftest::k_umma_probe<<<1, 128, 0, h->stream>>>(dA.p, dB.p, dD.p, h->status.p);
    h->launched("k_umma_probe");
    h->check_status("cbx_selftest_umma");
    CBX_CUDA(cudaMemcpyAsync(D, dD.p, 128 * 32 * 4, cudaMemcpyDeviceToHost, h->stream));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
  });
}

// The tensor-core block product alone: Y (ng x S, row-major) = Q (ng x ld,
// row-major FP32, ld % 4 == 0) V^T with V (S x ld, row-major FP32), S = 16 or
// 32, summed over its K splits in order on the host.
extern "C" int cbx_selftest_dense_tc(cbx_handle* h, const float* Q, int64_t ng, int64_t ld, const float* V,
                                     int32_t S, float* Y) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(S == 16 || S == 32 || S == 64, CBX_ERR_ARG, "S must be 16, 32 or 64");
    CBX_REQUIRE(ng > 0 && ld > 0 && ld % 4 == 0, CBX_ERR_ARG, "bad block shape");
    CBX_CUDA(cudaSetDevice(h->device));
    cbx::DevBuf<float> dQ, dV, dT;
    const int ks = cbx::dense_tc_ksplit(ng, ld, h->num_sms);
    dQ.resize((size_t)ng * ld);
    dV.resize((size_t)S * ld);
    dT.resize((size_t)ks * ng * S);
    CBX_CUDA(cudaMemcpyAsync(dQ.p, Q, (size_t)ng * ld * 4, cudaMemcpyHostToDevice, h->stream));
    CBX_CUDA(cudaMemcpyAsync(dV.p, V, (size_t)S * ld * 4, cudaMemcpyHostToDevice, h->stream));
    cbx::dense_tc(h, dQ.p, ng, ld, dV.p, S, ks, dT.p, nullptr, S);
    h->check_status("cbx_selftest_dense_tc");
    std::vector<float> T((size_t)ks * ng * S);
    CBX_CUDA(cudaMemcpyAsync(T.data(), dT.p, T.size() * 4, cudaMemcpyDeviceToHost, h->stream));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
    for (int64_t i = 0; i < ng * S; ++i) {
      float a = 0.0f;
      for (int k = 0; k < ks; ++k) a += T[(size_t)k * ng * S + i];
      Y[i] = a;
    }
  });
}

// The float-float block product alone: Y (ng x S, row-major FP64) = Q V^T with
// Q (ng x ld, row-major FP64, ld % 4 == 0) held as FP32 hi / lo parts and V
// (S x ld, row-major FP64).  rpw selects rows per warp (S = 32: 1 or 2; S = 16:
// 2 or 4; S = 1: 8); reps > 0 also times that many launches (ms_out, mean).
namespace {
__global__ void k_split_hilo(const double* __restrict__ q, int64_t n, float* __restrict__ hi,
                             float* __restrict__ lo) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float h = __double2float_rn(q[i]);
    hi[i] = h;
    lo[i] = __double2float_rn(q[i] - (double)h);
  }
}
__global__ void k_split_pairs(const double* __restrict__ v, int64_t n, float2* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float h = __double2float_rn(v[i]);
    out[i] = make_float2(h, __double2float_rn(v[i] - (double)h));
  }
}
template <int S, int R>
void launch_ff(cbx_handle* h, const float* qh, const float* ql, int64_t ng, int64_t ld, const float2* v, double* y) {
  const int smem = S * 256 * (int)sizeof(float2);
  CBX_CUDA(cudaFuncSetAttribute(cbx::sv::k_dense_ff<S, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  cbx::sv::k_dense_ff<S, R><<<(unsigned)((ng + 8 * R - 1) / (8 * R)), 256, smem, h->stream>>>(qh, ql, ng, ld, v, y,
                                                                                             nullptr);
  h->launched("k_dense_ff");
}
template <int S, int R>
void launch_ff2(cbx_handle* h, const float* qh, const float* ql, int64_t ng, int64_t ld, const float2* v, double* y) {
  const int smem = S * 256 * (int)sizeof(float2);
  CBX_CUDA(cudaFuncSetAttribute(cbx::sv::k_dense_ff2<S, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  cbx::sv::k_dense_ff2<S, R><<<(unsigned)((ng + 8 * R - 1) / (8 * R)), 256, smem, h->stream>>>(qh, ql, ng, ld, v, y,
                                                                                              nullptr);
  h->launched("k_dense_ff2");
}
}  // namespace

extern "C" int cbx_selftest_dense_ff(cbx_handle* h, const double* Q, int64_t ng, int64_t ld, const double* V,
                                     int32_t S, int32_t rpw, int32_t reps, double* Y, double* ms_out) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(ng > 0 && ld > 0 && ld % 4 == 0, CBX_ERR_ARG, "bad block shape");
    CBX_CUDA(cudaSetDevice(h->device));
    cbx::DevBuf<double> dQ, dV, dY;
    cbx::DevBuf<float> qh, ql;
    cbx::DevBuf<float2> vhl;
    dQ.resize((size_t)ng * ld);
    dV.resize((size_t)S * ld);
    dY.resize((size_t)ng * S);
    qh.resize((size_t)ng * ld);
    ql.resize((size_t)ng * ld);
    CBX_CUDA(cudaMemcpyAsync(dQ.p, Q, (size_t)ng * ld * 8, cudaMemcpyHostToDevice, h->stream));
    CBX_CUDA(cudaMemcpyAsync(dV.p, V, (size_t)S * ld * 8, cudaMemcpyHostToDevice, h->stream));
    k_split_hilo<<<1024, 256, 0, h->stream>>>(dQ.p, ng * ld, qh.p, ql.p);
    h->launched("k_split_hilo");
    vhl.resize((size_t)S * ld);
    k_split_pairs<<<256, 256, 0, h->stream>>>(dV.p, S * ld, vhl.p);
    h->launched("k_split_pairs");
    auto run = [&] {
      if (S == 32 && rpw == 1) launch_ff<32, 1>(h, qh.p, ql.p, ng, ld, vhl.p, dY.p);
      else if (S == 32 && rpw == 2) launch_ff<32, 2>(h, qh.p, ql.p, ng, ld, vhl.p, dY.p);
      else if (S == 16 && rpw == 2) launch_ff<16, 2>(h, qh.p, ql.p, ng, ld, vhl.p, dY.p);
      else if (S == 16 && rpw == 4) launch_ff<16, 4>(h, qh.p, ql.p, ng, ld, vhl.p, dY.p);
      else if (S == 1 && rpw == 8) launch_ff<1, 8>(h, qh.p, ql.p, ng, ld, vhl.p, dY.p);
      // negative rpw: the packed (f32x2) kernel with |rpw| rows per warp
      else if (S == 16 && rpw == -2) launch_ff2<16, 2>(h, qh.p, ql.p, ng, ld, vhl.p, dY.p);
      else if (S == 16 && rpw == -1) launch_ff2<16, 1>(h, qh.p, ql.p, ng, ld, vhl.p, dY.p);
      else if (S == 32 && rpw == -1) launch_ff2<32, 1>(h, qh.p, ql.p, ng, ld, vhl.p, dY.p);
      else throw cbx::Error(CBX_ERR_ARG, "unsupported (S, rpw)");
    };
    run();
    if (reps > 0) {
      cudaEvent_t a, b;
      CBX_CUDA(cudaEventCreate(&a));
      CBX_CUDA(cudaEventCreate(&b));
      CBX_CUDA(cudaEventRecord(a, h->stream));
      for (int i = 0; i < reps; ++i) run();
      CBX_CUDA(cudaEventRecord(b, h->stream));
      CBX_CUDA(cudaEventSynchronize(b));
      float ms = 0;
      CBX_CUDA(cudaEventElapsedTime(&ms, a, b));
      if (ms_out) *ms_out = ms / reps;
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
    CBX_CUDA(cudaMemcpyAsync(Y, dY.p, (size_t)ng * S * 8, cudaMemcpyDeviceToHost, h->stream));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
  });
}

// The fixed-point tensor-core product alone: Y (ng x S, row-major FP64) = Q V^T
// with Q (ng x ld, row-major FP64, ld % 4 == 0) held as FP32 hi / lo planes and V
// (S x ld, row-major FP64, S <= 32); reps > 0 also times that many products
// (ms_out, mean, including the column-digit and reduce kernels).
namespace {
__global__ void k_transpose_cols(const double* __restrict__ V, int S, int64_t ld, int64_t ng, double* __restrict__ X) {
  const int64_t total = ng * S;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = i / S;
    const int c = (int)(i - k * S);
    X[i] = V[(int64_t)c * ld + k];
  }
}
__global__ void k_iota(int32_t* __restrict__ g, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    g[i] = (int32_t)i;
}
}  // namespace

extern "C" int cbx_selftest_dense_fx(cbx_handle* h, const double* Q, int64_t ng, int64_t ld, const double* V,
                                     int32_t S, int32_t reps, double* Y, double* ms_out) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(ng > 0 && ld >= ng && ld % 4 == 0 && S >= 1 && S <= 32, CBX_ERR_ARG, "bad shape");
    CBX_CUDA(cudaSetDevice(h->device));
    cbx::DevBuf<double> dQ, dV, dX, dY, part;
    cbx::DevBuf<float> qh, ql;
    cbx::DevBuf<int32_t> rowexp, gmap, cexp;
    cbx::DevBuf<uint16_t> bdig;
    dQ.resize((size_t)ng * ld);
    dV.resize((size_t)S * ld);
    dX.resize((size_t)ng * S);
    dY.resize((size_t)ng * S);
    qh.resize((size_t)ng * ld);
    ql.resize((size_t)ng * ld);
    rowexp.resize(ng);
    gmap.resize(ng);
    CBX_CUDA(cudaMemcpyAsync(dQ.p, Q, (size_t)ng * ld * 8, cudaMemcpyHostToDevice, h->stream));
    CBX_CUDA(cudaMemcpyAsync(dV.p, V, (size_t)S * ld * 8, cudaMemcpyHostToDevice, h->stream));
    k_split_hilo<<<1024, 256, 0, h->stream>>>(dQ.p, ng * ld, qh.p, ql.p);
    h->launched("k_split_hilo");
    k_transpose_cols<<<256, 256, 0, h->stream>>>(dV.p, S, ld, ng, dX.p);
    h->launched("k_transpose_cols");
    k_iota<<<64, 256, 0, h->stream>>>(gmap.p, ng);
    h->launched("k_iota");
    cbx::fx_row_scales(h, qh.p, ng, ld, rowexp.p);
    auto run = [&] {
      cbx::fx_product(h, qh.p, ql.p, rowexp.p, ng, ld, dX.p, S, 0, gmap.p, S, bdig, cexp, part, dY.p, S, nullptr);
    };
    run();
    h->check_status("cbx_selftest_dense_fx");
    if (reps > 0) {
      cudaEvent_t a, b;
      CBX_CUDA(cudaEventCreate(&a));
      CBX_CUDA(cudaEventCreate(&b));
      CBX_CUDA(cudaEventRecord(a, h->stream));
      for (int i = 0; i < reps; ++i) run();
      CBX_CUDA(cudaEventRecord(b, h->stream));
      CBX_CUDA(cudaEventSynchronize(b));
      float ms = 0;
      CBX_CUDA(cudaEventElapsedTime(&ms, a, b));
      if (ms_out) *ms_out = ms / reps;
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      h->check_status("cbx_selftest_dense_fx");
    }
    CBX_CUDA(cudaMemcpyAsync(Y, dY.p, (size_t)ng * S * 8, cudaMemcpyDeviceToHost, h->stream));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
  });
}
