// Self-test entry points (not part of include/cbx.h): a single tcgen05 MMA on
// known small integers, using exactly the shared-memory layout, descriptors and
// TMEM read-back of the GRM kernel.  Used by the GPU tests to localise layout
// errors.  All accesses stay inside one 16 KB shared-memory tile set.
#include <cuda_fp16.h>
#include "handle.h"

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

}  // namespace selftest
}  // namespace cbx

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
