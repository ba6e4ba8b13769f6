// Dense Qinv block product that allocates no device memory.
//
// Some callers cannot allocate device memory while they run: code running
// inside a host framework that owns the whole device memory pool (its
// allocator must not be bypassed), and latency-critical loops that must not
// pay for cudaMalloc / cudaFree, which may synchronize the device.
// cbx_dense_apply_noalloc gives them Y = Qd X for the dense Qinv block of the
// handle's MME with every intermediate in a fixed static device array:
//   * the array holds kScratchBytes (32 MiB) and stays resident on every GPU
//     that loads libcbx until the process exits;
//   * its device address is resolved with cudaGetSymbolAddress by a handle's
//     first call (with the handle's device current) and kept in the handle, so
//     that first call should come before any stream capture;
//   * every call reuses the same array, which keeps the previous call's
//     contents; the padding the kernel reads is cleared on every call;
//   * calls that overlap on the GPU (two streams, two threads, two handles on
//     one device) race on the array.
#include "handle.h"
#include "solver.cuh"

namespace cbx {
namespace noalloc {

constexpr size_t kScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Vt[c][k] = X[c * q + k] for k < q, 0 for q <= k < ld (column-major X of nc columns)
__global__ void k_pad_cols(const double* __restrict__ X, int64_t q, int64_t ld, int nc, int S, double* __restrict__ Vt) {
  const int64_t total = (int64_t)S * ld;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / ld, k = idx - c * ld;
    Vt[idx] = (c < nc && k < q) ? X[c * q + k] : 0.0;
  }
}
// Y[c * q + i] = Tout[i * S + c]
__global__ void k_unpack(const double* __restrict__ Tout, int64_t q, int nc, int S, double* __restrict__ Y) {
  const int64_t total = q * nc;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / q, i = idx - c * q;
    Y[idx] = Tout[i * S + c];
  }
}

static unsigned grid1(int64_t n, int cap) {
  int64_t g = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

template <int S>
static void chunk(cbx_handle* h, const Mme& m, int nc, const double* X, double* Y, unsigned char* scratch) {
  double* Vt = reinterpret_cast<double*>(scratch);
  double* Tout = Vt + (size_t)S * m.ld;  // 32-byte aligned (ld % 4 == 0); written with scalar stores
  k_pad_cols<<<grid1((int64_t)S * m.ld, 4 * h->num_sms), 256, 0, h->stream>>>(X, m.q, m.ld, nc, S, Vt);
  h->launched("k_pad_cols");
  constexpr int R = sizeof(double) == 8 ? (S <= 8 ? 8 : (S == 16 ? 4 : 2)) : 8;
  constexpr int KT = 32 * sv::Vec16<double>::n * 4;
  const int smem = S * KT * (int)sizeof(double);
  ensure_smem((const void*)sv::k_dense<double, S, R>, smem, h->device);
  sv::k_dense<double, S, R><<<(unsigned)((m.ng + 8 * R - 1) / (8 * R)), 256, smem, h->stream>>>(
      m.Qd64.p, m.ng, m.ld, Vt, Tout, nullptr);
  h->launched("k_dense");
  k_unpack<<<grid1(m.q * nc, 4 * h->num_sms), 256, 0, h->stream>>>(Tout, m.q, nc, S, Y);
  h->launched("k_unpack");
}

}  // namespace noalloc
}  // namespace cbx

using namespace cbx;

extern "C" int cbx_dense_apply_noalloc(cbx_handle* h, int32_t nrhs, const double* X_dev, double* Y_dev) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create and cbx_mme_set_qinv_dense first");
    const Mme& m = *h->mme;
    CBX_REQUIRE(m.has_dense && !m.has_sparse && m.ng == m.q, CBX_ERR_UNSUPPORTED,
                "the no-allocation product covers a dense Qinv only");
    CBX_REQUIRE(nrhs > 0 && X_dev && Y_dev, CBX_ERR_ARG, "bad vectors");
    CBX_CUDA(cudaSetDevice(h->device));
    // columns per pass: 32, and for the last pass the smallest width that holds it
    auto width = [](int nc) { return nc > 16 ? 32 : nc > 8 ? 16 : nc > 4 ? 8 : nc > 2 ? 4 : nc > 1 ? 2 : 1; };
    const int S0 = width(std::min(32, (int)nrhs));
    const size_t need = sizeof(double) * ((size_t)S0 * m.ld + (size_t)m.ng * S0);
    CBX_REQUIRE(need <= noalloc::kScratchBytes, CBX_ERR_ARG,
                "q = " + std::to_string(m.q) + " with " + std::to_string(S0) + " columns per pass needs " +
                    std::to_string(need) + " bytes of scratch; the no-allocation product is limited to " +
                    std::to_string(noalloc::kScratchBytes) + " bytes (q <= ~65,000 at 32 columns)");
    // set-up on this handle's first call: the static array's device address
    if (!h->noalloc_scratch) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, noalloc::g_scratch);
      CBX_REQUIRE(e == cudaSuccess && p, CBX_ERR_CUDA,
                  std::string("cudaGetSymbolAddress of the scratch array: ") + cudaGetErrorString(e));
      h->noalloc_scratch = p;
    }
    unsigned char* scratch = static_cast<unsigned char*>(h->noalloc_scratch);
    for (int c0 = 0; c0 < nrhs; c0 += 32) {
      const int nc = std::min(32, nrhs - c0);
      const double* X = X_dev + (int64_t)c0 * m.q;
      double* Y = Y_dev + (int64_t)c0 * m.q;
      switch (width(nc)) {
        case 1: noalloc::chunk<1>(h, m, nc, X, Y, scratch); break;
        case 2: noalloc::chunk<2>(h, m, nc, X, Y, scratch); break;
        case 4: noalloc::chunk<4>(h, m, nc, X, Y, scratch); break;
        case 8: noalloc::chunk<8>(h, m, nc, X, Y, scratch); break;
        case 16: noalloc::chunk<16>(h, m, nc, X, Y, scratch); break;
        default: noalloc::chunk<32>(h, m, nc, X, Y, scratch); break;
      }
    }
  });
}
