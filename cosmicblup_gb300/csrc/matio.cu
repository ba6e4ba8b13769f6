// Relationship-matrix files written from the device-resident matrices.
//
// COSMIC_UPPER_PACKED (reference src/core/upper_packed_binary.cpp:27-68, header
// layout in src/core/upper_packed_binary.h): 32-byte magic "COSMIC_UPPER_PACKED"
// (NUL padded), int32 version 1, int64 n, int32 index base 1, int32 storage code 1
// (upper packed), int32 dtype code 1 (float64), int32 endian code 1 (little), then
// A(i, j) for i <= j, column by column, as FP64.  Written by the reference's
// write_matrix_bin (src/core/matrix_io.cpp:479-484) for G, G^-1 and the ssGBLUP
// blocks.
//
// GCTA .grm.bin / .grm.N.bin (GrmBuilder::save, src/core/grm_builder.cpp:1873-1922):
// G(i, j) for j <= i, row by row, as float, and the same layout of N_snps, which the
// VanRaden path fills with the valid-SNP count (grm_builder.cpp:403).
//
// The matrices are column-major on the device (element (i, j) at [j n + i]).  A
// packing kernel turns a range of columns into the file's order in a device staging
// buffer; the host copies each packed range out and appends it to the file, so the
// n(n+1)/2 values never pass through a host loop.  G is exactly symmetric (the GRM
// kernel writes both triangles from one value), so G's lower triangle row by row
// is its upper triangle column by column.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#include "handle.h"

namespace cbx {
namespace matio {

// out[j (j + 1) / 2 - base + i] = A[j lda + i] for i <= j, j in [j0, j1): one block per
// column, converted to T (double, or float with round-to-nearest as the
// reference's implicit conversion).
template <typename T>
__global__ void k_pack_upper(const double* __restrict__ A, int64_t lda, int64_t j0, int64_t base,
                             T* __restrict__ out) {
  const int64_t j = j0 + blockIdx.x;
  const double* col = A + j * lda;
  T* dst = out + (j * (j + 1) / 2 - base);
  for (int64_t i = threadIdx.x; i <= j; i += blockDim.x) dst[i] = (T)col[i];
}

// Largest column count from j0 whose packed values fit in cap elements (>= 1).
inline int64_t columns_fitting(int64_t j0, int64_t n, int64_t cap) {
  int64_t j1 = j0, used = 0;
  while (j1 < n && used + (j1 + 1) <= cap) used += ++j1;
  return std::max<int64_t>(j1, j0 + 1);
}

struct File {
  FILE* f = nullptr;
  std::string path;
  explicit File(const std::string& p) : path(p) {
    f = std::fopen(p.c_str(), "wb");
    CBX_REQUIRE(f, CBX_ERR_ARG, "cannot write matrix file: " + p);
  }
  ~File() {
    if (f) std::fclose(f);
  }
  void write(const void* p, size_t bytes) {
    CBX_REQUIRE(std::fwrite(p, 1, bytes, f) == bytes, CBX_ERR_ARG, "short write to " + path);
  }
  void close() {
    const int rc = std::fclose(f);
    f = nullptr;
    CBX_REQUIRE(rc == 0, CBX_ERR_ARG, "cannot close " + path);
  }
};

// Pinned host staging plus a device staging buffer of `cap` elements of T.
template <typename T>
struct Stage {
  DevBuf<T> dev;
  T* host = nullptr;
  explicit Stage(int64_t cap) {
    dev.resize(cap);
    CBX_CUDA(cudaMallocHost(&host, cap * sizeof(T)));
  }
  ~Stage() {
    if (host) cudaFreeHost(host);
  }
};

// Streams the packed upper triangle of the n x n device matrix A into each file
// (with fill = true, every value replaced by fill_value, for the N_snps file).
template <typename T>
void stream_upper(cbx_handle* h, const double* A, int64_t n, File& out, File* fill_out, T fill_value) {
  const int64_t total = n * (n + 1) / 2;
  const int64_t cap = std::min<int64_t>(total, int64_t(1) << 25);  // 32 Mi values per pass
  Stage<T> st(std::max<int64_t>(cap, n));
  std::vector<T> fill;
  if (fill_out) fill.assign(std::max<int64_t>(cap, n), fill_value);
  for (int64_t j0 = 0; j0 < n;) {
    const int64_t j1 = columns_fitting(j0, n, std::max<int64_t>(cap, n));
    const int64_t base = j0 * (j0 + 1) / 2, cnt = j1 * (j1 + 1) / 2 - base;
    k_pack_upper<T><<<(unsigned)(j1 - j0), 256, 0, h->stream>>>(A, n, j0, base, st.dev.p);
    h->launched("k_pack_upper");
    CBX_CUDA(cudaMemcpyAsync(st.host, st.dev.p, cnt * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
    CBX_CUDA(cudaStreamSynchronize(h->stream));
    out.write(st.host, cnt * sizeof(T));
    if (fill_out) fill_out->write(fill.data(), cnt * sizeof(T));
    j0 = j1;
  }
}

}  // namespace matio
}  // namespace cbx

using namespace cbx;

extern "C" int cbx_write_upper_packed(cbx_handle* h, int32_t which, const char* path) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(path && *path, CBX_ERR_ARG, "path is empty");
    CBX_REQUIRE(which == 0 || which == 1, CBX_ERR_ARG, "which must be 0 (G) or 1 (G^-1)");
    const double* A = which == 0 ? h->G.p : h->Ginv.p;
    const int64_t n = which == 0 ? h->G_n : h->Ginv_n;
    CBX_REQUIRE(A && n > 0, CBX_ERR_STATE,
                which == 0 ? "no device GRM (cbx_grm_bed)" : "no device G inverse (cbx_invert_psd)");
    CBX_CUDA(cudaSetDevice(h->device));
    matio::File out(path);
    char magic[32] = {0};
    std::memcpy(magic, "COSMIC_UPPER_PACKED", 19);
    const int32_t version = 1, index_base = 1, storage = 1, dtype = 1, endian = 1;
    const int64_t n64 = n;
    out.write(magic, 32);
    out.write(&version, 4);
    out.write(&n64, 8);
    out.write(&index_base, 4);
    out.write(&storage, 4);
    out.write(&dtype, 4);
    out.write(&endian, 4);
    matio::stream_upper<double>(h, A, n, out, nullptr, 0.0);
    out.close();
  });
}

extern "C" int cbx_write_grm_gcta(cbx_handle* h, const char* bin_path, const char* n_path, int64_t n_valid) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(bin_path && *bin_path && n_path && *n_path, CBX_ERR_ARG, "path is empty");
    CBX_REQUIRE(h->G.p && h->G_n > 0, CBX_ERR_STATE, "no device GRM (cbx_grm_bed)");
    CBX_REQUIRE(n_valid >= 0, CBX_ERR_ARG, "n_valid must be >= 0");
    CBX_CUDA(cudaSetDevice(h->device));
    matio::File bin(bin_path), nf(n_path);
    matio::stream_upper<float>(h, h->G.p, h->G_n, bin, &nf, (float)n_valid);
    bin.close();
    nf.close();
  });
}
