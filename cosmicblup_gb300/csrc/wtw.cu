// W'W of the mixed-model equations assembled on the device from the uploaded
// records (reference src/core/mme_builder.cpp:107-176: Eigen setFromTriplets
// over the records' triplets).
//
// Every record emits its triplets in the order of the host assembly: the fixed
// x fixed pairs (a <= b, the mirror when the columns differ), then, when the
// record has an animal, the fixed x animal pairs and the animal diagonal.  The
// triplets, keyed (row, column), are sorted stably (LSD radix sort, CUB), so
// equal keys keep their record order; each run of equal keys is summed in that
// order from 0.0.  That is the CSR, bit for bit, of one stable sort by (row,
// column) and a sequential sum, as the host path builds it.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <vector>
#include "handle.h"
#include "mme.h"

namespace cbx {
namespace wtw {

inline unsigned blocks(int64_t n, int threads, int cap) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cap, (n + threads - 1) / threads));
}

// triplets of record i (the emission order below)
__global__ void k_count(int64_t n_rec, int64_t q, const int32_t* __restrict__ xp, const int32_t* __restrict__ xc,
                        const int32_t* __restrict__ aid, int64_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_rec; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a0 = xp[i], a1 = xp[i + 1];
    int64_t c = 0;
    for (int32_t a = a0; a < a1; ++a)
      for (int32_t b = a; b < a1; ++b) c += xc[a] == xc[b] ? 1 : 2;
    const int32_t an = aid[i];
    if (an > 0 && an <= q) c += 2 * (int64_t)(a1 - a0) + 1;
    cnt[i] = c;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) cnt[n_rec] = 0;
}

__global__ void k_emit(int64_t n_rec, int64_t p, int64_t q, int cb, const int32_t* __restrict__ xp,
                       const int32_t* __restrict__ xc, const double* __restrict__ xv,
                       const int32_t* __restrict__ aid, const int64_t* __restrict__ off,
                       uint64_t* __restrict__ key, double* __restrict__ val) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_rec; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t o = off[i];
    auto emit = [&](int64_t r, int64_t c, double v) {
      key[o] = ((uint64_t)r << cb) | (uint64_t)c;
      val[o] = v;
      ++o;
    };
    const int32_t a0 = xp[i], a1 = xp[i + 1];
    for (int32_t a = a0; a < a1; ++a)
      for (int32_t b = a; b < a1; ++b) {
        const double v = xv[a] * xv[b];
        emit(xc[a], xc[b], v);
        if (xc[a] != xc[b]) emit(xc[b], xc[a], v);
      }
    const int32_t an = aid[i];
    if (an > 0 && an <= q) {
      const int64_t ck = p + an - 1;
      for (int32_t a = a0; a < a1; ++a) {
        emit(xc[a], ck, xv[a]);
        emit(ck, xc[a], xv[a]);
      }
      emit(ck, ck, 1.0);
    }
  }
}

// head[o] = 1 where a run of equal keys starts
__global__ void k_heads(int64_t n, const uint64_t* __restrict__ key, int64_t* __restrict__ head) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x)
    head[o] = (o == 0 || key[o] != key[o - 1]) ? 1 : 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) head[n] = 0;
}

// pos[u] = the start of run u (pos[nnz] = n)
__global__ void k_pos(int64_t n, const int64_t* __restrict__ head, const int64_t* __restrict__ rank,
                      int64_t nnz, int64_t* __restrict__ pos) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x)
    if (head[o]) pos[rank[o]] = o;
  if (blockIdx.x == 0 && threadIdx.x == 0) pos[nnz] = n;
}

constexpr int SHORT_RUN = 32;

// Run u summed in order from 0.0 into entry u (column, row, value); runs longer
// than SHORT_RUN go to the list of long runs (their entries are written by
// k_runs_long).
__global__ void k_runs(int64_t nnz, int cb, const uint64_t* __restrict__ key, const double* __restrict__ val,
                       const int64_t* __restrict__ pos, int32_t* __restrict__ col, double* __restrict__ out,
                       int32_t* __restrict__ row, int64_t* __restrict__ longs, unsigned long long* __restrict__ nlong) {
  const uint64_t mask = ((uint64_t)1 << cb) - 1;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nnz; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o0 = pos[u], o1 = pos[u + 1];
    const uint64_t k = key[o0];
    col[u] = (int32_t)(k & mask);
    row[u] = (int32_t)(k >> cb);
    if (o1 - o0 > SHORT_RUN) {
      longs[atomicAdd(nlong, 1ull)] = u;
      continue;
    }
    double v = 0.0;
    for (int64_t e = o0; e < o1; ++e) v += val[e];
    out[u] = v;
  }
}

// Long runs, one warp each: the lanes load 32 entries at a time (the next 32
// while the current ones are added) and every lane adds them in order, so the
// sum is the sequential one.
__global__ void k_runs_long(const int64_t* __restrict__ longs, const unsigned long long* __restrict__ nlong,
                            const int64_t* __restrict__ pos, const double* __restrict__ val,
                            double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t cnt = (int64_t)*nlong;
  for (int64_t w = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); w < cnt; w += nw) {
    const int64_t u = longs[w];
    const int64_t o0 = pos[u], o1 = pos[u + 1];
    double acc = 0.0;
    double x = o0 + lane < o1 ? val[o0 + lane] : 0.0;
    for (int64_t b = o0; b < o1; b += 32) {
      const double xn = b + 32 + lane < o1 ? val[b + 32 + lane] : 0.0;
      const int m = (int)min((int64_t)32, o1 - b);
      for (int j = 0; j < m; ++j) acc += __shfl_sync(0xffffffffu, x, j);
      x = xn;
    }
    if (lane == 0) out[u] = acc;
  }
}

// ptr[r] = the first entry of row >= r
__global__ void k_ptr(int64_t nnz, int64_t dim, const int32_t* __restrict__ row, int32_t* __restrict__ ptr) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u <= nnz; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r1 = u < nnz ? row[u] : dim;
    const int64_t r0 = u > 0 ? row[u - 1] + 1 : 0;
    for (int64_t r = r0; r <= r1; ++r) ptr[r] = (int32_t)u;
  }
}

// diag[r] = the (r, r) entry (0 when absent; binary search in the sorted row);
// A11 (p x p, zeroed) = the entries of the fixed rows in fixed columns (the
// first ones of each sorted row)
__global__ void k_diag_a11(int64_t dim, int64_t p, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                           const double* __restrict__ val, double* __restrict__ diag, double* __restrict__ A11) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
    int32_t lo = ptr[r], hi = ptr[r + 1];
    while (lo < hi) {
      const int32_t mid = lo + (hi - lo) / 2;
      if (col[mid] < r) lo = mid + 1; else hi = mid;
    }
    diag[r] = (lo < ptr[r + 1] && col[lo] == r) ? val[lo] : 0.0;
    if (r < p)
      for (int32_t j = ptr[r]; j < ptr[r + 1] && col[j] < p; ++j) A11[r * p + col[j]] = val[j];
  }
}

__global__ void k_to_f32(const double* __restrict__ a, int64_t n, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// device buffers of the assembly, kept by the handle between MMEs (grown, never
// shrunk: the kernels take explicit counts)
struct Scratch {
  DevBuf<int64_t> cnt, off, head, rank, pos, longs;
  DevBuf<unsigned char> tmp;
  DevBuf<uint64_t> k0, k1;
  DevBuf<double> v0, v1, a11;
  DevBuf<int32_t> row;
  DevBuf<unsigned long long> nlong;
};

template <typename T>
void need(DevBuf<T>& b, int64_t count) {
  if ((int64_t)b.n < count) b.resize((size_t)count);
}

}  // namespace wtw

// W'W of the records already on the device (m.x_ptr, m.x_col, m.x_val, m.aid)
// into m.D64 / m.D32 and its diagonal into m.diagD; the row pointers of the
// fixed rows (p + 1) and the fixed block X'X (p x p, row-major) come back to
// the host.
void wtw_device(cbx_handle* h, Mme& m, std::vector<int32_t>& ptr_fix, std::vector<double>& A11) {
  cudaStream_t s = h->stream;
  const int64_t n_rec = m.n_rec, p = m.p, q = m.q, dim = m.dim;
  const int sms = h->num_sms;
  int cb = 1;
  while (cb < 31 && (int64_t(1) << cb) < dim) ++cb;
  if (!h->wtw_slot) h->wtw_slot = std::make_shared<wtw::Scratch>();
  wtw::Scratch& w = *static_cast<wtw::Scratch*>(h->wtw_slot.get());
  auto& cnt = w.cnt;
  auto& off = w.off;
  wtw::need(cnt, n_rec + 1);
  wtw::need(off, n_rec + 1);
  wtw::k_count<<<wtw::blocks(n_rec, 256, 8 * sms), 256, 0, s>>>(n_rec, q, m.x_ptr.p, m.x_col.p, m.aid.p, cnt.p);
  h->launched("wtw::k_count");
  auto& tmp = w.tmp;
  size_t tb = 0;
  CBX_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt.p, off.p, n_rec + 1, s));
  wtw::need(tmp, std::max<int64_t>((int64_t)tb, 256));
  CBX_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, cnt.p, off.p, n_rec + 1, s));
  int64_t n = 0;
  CBX_CUDA(cudaMemcpyAsync(&n, off.p + n_rec, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  CBX_CUDA(cudaStreamSynchronize(s));
  auto &k0 = w.k0, &k1 = w.k1;
  auto &v0 = w.v0, &v1 = w.v1;
  const int64_t nb = std::max<int64_t>(n, 1);
  wtw::need(k0, nb); wtw::need(k1, nb); wtw::need(v0, nb); wtw::need(v1, nb);
  wtw::k_emit<<<wtw::blocks(n_rec, 256, 8 * sms), 256, 0, s>>>(n_rec, p, q, cb, m.x_ptr.p, m.x_col.p, m.x_val.p,
                                                               m.aid.p, off.p, k0.p, v0.p);
  h->launched("wtw::k_emit");
  // stable LSD radix sort of the 2 cb key bits; equal keys keep the record order
  tb = 0;
  CBX_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, k0.p, k1.p, v0.p, v1.p, n, 0, 2 * cb, s));
  wtw::need(tmp, (int64_t)tb);
  CBX_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, k0.p, k1.p, v0.p, v1.p, n, 0, 2 * cb, s));
  auto &head = w.head, &rank = w.rank;
  wtw::need(head, n + 1);
  wtw::need(rank, n + 1);
  wtw::k_heads<<<wtw::blocks(n, 256, 16 * sms), 256, 0, s>>>(n, k1.p, head.p);
  h->launched("wtw::k_heads");
  tb = 0;
  CBX_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, head.p, rank.p, n + 1, s));
  wtw::need(tmp, (int64_t)tb);
  CBX_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, head.p, rank.p, n + 1, s));
  int64_t nnz = 0;
  CBX_CUDA(cudaMemcpyAsync(&nnz, rank.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  CBX_CUDA(cudaStreamSynchronize(s));
  CBX_REQUIRE(nnz < (int64_t)INT32_MAX, CBX_ERR_UNSUPPORTED, "W'W has more than 2^31 entries");
  const int64_t nz = std::max<int64_t>(nnz, 1);
  m.D64.rows = m.D32.rows = (int32_t)dim;
  m.D64.nnz = m.D32.nnz = nnz;
  m.D64.ptr.resize(dim + 1); m.D32.ptr.resize(dim + 1);
  m.D64.col.resize(nz); m.D32.col.resize(nz);
  m.D64.val.resize(nz); m.D32.val.resize(nz);
  auto& row = w.row;
  auto &pos = w.pos, &longs = w.longs;
  auto& nlong = w.nlong;
  wtw::need(row, nz);
  wtw::need(pos, nnz + 1);
  wtw::need(longs, nz);
  wtw::need(nlong, 1);
  CBX_CUDA(cudaMemsetAsync(nlong.p, 0, sizeof(unsigned long long), s));
  wtw::k_pos<<<wtw::blocks(n, 256, 16 * sms), 256, 0, s>>>(n, head.p, rank.p, nnz, pos.p);
  h->launched("wtw::k_pos");
  wtw::k_runs<<<wtw::blocks(nnz, 256, 16 * sms), 256, 0, s>>>(nnz, cb, k1.p, v1.p, pos.p, m.D64.col.p, m.D64.val.p,
                                                              row.p, longs.p, nlong.p);
  h->launched("wtw::k_runs");
  wtw::k_runs_long<<<2 * sms, 256, 0, s>>>(longs.p, nlong.p, pos.p, v1.p, m.D64.val.p);
  h->launched("wtw::k_runs_long");
  wtw::k_ptr<<<wtw::blocks(nnz + 1, 256, 8 * sms), 256, 0, s>>>(nnz, dim, row.p, m.D64.ptr.p);
  h->launched("wtw::k_ptr");
  CBX_CUDA(cudaMemcpyAsync(m.D32.ptr.p, m.D64.ptr.p, (dim + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  CBX_CUDA(cudaMemcpyAsync(m.D32.col.p, m.D64.col.p, nz * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  wtw::k_to_f32<<<wtw::blocks(nz, 256, 8 * sms), 256, 0, s>>>(m.D64.val.p, nz, m.D32.val.p);
  h->launched("wtw::k_to_f32");
  m.diagD.resize(dim);
  auto& a11 = w.a11;
  wtw::need(a11, std::max<int64_t>(p * p, 1));
  CBX_CUDA(cudaMemsetAsync(a11.p, 0, std::max<int64_t>(p * p, 1) * sizeof(double), s));
  wtw::k_diag_a11<<<wtw::blocks(dim, 256, 8 * sms), 256, 0, s>>>(dim, p, m.D64.ptr.p, m.D64.col.p, m.D64.val.p,
                                                                 m.diagD.p, a11.p);
  h->launched("wtw::k_diag_a11");
  ptr_fix.resize(p + 1);
  A11.resize((size_t)p * p);
  CBX_CUDA(cudaMemcpyAsync(ptr_fix.data(), m.D64.ptr.p, (p + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  if (p > 0)
    CBX_CUDA(cudaMemcpyAsync(A11.data(), a11.p, (size_t)p * p * sizeof(double), cudaMemcpyDeviceToHost, s));
  CBX_CUDA(cudaStreamSynchronize(s));
}

}  // namespace cbx
