// Pedigree relationship inverse and the ssGBLUP H^-1 blocks.
//
// Replaces (reference files):
//  * genmatrix::ml and invertA_henderson (src/core/a_matrix.cpp:127-186, 392-439)
//    with complete_missing_parents_add_phantoms (:42-51) and
//    enforceSymmetryAndDiagonal(A, 1e-12, 1e-15) (:58-79) -- host C++;
//  * the ssGBLUP branch of MatrixBuilder::build
//    (src/io/relationship_builder.cpp:481-633): A22 extraction (:495-534),
//    tuneG (:539-565), alpha blend (:567-569), eigen-bent inverse (:571),
//    A22^-1 (:573-581), tau / omega scaling (:583-584), SplitMatrixAdapter (:630).
//
// A22 is not obtained from n_g sparse triangular solves on a factor of A^-1 as
// in the reference, but from the pedigree recursion A = T D T^T with
// T = (I - P)^-1 (P holds 1/2 for each known parent), applied to all
// genotyped unit vectors at once on the device: a backward pass that pulls from
// children, the D scaling, and a forward pass that pulls from parents, one
// kernel per generation.  The result is the same matrix A[geno, geno].
#include <algorithm>
#include <cmath>
#include <set>
#include <vector>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include "handle.h"
#include "solver.cuh"

namespace cbx {

// Defined in reml.cu / mme.cu.
void invert_psd_device(cbx_handle* h, const double* M_dev, int64_t n, double ridge, double* out_dev);
bool chol_inverse_device(cbx_handle* h, double* A_dev, int64_t n);

namespace ped {

// Meuwissen-Luo style inbreeding exactly as genmatrix::ml: the ancestor scan
// visits indices from max(sire, dam) downwards with positive path coefficient.
static void ml(const std::vector<int64_t>& dam, const std::vector<int64_t>& sire, std::vector<double>& f,
               std::vector<double>& dii) {
  const int64_t n = (int64_t)dam.size();
  f.assign(n, 0.0);
  dii.assign(n, 1.0);
  std::vector<double> L(n, 0.0);
  std::set<int64_t> pending;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t s = sire[i], d = dam[i];
    const bool s_ok = s >= 0 && s < n, d_ok = d >= 0 && d < n;
    const double Fs = s_ok ? f[s] : 0.0, Fd = d_ok ? f[d] : 0.0;
    if (s_ok && d_ok) dii[i] = 1.0 - 0.25 * (1.0 + Fs) - 0.25 * (1.0 + Fd);
    else if (s_ok) dii[i] = 1.0 - 0.25 * (1.0 + Fs);
    else if (d_ok) dii[i] = 1.0 - 0.25 * (1.0 + Fd);
    else dii[i] = 1.0;
    if (s_ok && d_ok) {
      L[s] += 0.5;
      pending.insert(s);
      L[d] += 0.5;
      pending.insert(d);
      double F_calc = 0.0;
      int64_t hi = std::max(s, d);
      while (!pending.empty()) {
        auto it = pending.upper_bound(hi);
        if (it == pending.begin()) break;
        --it;
        const int64_t j = *it;
        pending.erase(it);
        hi = j - 1;
        if (L[j] > 0.0) {
          F_calc += L[j] * L[j] * dii[j];
          const int64_t sj = sire[j], dj = dam[j];
          if (sj >= 0 && sj < n) { L[sj] += 0.5 * L[j]; pending.insert(sj); }
          if (dj >= 0 && dj < n) { L[dj] += 0.5 * L[j]; pending.insert(dj); }
          L[j] = 0.0;
        }
      }
      f[i] = F_calc + dii[i] - 1.0;
      if (f[i] < 0.0) f[i] = 0.0;
    } else {
      f[i] = 0.0;
    }
  }
}

struct Trip {
  int64_t r, c;
  double v;
};

// Backward pass of T^T: y_j = x_j + 1/2 sum over children c of y_c, for the
// animals of one generation (children already final).  Y row-major n x ng.
__global__ void k_pull_children(const int64_t* __restrict__ ids, int64_t count, const int64_t* __restrict__ cptr,
                                const int64_t* __restrict__ cidx, int64_t ng, double* __restrict__ Y) {
  for (int64_t t = blockIdx.y; t < count; t += gridDim.y) {
    const int64_t j = ids[t];
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ng; k += (int64_t)gridDim.x * blockDim.x) {
      double acc = 0.0;
      for (int64_t e = cptr[j]; e < cptr[j + 1]; ++e) acc += Y[cidx[e] * ng + k];
      Y[j * ng + k] += 0.5 * acc;
    }
  }
}
// D scaling fused with the forward pass of T: z_i = dii_i y_i + 1/2 (z_s + z_d)
__global__ void k_pull_parents(const int64_t* __restrict__ ids, int64_t count, const int64_t* __restrict__ sire,
                               const int64_t* __restrict__ dam, const double* __restrict__ dii, int64_t ng,
                               double* __restrict__ Y) {
  for (int64_t t = blockIdx.y; t < count; t += gridDim.y) {
    const int64_t i = ids[t];
    const int64_t s = sire[i], d = dam[i];
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ng; k += (int64_t)gridDim.x * blockDim.x) {
      double z = dii[i] * Y[i * ng + k];
      if (s >= 0) z += 0.5 * Y[s * ng + k];
      if (d >= 0) z += 0.5 * Y[d * ng + k];
      Y[i * ng + k] = z;
    }
  }
}
// Y[gmap[k], k] = 1 (Y zeroed before)
__global__ void k_set_units(const int32_t* __restrict__ gmap, int64_t ng, double* __restrict__ Y) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ng; k += (int64_t)gridDim.x * blockDim.x)
    Y[(int64_t)gmap[k] * ng + k] = 1.0;
}
// A22 (ng x ng, column-major) = Y[gmap, :] ; Y row-major n x ng
__global__ void k_gather_rows(const double* __restrict__ Y, const int32_t* __restrict__ gmap, int64_t ng,
                              double* __restrict__ A22) {
  const int64_t total = ng * ng;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx % ng, c = idx / ng;
    A22[idx] = Y[(int64_t)gmap[r] * ng + c];
  }
}
// partial sums: trace and total of a matrix
__global__ void k_sum_diag_all(const double* __restrict__ M, int64_t n, double* __restrict__ part) {
  __shared__ double red[256];
  double sd = 0, sa = 0;
  const int64_t total = n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const double v = M[idx];
    sa += v;
    if (idx % n == idx / n) sd += v;
  }
  double t = sv::block_sum_cols<1>(sd, red);
  if (threadIdx.x == 0) part[2 * blockIdx.x] = t;
  t = sv::block_sum_cols<1>(sa, red);
  if (threadIdx.x == 0) part[2 * blockIdx.x + 1] = t;
}
// out = (1 - alpha) (b G + a) + alpha A22
__global__ void k_blend(const double* __restrict__ G, const double* __restrict__ A22, int64_t total, double a,
                        double b, double alpha, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (1.0 - alpha) * (b * G[i] + a) + alpha * A22[i];
}
// Gd = tau Gbinv - omega A22inv
__global__ void k_combine(const double* __restrict__ Gbi, const double* __restrict__ Ai, int64_t total, double tau,
                          double omega, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = tau * Gbi[i] - omega * Ai[i];
}

static inline unsigned gridn(int64_t n, int threads, int cap) {
  int64_t g = (n + threads - 1) / threads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

}  // namespace ped
}  // namespace cbx

using namespace cbx;

// A^-1 by Henderson's rules with Meuwissen-Luo inbreeding.  dam / sire are
// 0-based parent indices (-1 = unknown; out-of-range values are treated as
// unknown).  Call with ptr == NULL to obtain nnz, then with arrays of that size.
extern "C" int cbx_ainv_henderson(cbx_handle* h, int64_t n, const int64_t* dam, const int64_t* sire,
                                  int64_t* nnz, int64_t* ptr, int32_t* col, double* val, double* F,
                                  double* dii_out) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(n > 0 && dam && sire && nnz, CBX_ERR_ARG, "bad pedigree arguments");
    std::vector<int64_t> d(dam, dam + n), s(sire, sire + n);
    for (int64_t j = 0; j < n; ++j) {
      if (!(d[j] >= 0 && d[j] < n)) d[j] = -1;
      if (!(s[j] >= 0 && s[j] < n)) s[j] = -1;
    }
    std::vector<double> f, dii;
    ped::ml(d, s, f, dii);
    std::vector<ped::Trip> t;
    t.reserve((size_t)n * 9);
    for (int64_t i = 0; i < n; ++i) {
      const int64_t di = d[i], si = s[i];
      const double dinv = 1.0 / dii[i];
      t.push_back({i, i, dinv});
      if (si >= 0) {
        t.push_back({i, si, -0.5 * dinv});
        t.push_back({si, i, -0.5 * dinv});
        t.push_back({si, si, 0.25 * dinv});
      }
      if (di >= 0) {
        t.push_back({i, di, -0.5 * dinv});
        t.push_back({di, i, -0.5 * dinv});
        t.push_back({di, di, 0.25 * dinv});
      }
      if (si >= 0 && di >= 0) {
        t.push_back({si, di, 0.25 * dinv});
        t.push_back({di, si, 0.25 * dinv});
      }
    }
    std::stable_sort(t.begin(), t.end(),
                     [](const ped::Trip& a, const ped::Trip& b) { return a.r != b.r ? a.r < b.r : a.c < b.c; });
    std::vector<int64_t> rp(n + 1, 0);
    std::vector<int32_t> cc;
    std::vector<double> vv;
    std::vector<bool> has_diag(n, false);
    for (size_t k = 0; k < t.size();) {
      size_t e = k;
      double v = 0.0;
      while (e < t.size() && t[e].r == t[k].r && t[e].c == t[k].c) v += t[e++].v;
      const int64_t r = t[k].r, c = t[k].c;
      if (r == c) {
        has_diag[r] = true;
        if (v < 1e-15) v = 1e-12;  // enforceSymmetryAndDiagonal(A, 1e-12, 1e-15)
      }
      if (std::fabs(v) > 1e-24) {  // prune(1e-12) with Eigen's dummy precision
        cc.push_back((int32_t)c);
        vv.push_back(v);
        rp[r + 1]++;
      }
      k = e;
    }
    // every row has a diagonal (a founder-only animal at least has 1/dii)
    for (int64_t i = 0; i < n; ++i) CBX_REQUIRE(has_diag[i], CBX_ERR_ARG, "internal: missing diagonal");
    for (int64_t i = 0; i < n; ++i) rp[i + 1] += rp[i];
    *nnz = (int64_t)cc.size();
    if (ptr) {
      CBX_REQUIRE(col && val, CBX_ERR_ARG, "col / val must be given with ptr");
      std::copy(rp.begin(), rp.end(), ptr);
      std::copy(cc.begin(), cc.end(), col);
      std::copy(vv.begin(), vv.end(), val);
    }
    if (F) std::copy(f.begin(), f.end(), F);
    if (dii_out) std::copy(dii.begin(), dii.end(), dii_out);
  });
}

// ssGBLUP: Qinv = A^-1 + S (tau Gb^-1 - omega A22^-1) S^T on the MME of this handle.
extern "C" int cbx_ssgblup_qinv(cbx_handle* h, int64_t n, const int64_t* dam, const int64_t* sire, int64_t ng,
                                const int32_t* gmap, const double* G, double alpha, int32_t tune_g, double tau,
                                double omega, double ridge, double* A22_out, double* Gd_out) {
  return cbx_guard(h, [&] {
    CBX_REQUIRE(h->mme, CBX_ERR_STATE, "call cbx_mme_create (q = pedigree size) first");
    CBX_REQUIRE(h->mme->q == n, CBX_ERR_ARG, "MME q must equal the pedigree size");
    CBX_REQUIRE(ng > 0 && ng <= n && gmap, CBX_ERR_ARG, "bad genotyped map");
    CBX_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    // A^-1 and inbreeding on the host
    int64_t nnz = 0;
    if (int rc = cbx_ainv_henderson(h, n, dam, sire, &nnz, nullptr, nullptr, nullptr, nullptr, nullptr); rc != CBX_OK)
      throw Error(rc, h->last_error);
    std::vector<int64_t> ap(n + 1);
    std::vector<int32_t> ac(nnz);
    std::vector<double> av(nnz), dii(n);
    if (int rc = cbx_ainv_henderson(h, n, dam, sire, &nnz, ap.data(), ac.data(), av.data(), nullptr, dii.data());
        rc != CBX_OK)
      throw Error(rc, h->last_error);
    // generations and children lists (parents first)
    std::vector<int64_t> d(dam, dam + n), sr(sire, sire + n), level(n, 0);
    for (int64_t i = 0; i < n; ++i) {
      if (!(d[i] >= 0 && d[i] < n)) d[i] = -1;
      if (!(sr[i] >= 0 && sr[i] < n)) sr[i] = -1;
      CBX_REQUIRE(d[i] < i && sr[i] < i, CBX_ERR_ARG,
                  "pedigree must list parents before their progeny (as genmatrix::ml assumes)");
      int64_t lv = 0;
      if (d[i] >= 0) lv = std::max(lv, level[d[i]] + 1);
      if (sr[i] >= 0) lv = std::max(lv, level[sr[i]] + 1);
      level[i] = lv;
    }
    const int64_t nlev = n ? *std::max_element(level.begin(), level.end()) + 1 : 0;
    std::vector<int64_t> order(n);
    for (int64_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return level[a] < level[b]; });
    std::vector<int64_t> lstart(nlev + 1, 0);
    for (int64_t i = 0; i < n; ++i) lstart[level[i] + 1]++;
    for (int64_t l = 0; l < nlev; ++l) lstart[l + 1] += lstart[l];
    std::vector<int64_t> cptr(n + 1, 0), cidx;
    for (int64_t i = 0; i < n; ++i) {
      if (d[i] >= 0) cptr[d[i] + 1]++;
      if (sr[i] >= 0) cptr[sr[i] + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) cptr[i + 1] += cptr[i];
    cidx.resize(cptr[n]);
    {
      std::vector<int64_t> fill(cptr.begin(), cptr.end() - 1);
      for (int64_t i = 0; i < n; ++i) {
        if (d[i] >= 0) cidx[fill[d[i]]++] = i;
        if (sr[i] >= 0) cidx[fill[sr[i]]++] = i;
      }
    }
    // device buffers
    DevBuf<int64_t> d_order, d_cptr, d_cidx, d_sire, d_dam;
    DevBuf<double> d_dii, Y;
    DevBuf<int32_t> d_gmap;
    d_order.resize(n); d_cptr.resize(n + 1); d_cidx.resize(std::max<int64_t>(1, cptr[n]));
    d_sire.resize(n); d_dam.resize(n); d_dii.resize(n); d_gmap.resize(ng);
    CBX_CUDA(cudaMemcpyAsync(d_order.p, order.data(), n * 8, cudaMemcpyHostToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(d_cptr.p, cptr.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s));
    if (cptr[n]) CBX_CUDA(cudaMemcpyAsync(d_cidx.p, cidx.data(), cptr[n] * 8, cudaMemcpyHostToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(d_sire.p, sr.data(), n * 8, cudaMemcpyHostToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(d_dam.p, d.data(), n * 8, cudaMemcpyHostToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(d_dii.p, dii.data(), n * 8, cudaMemcpyHostToDevice, s));
    CBX_CUDA(cudaMemcpyAsync(d_gmap.p, gmap, ng * 4, cudaMemcpyHostToDevice, s));
    // Y = S (n x ng row-major): unit vector of genotyped animal k in column k
    Y.resize((size_t)n * ng);
    Y.zero(s);
    for (int64_t k = 0; k < ng; ++k) CBX_REQUIRE(gmap[k] >= 0 && gmap[k] < n, CBX_ERR_ARG, "genotyped map out of range");
    ped::k_set_units<<<ped::gridn(ng, 256, 1024), 256, 0, s>>>(d_gmap.p, ng, Y.p);
    h->launched("k_set_units");
    const unsigned gx = ped::gridn(ng, 256, 64);
    for (int64_t l = nlev - 1; l >= 0; --l) {
      const int64_t cnt = lstart[l + 1] - lstart[l];
      ped::k_pull_children<<<dim3(gx, (unsigned)std::min<int64_t>(cnt, 65535)), 256, 0, s>>>(
          d_order.p + lstart[l], cnt, d_cptr.p, d_cidx.p, ng, Y.p);
      h->launched("k_pull_children");
    }
    for (int64_t l = 0; l < nlev; ++l) {
      const int64_t cnt = lstart[l + 1] - lstart[l];
      ped::k_pull_parents<<<dim3(gx, (unsigned)std::min<int64_t>(cnt, 65535)), 256, 0, s>>>(
          d_order.p + lstart[l], cnt, d_sire.p, d_dam.p, d_dii.p, ng, Y.p);
      h->launched("k_pull_parents");
    }
    DevBuf<double> A22, Gd, Gb;
    A22.resize((size_t)ng * ng);
    ped::k_gather_rows<<<ped::gridn(ng * ng, 256, 8 * h->num_sms), 256, 0, s>>>(Y.p, d_gmap.p, ng, A22.p);
    h->launched("k_gather_rows");
    Y.release();
    if (A22_out) CBX_CUDA(cudaMemcpyAsync(A22_out, A22.p, (size_t)ng * ng * 8, cudaMemcpyDeviceToHost, s));
    // G: host input or the device GRM of this handle
    DevBuf<double> Gh;
    const double* Gp = nullptr;
    if (G) {
      Gh.resize((size_t)ng * ng);
      CBX_CUDA(cudaMemcpyAsync(Gh.p, G, (size_t)ng * ng * 8, cudaMemcpyHostToDevice, s));
      Gp = Gh.p;
    } else {
      CBX_REQUIRE(h->G.p && h->G_n == ng, CBX_ERR_STATE, "no device GRM of order ng (cbx_grm_bed)");
      Gp = h->G.p;
    }
    // tuneG (relationship_builder.cpp:539-565)
    double a = 0.0, b = 1.0;
    if (tune_g) {
      const unsigned g = ped::gridn(ng * ng, 256, 4 * h->num_sms);
      DevBuf<double> pg, pa;
      pg.resize(2 * g);
      pa.resize(2 * g);
      ped::k_sum_diag_all<<<g, 256, 0, s>>>(Gp, ng, pg.p);
      h->launched("k_sum_diag_all");
      ped::k_sum_diag_all<<<g, 256, 0, s>>>(A22.p, ng, pa.p);
      h->launched("k_sum_diag_all");
      std::vector<double> hg(2 * g), ha(2 * g);
      CBX_CUDA(cudaMemcpyAsync(hg.data(), pg.p, 2 * g * 8, cudaMemcpyDeviceToHost, s));
      CBX_CUDA(cudaMemcpyAsync(ha.data(), pa.p, 2 * g * 8, cudaMemcpyDeviceToHost, s));
      CBX_CUDA(cudaStreamSynchronize(s));
      double sgd = 0, sga = 0, sad = 0, saa = 0;
      for (unsigned k = 0; k < g; ++k) {
        sgd += hg[2 * k]; sga += hg[2 * k + 1];
        sad += ha[2 * k]; saa += ha[2 * k + 1];
      }
      const double mgd = sgd / ng, mad = sad / ng;
      const double noff = (double)ng * (ng - 1);
      const double mgo = noff > 0 ? (sga - sgd) / noff : 0.0;
      const double mao = noff > 0 ? (saa - sad) / noff : 0.0;
      if (std::abs(mgd - mgo) > 1e-12) b = (mad - mao) / (mgd - mgo);
      a = mad - b * mgd;
    }
    Gb.resize((size_t)ng * ng);
    ped::k_blend<<<ped::gridn(ng * ng, 256, 8 * h->num_sms), 256, 0, s>>>(Gp, A22.p, ng * ng, a, b, alpha, Gb.p);
    h->launched("k_blend");
    Gh.release();
    // Gb^-1 (eigen-bending), A22^-1 (Cholesky, ridge on the diagonal first)
    DevBuf<double> Gbi;
    Gbi.resize((size_t)ng * ng);
    invert_psd_device(h, Gb.p, ng, ridge, Gbi.p);
    Gb.release();
    if (ridge > 0.0) {
      std::vector<double> diag(ng);
      CBX_CUDA(cudaMemcpy2DAsync(diag.data(), 8, A22.p, (ng + 1) * 8, 8, ng, cudaMemcpyDeviceToHost, s));
      CBX_CUDA(cudaStreamSynchronize(s));
      for (auto& v : diag) v += ridge;
      CBX_CUDA(cudaMemcpy2DAsync(A22.p, (ng + 1) * 8, diag.data(), 8, 8, ng, cudaMemcpyHostToDevice, s));
    }
    CBX_REQUIRE(chol_inverse_device(h, A22.p, ng), CBX_ERR_FACTOR, "A22 is not positive definite");
    Gd.resize((size_t)ng * ng);
    ped::k_combine<<<ped::gridn(ng * ng, 256, 8 * h->num_sms), 256, 0, s>>>(Gbi.p, A22.p, ng * ng, tau, omega, Gd.p);
    h->launched("k_combine");
    if (Gd_out) CBX_CUDA(cudaMemcpyAsync(Gd_out, Gd.p, (size_t)ng * ng * 8, cudaMemcpyDeviceToHost, s));
    CBX_CUDA(cudaStreamSynchronize(s));
    // the block stays on the device for later MMEs of this handle
    h->Hd = std::move(Gd);
    h->Hd_n = ng;
    ++h->Hd_gen;
    if (int rc = cbx_mme_set_qinv_split(h, ap.data(), ac.data(), av.data(), nullptr, ng, gmap); rc != CBX_OK)
      throw Error(rc, h->last_error);
  });
}
