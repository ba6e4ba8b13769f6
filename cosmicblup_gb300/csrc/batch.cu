// Batched independent GBLUP problems on one GPU (cbx_batch_reml).
//
// The reference runs one problem per process: GrmBuilder::compute
// (src/core/grm_builder.cpp:63-405), invert_psd_matrix
// (src/core/matrix_io.cpp:488-501) and AI_REML::solve (src/core/vce.cpp:741-837).
// Here a pool of host threads, each owning a cbx_handle (its own stream,
// cuSOLVER / cuBLAS handles and device buffers), takes the problems largest
// first.  The small problems of a batch are latency-bound one at a time; their
// streams overlap on the GPU.  Each problem runs exactly the single-problem
// calls, so its results do not depend on the batch it is in.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>
#include "handle.h"

extern "C" int cbx_batch_reml(int device, int32_t nprob, const cbx_batch_problem* probs, float min_maf,
                              const cbx_reml_config* cfg, int32_t nworkers, cbx_batch_result* results) {
  if (nprob < 0 || (nprob > 0 && (!probs || !results)) || !cfg || nworkers < 1) return CBX_ERR_ARG;
  if (nprob == 0) return CBX_OK;
  // largest first (GRM and inverse work grows with n^2 m and n^3)
  std::vector<int32_t> order(nprob);
  for (int32_t i = 0; i < nprob; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    const double wa = (double)probs[a].n * probs[a].n * ((double)probs[a].m + probs[a].n);
    const double wb = (double)probs[b].n * probs[b].n * ((double)probs[b].m + probs[b].n);
    return wa > wb;
  });
  for (int32_t i = 0; i < nprob; ++i) results[i].status = CBX_ERR_STATE;
  std::atomic<int32_t> next{0};
  const int32_t nw = std::min(nworkers, nprob);
  auto worker = [&]() {
    cbx_handle* h = nullptr;
    if (cbx_create(device, &h) != CBX_OK) {
      if (h) cbx_destroy(h);
      return;  // the problems this worker would have taken stay CBX_ERR_STATE
    }
    for (int32_t k = next.fetch_add(1); k < nprob; k = next.fetch_add(1)) {
      const int32_t i = order[k];
      const cbx_batch_problem& pb = probs[i];
      cbx_batch_result& r = results[i];
      const auto t0 = std::chrono::steady_clock::now();
      double s2pq = 0.0;
      int64_t nval = 0;
      int rc = cbx_grm_bed(h, pb.bed, pb.bed_bytes, pb.n, pb.m, min_maf, 1, 2048, nullptr, nullptr, nullptr, &s2pq,
                           &nval);
      if (rc == CBX_OK) rc = cbx_invert_psd(h, nullptr, pb.n, 0.0, nullptr);
      if (rc == CBX_OK)
        rc = cbx_mme_create(h, pb.n_rec, pb.p, pb.n, pb.y, pb.aid, pb.fx_ptr, pb.fx_col, pb.fx_val);
      if (rc == CBX_OK) rc = cbx_mme_set_qinv_dense(h, nullptr, pb.n);
      double vu = pb.var_u, ve = pb.var_e;
      int32_t it = 0, conv = 0;
      if (rc == CBX_OK) {
        std::vector<cbx_reml_iter_info> hist((size_t)std::max(cfg->max_iter, 1));
        rc = cbx_reml_solve(h, cfg, &vu, &ve, &it, &conv, r.solution, hist.data());
        int64_t pi = 0;
        for (int32_t j = 0; j < it && j < (int32_t)hist.size(); ++j) pi += hist[j].pcg_iters;
        r.pcg_iters = pi;
      }
      r.status = rc;
      r.var_u = vu;
      r.var_e = ve;
      r.iterations = it;
      r.converged = conv;
      r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    cbx_destroy(h);
  };
  std::vector<std::thread> pool;
  for (int32_t t = 0; t < nw; ++t) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
  for (int32_t i = 0; i < nprob; ++i)
    if (results[i].status != CBX_OK) return results[i].status;
  return CBX_OK;
}
