// Device-resident mixed-model equations (one random component).
//
// LHS(lambda) = D + lambda [0 0; 0 Qinv], with
//   D    = W'W as CSR over dim = p + q rows (W = [X Z], records on the host),
//   Qinv = Qs + S Qd S^T: Qs an optional sparse q x q CSR (A^-1 in ssGBLUP),
//          Qd an optional dense ng x ng block (G^-1, or G_blend^-1 - A22^-1
//          pre-combined), S the genotyped scatter map (ng -> [0, q)).
// FP64 copies drive refinement and the plain FP64 path; FP32 copies drive the
// mixed-precision bulk iterations.
#pragma once
#include <algorithm>
#include <memory>
#include <vector>
#include "devbuf.h"

namespace cbx {

template <typename T>
struct Csr {
  int32_t rows = 0;
  int64_t nnz = 0;
  DevBuf<int32_t> ptr;  // rows + 1 (int32 offsets; nnz < 2^31)
  DevBuf<int32_t> col;
  DevBuf<T> val;
};

// Type-erased per-RHS-count solver workspace (see mme.cu).
struct SolverBase {
  virtual ~SolverBase() = default;
  // forget everything derived from an MME (kept buffers are re-checked and
  // rewritten before use) when the solver moves to a rebuilt MME of the same size
  virtual void rebind() = 0;
};

struct Mme {
  int64_t n_rec = 0, p = 0, q = 0, dim = 0;
  // records
  DevBuf<double> y;                // n_rec
  DevBuf<int32_t> aid;             // n_rec, 1-based into Qinv, 0 = none
  DevBuf<int32_t> x_ptr, x_col;    // fixed-effect design CSR (n_rec rows)
  DevBuf<double> x_val;
  Csr<double> D64;                 // W'W
  Csr<float> D32;
  DevBuf<double> rhs;              // W'y (dim)
  // fixed-effect rows of W'W cut into segments of at most FIX_SEG entries
  int32_t nseg = 0;
  DevBuf<int32_t> seg_row, seg_lo, seg_hi, fix_seg_ptr;  // fix_seg_ptr: p + 1
  DevBuf<double> diagD;            // diag(W'W) (dim)
  // Qinv
  bool has_dense = false, has_sparse = false;
  int64_t ng = 0, ld = 0;          // dense block order and row pitch (multiple of 4)
  DevBuf<double> Qd64;             // ng x ld row-major
  // Low-precision copies hold the block minus a constant, Qd - qshift (qshift
  // = the mean off-diagonal entry), so that a large common offset -- an
  // eigen-bent G^-1 adds clamp^-1 / n to every entry -- does not eat the FP32
  // mantissa; the products add qshift * (column sum) back, the column sums
  // taken in FP64.  ng x ld each.
  DevBuf<float> Qd32;              // fl32(Qd - qshift)
  DevBuf<float> Qlo32;             // fl32(Qd - qshift - Qd32): with Qd32 the float-float block
  double qshift = 0.0;
  DevBuf<uint16_t> Qbf;            // bf16(Qd - qshift), ng x ld (only with CBX_BF16=1)
  // the handle's device block these copies were made from (G^-1 of
  // cbx_invert_psd or the H^-1 block of cbx_ssgblup_qinv) and its generation
  // there; a later MME built from the same, unchanged block keeps them
  const void* planes_src = nullptr;
  int64_t planes_gen = -1;
  // row scales of the Qd32 / Qlo32 planes for the fixed-point tensor-core
  // refinement product (valid while fx_rows_ok), and its scratch
  DevBuf<int32_t> fx_rowexp;
  bool fx_rows_ok = false;
  DevBuf<uint16_t> fx_bdig;
  DevBuf<int32_t> fx_cexp;
  DevBuf<double> fx_part;
  DevBuf<int32_t> gmap;            // ng -> u index
  DevBuf<int32_t> ginv;            // q -> dense index or -1
  Csr<double> Qs64;
  Csr<float> Qs32;
  DevBuf<double> diagQ;            // diag(Qinv) (q)
  // block-Jacobi fixed block: (X'X + ridge I)^-1, p x p
  DevBuf<double> A11inv64;
  DevBuf<float> A11inv32;
  // host copies used by the REML driver: records, the fixed-effect design
  // (CSR per record) and W'y
  std::vector<double> y_host;
  double yty = 0.0;
  std::vector<int32_t> aid_host, xp_host, xc_host;
  std::vector<double> xv_host, rhs_host;
  // warm start of the data solve (the reference keeps last_solution)
  DevBuf<double> last_solution;
  bool has_last = false;
  // residual b - A(last_lam) last_solution left by a mixed-precision data solve
  DevBuf<double> last_resid;
  bool has_last_resid = false;
  double last_lam = 0.0;
  // probe solutions of the previous REML iteration or gradient (the probe
  // stream repeats at every call), with their residuals and lambda per column
  DevBuf<double> probe_x, probe_r;
  std::vector<double> probe_lam;   // per stored column
  std::vector<char> probe_r_ok;    // residual column valid (mixed-precision solve)
  int probe_seed = -1;
  // right-hand sides of the EM iteration and the gradient, column-major
  // dim x (1 + probe_cap): column 0 = W'y, column 1 + j = [0; z_j] for
  // Rademacher probe j.  The probe stream restarts at the same seed at every
  // call, so each batch of probes is generated on the host and uploaded once
  // (probe_have[j]).
  DevBuf<double> em_B;
  std::vector<char> probe_have;
  int em_B_seed = -1;
  int probe_cap = 0;               // probe columns allocated in em_B / probe_x / probe_r / probe_zv
  // z_j' Qinv C^uu z_j of every probe column solved by the last forward pass
  DevBuf<double> probe_zv;
  // Forward state of the last EM iteration (or gradient): its point (var_u,
  // var_e), solver settings, e'e and u'Qinv u of its data solve, and how many
  // leading probe columns were solved there (their probe_zv values are valid).
  // The REML score at that point needs nothing else.
  struct Forward {
    bool valid = false;
    double vu = 0.0, ve = 0.0, pcg_tol = 0.0;
    int precision = -1, seed = -1, solved = 0;
    double uQu = 0.0, e_sse = 0.0;
  } fwd;
  // The operator changed: residual carries and the forward state no longer hold.
  // keep_solutions leaves the last solutions as starting points of the next solves.
  void drop_carry(bool keep_solutions = false) {
    has_last_resid = false;
    std::fill(probe_r_ok.begin(), probe_r_ok.end(), 0);
    fwd.valid = false;
    if (!keep_solutions) {
      has_last = false;
      probe_lam.clear();
      probe_r_ok.clear();
    }
  }
  // persistent solver workspaces, indexed by log2 of the RHS block width
  std::unique_ptr<SolverBase> solvers[8];
  // scratch column-major buffers of the C ABI
  DevBuf<double> io_b, io_x;
};

}  // namespace cbx
