// Host-side interface of the multi-RHS PCG and of the Qinv product.
#pragma once
#include <vector>
#include "handle.h"

namespace cbx {

struct PcgResult {
  std::vector<int> iters;      // CG iterations per column (inner FP32 ones in mixed mode)
  std::vector<int> status;     // sv::ColStatus
  std::vector<double> relres;  // final relative residual (absolute in abs-tol mode)
  int refinements = 0;         // FP64 refinement steps (mixed mode)
  int64_t matvecs = 0;         // operator applications (all columns share one matrix read)
};

// Solve LHS(lambda) X = B for ncols right-hand sides stored column-major
// (dim x ncols) on the device.  X holds x0 when use_x0.  precision 0: FP64 PCG
// with the reference's relative recursive-residual stop; 1: FP32 PCG on the
// correction equation with FP64 true-residual refinement (stop on the true
// residual).  abs_tol: stop on ||r|| < tol (MatrixFreePCG) instead.
// Residual carried between mixed-precision solves of the same right-hand sides
// at neighbouring lambdas.  r_prev (column-major dim x ncols) = b - A(lam -
// dlam) x0 for the x0 passed in X; the initial residual at lam follows from it
// exactly with one sparse W'W product (k_carry_resid), no dense product.
// r_out receives the final residual b - A(lam) x of a mixed-precision solve.
// Either pointer may be null.
struct ResidCarry {
  const double* r_prev = nullptr;
  double dlam = 0.0;
  double* r_out = nullptr;
};

void pcg_solve(cbx_handle* h, double lam, int ncols, const double* B_cm, double* X_cm, bool use_x0,
               double tol, int maxit, int abs_tol, int precision, PcgResult& res,
               const ResidCarry* carry = nullptr);

// Y = Qinv X for ncols column-major q-vectors on the device.
void qinv_apply(cbx_handle* h, int ncols, const double* X_cm, double* Y_cm);

// Y = Qinv X_u for solutions X of A(lam) X = B whose true residuals R = B - A X
// are known (the mixed solver returns them): from A x = W'W x + lam [0; Qinv u],
// Qinv u = ((b - r)_u - (W'W x)_u) / lam, which needs only the sparse W'W.  Its
// error is that of r, i.e. of an FP64 residual.  Column-major: B, X, R are
// dim x ncols, Y is q x ncols.
void qinv_from_solution(cbx_handle* h, double lam, int ncols, const double* B_cm, const double* X_cm,
                        const double* R_cm, double* Y_cm);

// Record residual e = y - W sol (sol: dim) on the device; returns e'e.
double record_residual(cbx_handle* h, const double* sol_dev, double* e_dev);

}  // namespace cbx
