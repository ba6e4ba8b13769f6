"""Oracle: multi-trait GBLUP (test infrastructure).

Restates, in numpy FP64:
* ``MvEigenVce`` (src/core/eigen_vce.cpp:106-266) as GSVce calls it
  (src/variance/variance_estimator.cpp:289-298): projection of Y and G onto
  the null space of X' (Householder QR, Q.rightCols(n - p)), eigen-decomposition
  of the projected G with negative eigenvalues set to 0, Y rotated into that
  basis, Vg = Ve = Cov(Y) / 2 with the divisor n - p - 1, then EM updates
  ``updateEM`` (:163-237) until both relative Frobenius changes are below tol
  (``runNullModel``, :239-264);
* ``GSSolve::solveMultiTrait`` (src/solve/mixed_model_solver.cpp:425-524): the
  explicit Kronecker-product LHS (trait-major order) solved directly.

Vg and Ve do not depend on which orthonormal null-space basis the QR returns:
the projected eigenvectors A U are unique up to sign and rotations inside
repeated eigenvalues, and the EM sums are invariant to both.
"""
from __future__ import annotations

import numpy as np


def mv_prepare(Y, X, G):
    """Projection + eigen-decomposition; returns (D, Uty, n_eff, Vg0, Ve0)."""
    Y = np.asarray(Y, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    n, t = Y.shape
    p = X.shape[1]
    if p > 0:
        Q, _ = np.linalg.qr(X, mode="complete")
        A = Q[:, p:]
        Yr = A.T @ Y
        Gr = A.T @ G @ A
        n_eff = n - p
    else:
        Yr, Gr, n_eff = Y, np.asarray(G, dtype=np.float64), n
    D, U = np.linalg.eigh(0.5 * (Gr + Gr.T))
    D = np.where(D < 0, 0.0, D)
    Uty = U.T @ Yr
    Yc = Y - Y.mean(axis=0)
    cov = (Yc.T @ Yc) / (n_eff - 1)
    return D, Uty, n_eff, 0.5 * cov, 0.5 * cov


def em_update(D, Uty, Vg, Ve):
    """One ``updateEM`` pass (no covariates after projection), vectorised over samples."""
    n, t = Uty.shape
    V = D[:, None, None] * Vg[None] + Ve[None]          # n x t x t
    P = np.linalg.inv(V)
    Wg = D[:, None, None] * np.einsum("ab,ibc->iac", Vg, P)
    uh = np.einsum("iab,ib->ia", Wg, Uty)
    big = D > 1e-12
    Dsafe = np.where(big, D, 1.0)
    Sg = np.einsum("ia,ib->ab", uh[big] / Dsafe[big, None], uh[big]) \
        + big.sum() * Vg - np.einsum("iab,bc->ac", Wg[big], Vg) + (~big).sum() * Vg
    We = np.einsum("ab,ibc->iac", Ve, P)
    eh = np.einsum("iab,ib->ia", We, Uty)
    Se = eh.T @ eh + n * Ve - np.einsum("iab,bc->ac", We, Ve)
    return Sg / n, Se / n


def mv_eigen_vce(Y, X, G, max_iter=500, tol=1e-4):
    D, Uty, n_eff, Vg, Ve = mv_prepare(Y, X, G)
    for it in range(max_iter):
        Vg_new, Ve_new = em_update(D, Uty, Vg, Ve)
        dg = np.linalg.norm(Vg_new - Vg) / max(np.linalg.norm(Vg), 1e-12)
        de = np.linalg.norm(Ve_new - Ve) / max(np.linalg.norm(Ve), 1e-12)
        Vg, Ve = Vg_new, Ve_new
        if dg < tol and de < tol:
            return {"Vg": Vg, "Ve": Ve, "iterations": it + 1, "converged": True, "D": D, "Uty": Uty}
    return {"Vg": Vg, "Ve": Ve, "iterations": max_iter, "converged": False, "D": D, "Uty": Uty}


def mt_lhs_rhs(Y, X, Ginv, Vg, Ve):
    """The reference's explicit multi-trait MME (trait-major unknowns: beta then u)."""
    Y = np.asarray(Y, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    n, t = Y.shape
    p = X.shape[1]
    Vei, Vgi = np.linalg.inv(Ve), np.linalg.inv(Vg)
    C11 = np.kron(Vei, X.T @ X)
    C12 = np.kron(Vei, X.T)
    C22 = np.kron(Vei, np.eye(n)) + np.kron(Vgi, Ginv)
    L = np.block([[C11, C12], [C12.T, C22]])
    r1 = (X.T @ Y @ Vei.T).reshape(-1, order="F")
    r2 = (Y @ Vei.T).reshape(-1, order="F")
    return L, np.concatenate([r1, r2]), p * t


def mt_solve(Y, X, Ginv, Vg, Ve):
    L, r, pt = mt_lhs_rhs(Y, X, Ginv, Vg, Ve)
    sol = np.linalg.solve(L, r)
    return {"beta": sol[:pt], "u": sol[pt:], "sol": sol}
