"""Mixed-model equations on the device (mirror of MMELHSBuilder + PCGSolver).

Reference interfaces mirrored: ``MMELHSBuilder(recs, fd, components)``,
``build_lhs(lambda)``, ``build_rhs`` (src/core/mme_builder.h:26-71) and
``PCGSolver::solve(tol, max_iter, .., initial_guess)``
(src/core/pcg_solver.h:436-536).  Records follow ``GenRecord`` (aid is a 1-based
index into Qinv, 0 = none) and ``FixedDesignG::rows`` (src/core/design.h:20-38).
"""
from __future__ import annotations

import numpy as np

from ._lib import Handle, lib, ptr

FP64, MIXED = 0, 1
REL, ABS = 0, 1


def rows_to_csr(rows):
    """FixedDesignG::rows (list of (col, val) lists) -> (ptr int64, col int32, val float64)."""
    ptr_ = np.zeros(len(rows) + 1, dtype=np.int64)
    for i, r in enumerate(rows):
        ptr_[i + 1] = ptr_[i] + len(r)
    col = np.array([c for r in rows for c, _ in r], dtype=np.int32)
    val = np.array([v for r in rows for _, v in r], dtype=np.float64)
    return ptr_, col, val


class DeviceMME:
    def __init__(self, handle: Handle, y, aid, rows, p: int, q: int):
        self.h = handle
        self.p, self.q = int(p), int(q)
        self.dim = self.p + self.q
        y = np.ascontiguousarray(y, dtype=np.float64)
        aid = np.ascontiguousarray(aid, dtype=np.int32)
        fp, fc, fv = rows_to_csr(rows) if not isinstance(rows, tuple) else rows
        self._keep = (y, aid, fp, fc, fv)
        handle.check(lib().cbx_mme_create(handle.raw, y.size, self.p, self.q, ptr(y), ptr(aid),
                                          ptr(fp), ptr(fc), ptr(fv)))

    def set_qinv_dense(self, Qinv=None):
        if Qinv is None:
            self.h.check(lib().cbx_mme_set_qinv_dense(self.h.raw, None, self.q))
        else:
            Q = np.ascontiguousarray(Qinv, dtype=np.float64)
            self.h.check(lib().cbx_mme_set_qinv_dense(self.h.raw, ptr(Q), self.q))

    def set_qinv_split(self, a_ptr, a_col, a_val, Gd=None, gmap=None):
        """Qinv = A^-1 (CSR) + S Gd S^T.  Gd None with a gmap uses the dense block
        that ssgblup_qinv left on the device (order len(gmap))."""
        a_ptr = np.ascontiguousarray(a_ptr, dtype=np.int64)
        a_col = np.ascontiguousarray(a_col, dtype=np.int32)
        a_val = np.ascontiguousarray(a_val, dtype=np.float64)
        gmap = None if gmap is None else np.ascontiguousarray(gmap, dtype=np.int32)
        ng = Gd.shape[0] if Gd is not None else (0 if gmap is None else gmap.size)
        Gd = None if Gd is None else np.ascontiguousarray(Gd, dtype=np.float64)
        self.h.check(lib().cbx_mme_set_qinv_split(self.h.raw, ptr(a_ptr), ptr(a_col), ptr(a_val),
                                                  ptr(Gd), ng, ptr(gmap)))

    def pcg_solve(self, lam, B, X0=None, tol=1e-10, maxit=10000, tol_mode=REL, precision=FP64):
        """Solve LHS(lam) X = B; B is (dim,) or (dim, k).  Returns (X, iters, relres)."""
        B = np.asarray(B, dtype=np.float64)
        one = B.ndim == 1
        Bc = np.ascontiguousarray(B.reshape(self.dim, -1).T)  # column-major = row per RHS
        k = Bc.shape[0]
        X = np.zeros_like(Bc) if X0 is None else np.ascontiguousarray(
            np.asarray(X0, dtype=np.float64).reshape(self.dim, -1).T)
        it = np.zeros(k, dtype=np.int32)
        rr = np.zeros(k, dtype=np.float64)
        self.h.check(lib().cbx_pcg_solve(self.h.raw, float(lam), k, ptr(Bc), ptr(X),
                                         0 if X0 is None else 1, float(tol), int(maxit),
                                         int(tol_mode), int(precision), ptr(it), ptr(rr)))
        X = X.T
        return (X[:, 0] if one else X), it, rr

    def qinv_apply(self, X):
        X = np.asarray(X, dtype=np.float64)
        one = X.ndim == 1
        Xc = np.ascontiguousarray(X.reshape(self.q, -1).T)
        Y = np.zeros_like(Xc)
        self.h.check(lib().cbx_qinv_apply(self.h.raw, Xc.shape[0], ptr(Xc), ptr(Y)))
        Y = Y.T
        return Y[:, 0] if one else Y
