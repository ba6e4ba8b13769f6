"""Oracle: single-component AI_REML iterations (test infrastructure).

Restates ``AI_REML`` for one random component with a dense Qinv
(src/core/vce.cpp):
* the outer loop and stop rule sum|delta| < tol (:741-837);
* the EM branch with Hutchinson traces (:1490-1574) through
  ``estimate_trace_Qinv_Cuu`` (:1266-1315) and the adaptive estimator
  (oracle.rng.adaptive_trace), each MME solve by block-Jacobi PCG warm-started
  from the previous solve's solution (``last_solution``, :1226-1235);
* ``stabilize_variance`` clamping to [0.1x, 10x] of the previous value (:1379-1389);
* ``run_dense_exact_step`` (:2949-3195) with ``project_spd_2x2`` (:267-283);
* ``ai_data_step``: ``run_aireml_step`` (:2414-2857) on its direct-solver
  branch, with ``calc_logL_internal`` (:3533-3588);
* ``SparseEM``: the same EM iteration on a sparse MME (single-step H^-1 of
  thousands of animals), each system solved directly by sparse LU.
"""
from __future__ import annotations

import numpy as np

from .mme import BlockJacobi, pcg
from .rng import adaptive_trace


def project_spd_2x2(A, eps_rel=1e-8, eps_abs=1e-12):
    S = 0.5 * (A + A.T)
    w, Q = np.linalg.eigh(S)
    floor = max(eps_abs, eps_rel * max(w.max(), 0.0))
    w = np.maximum(w, floor)
    return (Q * w) @ Q.T


class AIREML:
    def __init__(self, mme, Qinv, var_u, var_e, max_iter=20, tol=1e-4, mc_samples=100,
                 pcg_tol=1e-10, pcg_maxit=10000):
        self.mme, self.Qinv = mme, np.asarray(Qinv, dtype=np.float64)
        self.var_u, self.var_e = float(var_u), float(var_e)
        self.max_iter, self.tol, self.mc_samples = max_iter, tol, mc_samples
        self.pcg_tol, self.pcg_maxit = pcg_tol, pcg_maxit
        self.last_solution = None
        y = mme.y
        self.y_var = max(1e-12, ((y - y.mean()) ** 2).sum() / (len(y) - 1)) if len(y) > 1 \
            else max(1e-12, float(y @ y))
        self.history = []
        self.pcg_iters = []
        self.dense_initialized = False

    # --- helpers --------------------------------------------------------------
    def stabilize(self, proposed, previous):
        floor, ceil = 1e-12, max(1.0, self.y_var * 1e6)
        if not np.isfinite(proposed) or proposed <= 0.0:
            return max(previous, floor)
        lo, hi = floor, ceil
        if np.isfinite(previous) and previous > 0.0:
            lo = max(lo, previous * 0.1)
            hi = min(hi, previous * 10.0)
        if lo > hi:
            lo = floor
        return min(max(proposed, lo), hi)

    def lam(self, vu=None, ve=None):
        vu = self.var_u if vu is None else vu
        ve = self.var_e if ve is None else ve
        return ve / max(vu, 1e-9)

    def solve_lhs(self, A, rhs, precond):
        x, it, rel, _ = pcg(lambda v: A @ v, rhs, precond, self.pcg_tol, self.pcg_maxit,
                            x0=self.last_solution)
        self.pcg_iters.append(it)
        self.last_solution = x
        return x

    # --- EM with Hutchinson traces ----------------------------------------------
    def em_iteration(self):
        m = self.mme
        p, q, n = m.p, m.q, m.n
        start_vu, start_ve = self.var_u, self.var_e
        lam = self.lam()
        A = m.lhs(self.Qinv, lam)
        M = BlockJacobi(A, p)
        sol = self.solve_lhs(A, m.rhs(), M)
        b, u = sol[:p], sol[p:]
        e = m.y - m.mult_design(b, u)
        e_sse = e @ e
        uQu = u @ (self.Qinv @ u)
        n_samp = max(5, self.mc_samples // 2)

        def op(z):
            rhs = np.zeros(p + q)
            rhs[p:] = z
            s = self.solve_lhs(A, rhs, M)
            return self.Qinv @ s[p:]

        tr, used, vals = adaptive_trace(q, op, max(30, n_samp // 3), max(100, n_samp), 0.05, 42)
        self.last_trace = (tr, used, vals)
        vu_new = (uQu + tr * self.var_e) / q
        self.var_u = self.stabilize(vu_new, start_vu)
        tr_c = (p + q) - lam * tr
        ve_new = (e_sse + start_ve * tr_c) / n
        self.var_e = self.stabilize(ve_new, start_ve)
        self.solution = sol
        self.history.append(("EM", self.var_u, self.var_e))
        return {"sol": sol, "e_sse": e_sse, "uQu": uQu, "trace": tr, "samples": used}

    # --- dense exact AI step ------------------------------------------------------
    def _init_dense(self):
        m = self.mme
        L = np.linalg.cholesky(self.Qinv)
        Linv = np.linalg.inv(L)
        self.A_dense = Linv.T @ Linv
        self.log_det_A = -2.0 * np.log(np.diag(L)).sum()
        idx = m.aid - 1
        ok = (m.aid > 0) & (m.aid <= m.q)
        Z = np.zeros((m.n, m.n))
        sub = np.where(ok)[0]
        Z[np.ix_(sub, sub)] = self.A_dense[np.ix_(idx[sub], idx[sub])]
        self.ZAZt = Z
        self.dense_initialized = True

    def logL(self, vu, ve):
        m = self.mme
        n, p, q = m.n, m.p, m.q
        C = m.lhs(self.Qinv, ve / vu)
        try:
            Lc = np.linalg.cholesky(C)
        except np.linalg.LinAlgError:
            return -1e18
        ld_C = 2.0 * np.log(np.diag(Lc)).sum()
        s = np.linalg.solve(C, m.rhs())
        e = m.y - m.mult_design(s[:p], s[p:])
        yPy = m.y @ e / ve
        m2 = ld_C + (n - p - q) * np.log(ve) + q * np.log(vu) + yPy + self.log_det_A
        return -0.5 * m2

    def dense_exact_step(self):
        if not self.dense_initialized:
            self._init_dense()
        m = self.mme
        n, p, q = m.n, m.p, m.q
        vu, ve = self.var_u, self.var_e
        C = m.lhs(self.Qinv, ve / vu)
        Lc = np.linalg.cholesky(C)
        ld_C = 2.0 * np.log(np.diag(Lc)).sum()
        sol = np.linalg.solve(C, m.rhs())
        e = m.y - m.mult_design(sol[:p], sol[p:])
        cur = -0.5 * (ld_C + (n - p - q) * np.log(ve) + q * np.log(vu) + m.y @ e / ve
                      + self.log_det_A)
        CiWt = np.linalg.solve(C, m.W.T)
        H = m.W @ CiWt
        P = -H / ve
        P[np.diag_indices(n)] += 1.0 / ve
        Mu = P @ self.ZAZt
        AI = 0.5 * np.array([[np.sum(Mu * Mu.T), np.sum(Mu * P)],
                             [np.sum(Mu * P), np.sum(P * P)]])
        Py = e / ve
        grad = np.array([-0.5 * np.trace(Mu) + 0.5 * Py @ (self.ZAZt @ Py),
                         -0.5 * np.trace(P) + 0.5 * Py @ Py])
        AI = project_spd_2x2(AI)
        delta = np.linalg.solve(AI, grad)
        self.last_ai = (AI, grad, cur)
        new = cur
        for k in range(6):
            vu_n, ve_n = vu + delta[0], ve + delta[1]
            if vu_n > 0 and ve_n > 0:
                new = self.logL(vu_n, ve_n)
                if new > cur or k == 5:
                    self.var_u, self.var_e = vu_n, ve_n
                    self.history.append(("AI(Exact)", new, vu, ve_n))
                    self.solution = sol
                    return True
            delta = delta * 0.5
        return False

    # --- data-driven AI step (direct-solver branch) -----------------------------------
    def logL_internal(self, vu, ve):
        """calc_logL_internal (vce.cpp:3533-3588): log|C| from the factor of the LHS,
        -1e20 when it is not positive definite."""
        m = self.mme
        n, p, q = m.n, m.p, m.q
        C = m.lhs(self.Qinv, ve / max(vu, 1e-9))
        try:
            L = np.linalg.cholesky(C)
        except np.linalg.LinAlgError:
            return -1e20
        ld = 2.0 * np.log(np.diag(L)).sum()
        rhs = m.rhs()
        sol = np.linalg.solve(C, rhs)
        yPy = (m.y @ m.y - sol @ rhs) / ve
        return -0.5 * (ld + (n - p - q) * np.log(ve) + q * np.log(max(vu, 1e-9)) + yPy)

    def ai_data_step(self):
        """run_aireml_step (vce.cpp:2414-2857) with a direct solver: the exact
        trace tr(Qinv C^uu) (the Takahashi value), AI_ij = 1/2 v_i' P v_j from two
        extra solves (:2596-2633), the EM-consistent score (:2648-2675),
        project_spd_2x2, the Newton direction with its fallbacks (:2697-2737),
        the 100x / 5x step guards and up to 15 logL-checked halvings (:2760-2839).
        Returns False when the step fails (the caller runs EM)."""
        m = self.mme
        n, p, q = m.n, m.p, m.q
        if not np.isfinite(self.var_u) or self.var_u <= 0:
            self.var_u = 1e-6
        if not np.isfinite(self.var_e) or self.var_e <= 0:
            self.var_e = 1e-6
        vu, ve = self.var_u, self.var_e
        lam = ve / max(vu, 1e-9)
        C = m.lhs(self.Qinv, lam)
        rhs = m.rhs()
        sol = np.linalg.solve(C, rhs)
        u = sol[p:]
        e = m.y - m.mult_design(sol[:p], u)
        Ci = np.linalg.inv(C)
        tr = float(np.sum(self.Qinv * Ci[p:, p:]))
        v_u = m.Z @ u / vu
        v_e = e / ve

        def Pv(v):
            x = np.linalg.solve(C, m.W.T @ v)
            return (v - m.W @ x) / ve

        Pvu, Pve = Pv(v_u), Pv(v_e)
        AI = 0.5 * np.array([[v_u @ Pvu, v_u @ Pve], [v_u @ Pve, v_e @ Pve]])
        ltr = min(lam * tr, q - 1e-6)
        grad = np.array([0.5 * (u @ (self.Qinv @ u) + tr * ve - q * vu) / vu**2,
                         0.5 * (e @ e - ve * (n - p - q + ltr)) / ve**2])
        AI = project_spd_2x2(AI)
        try:
            np.linalg.cholesky(AI)
            delta = np.linalg.solve(AI, grad)
        except np.linalg.LinAlgError:
            det = np.linalg.det(AI)
            if abs(det) < 1e-20:
                mx = max(abs(grad[0]) / vu, abs(grad[1]) / ve)
                delta = grad * (0.1 / mx if mx > 0 else 0.0)
            else:
                delta = np.linalg.inv(AI) @ grad
        if not np.all(np.isfinite(delta)):
            return False
        if abs(delta[0]) > 100 * vu or abs(delta[1]) > 100 * ve:
            return False
        cur = self.logL_internal(vu, ve)
        if not np.isfinite(cur):
            cur = -1e18
        for _ in range(15):
            vu_n, ve_n = vu + delta[0], ve + delta[1]
            if vu_n <= 0 or ve_n <= 0 or abs(delta[0]) > 5 * vu or abs(delta[1]) > 5 * ve:
                delta = delta * 0.5
                continue
            new = self.logL_internal(vu_n, ve_n)
            if np.isfinite(new) and new > cur:
                self.var_u, self.var_e = vu_n, ve_n
                self.history.append(("AI(data)", new, vu_n, ve_n))
                self.last_ai_step = {"trace": tr, "logL": new, "AI": AI, "grad": grad}
                self.solution = sol
                return True
            delta = delta * 0.5
        return False

    # --- outer loop -----------------------------------------------------------------
    def solve(self, dense_exact=None):
        dim = self.mme.dim
        if dense_exact is None:
            dense_exact = dim < 5000
        self.converged = False
        for it in range(self.max_iter):
            old_u, old_e = self.var_u, self.var_e
            if dense_exact:
                if not self.dense_exact_step():
                    self.em_iteration()
            else:
                self.em_iteration()
            diff = abs(self.var_e - old_e) + abs(self.var_u - old_u)
            self.iterations = it + 1
            if diff < self.tol:
                self.converged = True
                break
        return self.var_u, self.var_e


def hinv_sparse(Ainv_csr, Gd, gmap):
    """H^-1 = A^-1 + S Gd S^T as a scipy CSR matrix (SplitMatrixAdapter's operator,
    src/core/matrix_adapter.h:252-278, formed explicitly)."""
    import scipy.sparse as sp
    ptr, col, val = Ainv_csr
    q = len(ptr) - 1
    A = sp.csr_matrix((val, col, ptr), shape=(q, q))
    g = np.asarray(gmap)
    r = np.repeat(g, g.size)
    c = np.tile(g, g.size)
    D = sp.csr_matrix((np.asarray(Gd).ravel(), (r, c)), shape=(q, q))
    return (A + D).tocsr()


class SparseEM:
    """EM + Hutchinson REML iterations (vce.cpp:1490-1574) on a sparse MME.

    The same algorithm as AIREML.em_iteration -- data solve, e'e, u'Qinv u, the
    adaptive trace estimator of tr(Qinv C^uu) with the reference's probe stream
    (oracle.rng.adaptive_trace), the EM updates and stabilize_variance -- for
    problems too large for the dense restatement.  Each system is solved
    directly (scipy sparse LU of W'W + lambda [0 0; 0 Qinv]): the exact value
    the reference's PCG approximates to relative residual 1e-10.
    """

    def __init__(self, W, y, Qinv, p, var_u, var_e, mc_samples=100, seed=42):
        import scipy.sparse as sp
        self.W = sp.csr_matrix(W)
        self.y = np.asarray(y, dtype=np.float64)
        self.Qinv = sp.csr_matrix(Qinv)
        self.p = int(p)
        self.q = self.Qinv.shape[0]
        self.n = self.y.size
        self.WtW = (self.W.T @ self.W).tocsc()
        self.rhs = self.W.T @ self.y
        self.var_u, self.var_e = float(var_u), float(var_e)
        self.mc_samples, self.seed = mc_samples, seed
        y = self.y
        self.y_var = max(1e-12, ((y - y.mean()) ** 2).sum() / (len(y) - 1)) if len(y) > 1 \
            else max(1e-12, float(y @ y))

    stabilize = AIREML.stabilize

    def lhs(self, lam):
        import scipy.sparse as sp
        Z = sp.csr_matrix((self.p, self.p))
        return (self.WtW + sp.block_diag([Z, lam * self.Qinv])).tocsc()

    def em_iteration(self):
        from scipy.sparse.linalg import splu
        p, q, n = self.p, self.q, self.n
        start_vu, start_ve = self.var_u, self.var_e
        lam = start_ve / max(start_vu, 1e-9)
        lu = splu(self.lhs(lam), permc_spec="MMD_AT_PLUS_A")  # symmetric ordering: little fill
        sol = lu.solve(self.rhs)
        u = sol[p:]
        e = self.y - self.W @ sol
        e_sse = float(e @ e)
        uQu = float(u @ (self.Qinv @ u))
        n_samp = max(5, self.mc_samples // 2)

        def op(z):
            b = np.zeros(p + q)
            b[p:] = z
            return self.Qinv @ lu.solve(b)[p:]

        tr, used, _ = adaptive_trace(q, op, max(30, n_samp // 3), max(100, n_samp), 0.05, self.seed)
        self.var_u = self.stabilize((uQu + tr * start_ve) / q, start_vu)
        self.var_e = self.stabilize((e_sse + start_ve * ((p + q) - lam * tr)) / n, start_ve)
        self.solution = sol
        return {"sol": sol, "e_sse": e_sse, "uQu": uQu, "trace": tr, "samples": used}
