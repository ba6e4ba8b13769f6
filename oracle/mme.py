"""Oracle: fixed-effect design, mixed-model equations and PCG (test infrastructure).

Restates, in FP64 numpy:
* ``buildFixedDesignGeneric`` (src/core/design.cpp:13-109): column 0 is mu;
  each categorical factor contributes its levels in std::set (byte-wise
  lexicographic) order except the first (base) level; then numeric covariates;
* ``MMELHSBuilder`` (src/core/mme_builder.cpp:72-423): LHS =
  [X'X X'Z; Z'X Z'Z + lambda Qinv], RHS = W'v, W x = X b + Z u; ``aid`` is a
  1-based index into Qinv, 0 for "no animal";
* ``invert_psd_matrix`` (src/core/matrix_io.cpp:488-501);
* ``PCGSolver::solve`` with the block-Jacobi and Jacobi preconditioners
  (src/core/pcg_solver.h:35-128, 436-536), relative recursive-residual stop;
* ``MatrixFreePCG::solve`` (src/core/matrix_free_pcg.h:20-66), absolute stop.
"""
from __future__ import annotations

import numpy as np


def build_fixed_design(cats, nums=None):
    """Return (p, rows, names); rows[i] is a list of (column, value)."""
    n = len(cats)
    ncat = len(cats[0]) if n else 0
    levels = []
    for j in range(ncat):
        lv = sorted({c[j] for c in cats if c[j] != ""}, key=lambda s: s.encode())
        levels.append(lv)
    names = ["mu"]
    p = 1
    for j, lv in enumerate(levels):
        for k in lv[1:]:
            names.append(f"factor{j + 1}_{k}")
            p += 1
    nnum = len(nums[0]) if (nums is not None and n) else 0
    names += [f"cov{j + 1}" for j in range(nnum)]
    p += nnum
    rows = []
    for i in range(n):
        nz = [(0, 1.0)]
        col = 1
        for j, lv in enumerate(levels):
            if not lv:
                continue
            for k in lv[1:]:
                if cats[i][j] == k:
                    nz.append((col, 1.0))
                col += 1
        for j in range(nnum):
            nz.append((col, float(nums[i][j])))
            col += 1
        rows.append(nz)
    return p, rows, names


class MME:
    """Dense-matrix restatement of the single-component MME (small sizes only).

    W'W = W^T W.  For records whose fixed-effect columns are distinct (every
    design FixedDesignG builds: one column per factor level or covariate) this is
    the reference's triplet assembly (src/core/mme_builder.cpp:107-176), which
    emits a record's (c_a, c_b) product once per pair a <= b."""

    def __init__(self, y, aid, rows, p, q):
        self.y = np.asarray(y, dtype=np.float64)
        self.aid = np.asarray(aid, dtype=np.int64)
        self.rows = rows
        self.p, self.q = int(p), int(q)
        self.n = len(self.y)
        X = np.zeros((self.n, self.p))
        for i, nz in enumerate(rows):
            for c, v in nz:
                if c < self.p:
                    X[i, c] += v
        Z = np.zeros((self.n, self.q))
        for i, a in enumerate(self.aid):
            if 0 < a <= self.q:
                Z[i, a - 1] = 1.0
        self.X, self.Z = X, Z
        self.W = np.hstack([X, Z])
        self.WtW = self.W.T @ self.W

    @property
    def dim(self):
        return self.p + self.q

    def lhs(self, Qinv, lam):
        L = self.WtW.copy()
        L[self.p:, self.p:] += lam * Qinv
        return L

    def rhs(self, v=None):
        return self.W.T @ (self.y if v is None else v)

    def mult_design(self, b, u):
        return self.X @ b + self.Z @ u


def invert_psd_matrix(M, ridge=0.0):
    """Eigen-bending inverse: clamp eigenvalues below max(1e-12 lmax, 1e-6)."""
    M = np.array(M, dtype=np.float64, copy=True)
    if ridge > 0.0:
        M[np.diag_indices_from(M)] += ridge
    w, U = np.linalg.eigh(M)
    eps = max(1e-12 * w.max(), 1e-6)
    w = np.where(w < eps, eps, w)
    return (U / w) @ U.T


class BlockJacobi:
    """LDLT of the fixed block (+ ridge) and Jacobi on the random part."""

    def __init__(self, A, p):
        self.p = p
        d = np.diag(A).copy()
        if p > 0:
            A11 = A[:p, :p].copy()
            ridge = max(1e-8 * np.abs(np.diag(A11)).max(), 1e-6)
            A11[np.diag_indices(p)] += ridge
            self.A11 = A11
        self.dinv = np.where(np.abs(d[p:]) > 1e-12, 1.0 / np.where(d[p:] == 0, 1, d[p:]), 1.0)

    def __call__(self, v):
        r = np.empty_like(v)
        if self.p > 0:
            r[:self.p] = np.linalg.solve(self.A11, v[:self.p])
        r[self.p:] = self.dinv * v[self.p:]
        return r


class Jacobi:
    def __init__(self, d):
        d = np.asarray(d, dtype=np.float64)
        self.dinv = np.where(np.abs(d) > 1e-12, 1.0 / np.where(d == 0, 1, d), 1.0)

    def __call__(self, v):
        return self.dinv * v


def pcg(matvec, b, precond, tol=1e-10, maxit=1000, x0=None):
    """PCGSolver::solve.  Returns (x, iterations, relative residual, restarts)."""
    n = b.shape[0]
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    r = b - matvec(x)
    z = precond(r)
    p = z.copy()
    rsold = r @ z
    bnorm = np.linalg.norm(b) or 1.0
    restarted = False
    restarts = 0
    for it in range(maxit):
        Ap = matvec(p)
        denom = p @ Ap
        if abs(denom) < 1e-300:
            if not restarted:
                z = precond(r)
                p = z.copy()
                rsold = r @ z
                restarted = True
                restarts += 1
                continue
            break
        alpha = rsold / denom
        x += alpha * p
        r -= alpha * Ap
        rel = np.linalg.norm(r) / bnorm
        if rel < tol:
            return x, it + 1, rel, restarts
        z = precond(r)
        rsnew = r @ z
        beta = rsnew / rsold
        p = z + beta * p
        rsold = rsnew
        if not (np.all(np.isfinite(x)) and np.all(np.isfinite(r))):
            break
    rel = np.linalg.norm(b - matvec(x)) / bnorm if np.linalg.norm(b) > 0 else 0.0
    return x, maxit, rel, restarts


def matrix_free_pcg(matvec, b, diag, tol=1e-10, maxit=1000, x0=None):
    """MatrixFreePCG::solve with a Jacobi preconditioner and ABSOLUTE stop ||r|| < tol."""
    n = b.shape[0]
    M = Jacobi(diag)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    r = b - matvec(x)
    if np.linalg.norm(r) < 1e-20:
        return x, 0
    z = M(r)
    p = z.copy()
    rz = r @ z
    for it in range(maxit):
        Ap = matvec(p)
        alpha = rz / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        if np.linalg.norm(r) < tol:
            return x, it + 1
        z = M(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, maxit


def sparse_data_part(aid, rows, p, q):
    """W'W as a scipy CSR matrix (dim x dim) and W as CSR (n x dim), for large cases."""
    import scipy.sparse as sp
    n = len(rows)
    r_idx, c_idx, vals = [], [], []
    for i, nz in enumerate(rows):
        for c, v in nz:
            r_idx.append(i)
            c_idx.append(c)
            vals.append(v)
    aid = np.asarray(aid)
    ok = (aid > 0) & (aid <= q)
    r_idx.extend(np.nonzero(ok)[0].tolist())
    c_idx.extend((p + aid[ok] - 1).tolist())
    vals.extend([1.0] * int(ok.sum()))
    W = sp.csr_matrix((vals, (r_idx, c_idx)), shape=(n, p + q))
    return (W.T @ W).tocsr(), W
