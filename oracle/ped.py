"""Oracle: pedigree relationship inverse and ssGBLUP H^-1 pieces (test infrastructure).

Restates (reference src/core/a_matrix.cpp and src/io/relationship_builder.cpp):
* ``complete_missing_parents_add_phantoms`` (a_matrix.cpp:42-51): parents outside
  [0, n) become unknown (-1);
* ``ml`` (a_matrix.cpp:127-186): inbreeding by the ancestor scan with path
  coefficients L; the scan runs over indices from max(sire, dam) down to 0 in
  decreasing order and visits every index whose L is positive -- here a sorted
  set of pending indices gives the same visiting order (and the same leftover
  L values for pedigrees that are not sorted parents-first);
* ``invertA_henderson`` (a_matrix.cpp:392-439) with
  ``enforceSymmetryAndDiagonal(A, 1e-12, 1e-15)`` (:58-79);
* the ssGBLUP assembly of ``MatrixBuilder::build`` (relationship_builder.cpp:
  495-584): A22, tuneG, alpha blend, eigen-bent inverse, A22^-1.
"""
from __future__ import annotations

import bisect

import numpy as np


def complete_parents(dam, sire):
    n = len(dam)
    d = np.array(dam, dtype=np.int64)
    s = np.array(sire, dtype=np.int64)
    d[(d < 0) | (d >= n)] = -1
    s[(s < 0) | (s >= n)] = -1
    return d, s


def ml(dam, sire):
    """Return (F, dii) restating genmatrix::ml."""
    n = len(dam)
    f = np.zeros(n)
    dii = np.ones(n)
    L = {}
    pending = []  # sorted list of indices with L > 0
    for i in range(n):
        s, d = int(sire[i]), int(dam[i])
        s_ok, d_ok = 0 <= s < n, 0 <= d < n
        Fs = f[s] if s_ok else 0.0
        Fd = f[d] if d_ok else 0.0
        if s_ok and d_ok:
            dii[i] = 1.0 - 0.25 * (1.0 + Fs) - 0.25 * (1.0 + Fd)
        elif s_ok:
            dii[i] = 1.0 - 0.25 * (1.0 + Fs)
        elif d_ok:
            dii[i] = 1.0 - 0.25 * (1.0 + Fd)
        else:
            dii[i] = 1.0
        if s_ok and d_ok:
            for par in (s, d):
                if L.get(par, 0.0) <= 0.0:
                    bisect.insort(pending, par)
                L[par] = L.get(par, 0.0) + 0.5
            F_calc = 0.0
            j_hi = max(s, d)
            while True:
                k = bisect.bisect_right(pending, j_hi)
                if k == 0:
                    break
                j = pending.pop(k - 1)
                j_hi = j - 1
                lj = L.get(j, 0.0)
                if lj > 0.0:
                    F_calc += lj * lj * dii[j]
                    sj, dj = int(sire[j]), int(dam[j])
                    for par in (sj, dj):
                        if 0 <= par < n:
                            if L.get(par, 0.0) <= 0.0 and 0.5 * lj > 0.0:
                                bisect.insort(pending, par)
                            L[par] = L.get(par, 0.0) + 0.5 * lj
                    L[j] = 0.0
            f[i] = F_calc + dii[i] - 1.0
            if f[i] < 0.0:
                f[i] = 0.0
        else:
            f[i] = 0.0
    return f, dii


def ainv_henderson(dam, sire):
    """A^-1 as a dense-free dict of (r, c) -> value, then CSR arrays (ptr, col, val)."""
    d, s = complete_parents(dam, sire)
    n = len(d)
    F, dii = ml(d, s)
    ent = {}

    def add(r, c, v):
        ent[(r, c)] = ent.get((r, c), 0.0) + v

    for i in range(n):
        di, si = int(d[i]), int(s[i])
        dinv = 1.0 / dii[i]
        add(i, i, dinv)
        if si >= 0:
            add(i, si, -0.5 * dinv)
            add(si, i, -0.5 * dinv)
            add(si, si, 0.25 * dinv)
        if di >= 0:
            add(i, di, -0.5 * dinv)
            add(di, i, -0.5 * dinv)
            add(di, di, 0.25 * dinv)
        if si >= 0 and di >= 0:
            add(si, di, 0.25 * dinv)
            add(di, si, 0.25 * dinv)
    for i in range(n):
        v = ent.get((i, i))
        if v is None or v < 1e-15:
            ent[(i, i)] = 1e-12
    keys = sorted(ent)
    ptr = np.zeros(n + 1, dtype=np.int64)
    col = np.empty(len(keys), dtype=np.int32)
    val = np.empty(len(keys))
    for k, (r, c) in enumerate(keys):
        ptr[r + 1] += 1
        col[k] = c
        val[k] = ent[(r, c)]
    np.cumsum(ptr, out=ptr)
    keep = np.abs(val) > 1e-24  # Eigen prune(1e-12) with dummy precision 1e-12
    if not keep.all():
        rows = np.repeat(np.arange(n), np.diff(ptr))[keep]
        col, val = col[keep], val[keep]
        ptr = np.zeros(n + 1, dtype=np.int64)
        np.add.at(ptr, rows + 1, 1)
        np.cumsum(ptr, out=ptr)
    return ptr, col, val, F, dii


def csr_to_dense(ptr, col, val, n):
    M = np.zeros((n, n))
    for i in range(n):
        M[i, col[ptr[i]:ptr[i + 1]]] = val[ptr[i]:ptr[i + 1]]
    return M


def a_columns(dam, sire, dii, cols):
    """A[:, cols] by the pedigree recursion A = T D T^T with T = (I - P)^-1."""
    d, s = complete_parents(dam, sire)
    n = len(d)
    Y = np.zeros((n, len(cols)))
    Y[np.asarray(cols), np.arange(len(cols))] = 1.0
    for i in range(n - 1, -1, -1):  # (I - P)^T y = x, children before parents
        if s[i] >= 0:
            Y[s[i]] += 0.5 * Y[i]
        if d[i] >= 0:
            Y[d[i]] += 0.5 * Y[i]
    Y *= dii[:, None]
    for i in range(n):  # (I - P) z = y, parents before children
        if s[i] >= 0:
            Y[i] += 0.5 * Y[s[i]]
        if d[i] >= 0:
            Y[i] += 0.5 * Y[d[i]]
    return Y


def tune_g(G, A22):
    """tuneG alignment (relationship_builder.cpp:539-565)."""
    n = G.shape[0]
    sgd, sad = np.trace(G), np.trace(A22)
    sgo, sao = G.sum() - sgd, A22.sum() - sad
    mgd, mad = sgd / n, sad / n
    noff = float(n) * (n - 1)
    mgo = sgo / noff if noff > 0 else 0.0
    mao = sao / noff if noff > 0 else 0.0
    b = 1.0
    if abs(mgd - mgo) > 1e-12:
        b = (mad - mao) / (mgd - mgo)
    a = mad - b * mgd
    return b * G + a, a, b
