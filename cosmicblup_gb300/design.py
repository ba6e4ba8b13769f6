"""Fixed-effect design for the MME, as ``buildFixedDesignGeneric`` builds it
(src/core/design.cpp:13-109): column 0 is mu; every categorical factor adds
one column per level except its first (base) level, levels ordered as
std::set<std::string> orders them (byte-wise); numeric covariates follow.
Empty strings are "no level" for that factor.

``fixed_design`` returns the rows directly as CSR arrays (the form
``cbx_mme_create`` takes), built with numpy array operations.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class FixedDesign:
    p: int
    ptr: np.ndarray          # int64, n + 1
    col: np.ndarray          # int32
    val: np.ndarray          # float64
    names: list = field(default_factory=list)

    def csr(self) -> tuple:
        return self.ptr, self.col, self.val

    def dense(self) -> np.ndarray:
        n = self.ptr.size - 1
        X = np.zeros((n, self.p))
        rows = np.repeat(np.arange(n), np.diff(self.ptr))
        X[rows, self.col] = self.val
        return X


def fixed_design(cats, nums=None, cat_names=None, num_names=None) -> FixedDesign:
    n = len(cats)
    ncat = len(cats[0]) if n else 0
    names = ["mu"]
    p = 1
    entries = [np.zeros(n, dtype=np.int64)]          # column 0 = mu for every record
    vals = [np.ones(n)]
    for j in range(ncat):
        keys = np.array([c[j].encode() for c in cats], dtype=object)
        present = np.array([len(k) > 0 for k in keys])
        lv = sorted(set(keys[present]))
        if not lv:
            continue
        prefix = cat_names[j] if cat_names and j < len(cat_names) else f"factor{j + 1}"
        index = {k: i for i, k in enumerate(lv)}
        code = np.array([index.get(k, -1) for k in keys], dtype=np.int64)
        for k in lv[1:]:
            names.append(f"{prefix}_{k.decode()}")
        hit = code >= 1                                  # base level (0) and missing add nothing
        col = np.where(hit, p + code - 1, -1)
        entries.append(col)
        vals.append(np.where(hit, 1.0, 0.0))
        p += len(lv) - 1
    if nums is not None and n:
        N = np.asarray(nums, dtype=np.float64).reshape(n, -1)
        for j in range(N.shape[1]):
            names.append(num_names[j] if num_names and j < len(num_names) else f"cov{j + 1}")
            entries.append(np.full(n, p, dtype=np.int64))
            vals.append(N[:, j].copy())
            p += 1
    E = np.stack(entries, axis=1) if entries else np.zeros((n, 0), dtype=np.int64)
    V = np.stack(vals, axis=1) if vals else np.zeros((n, 0))
    keep = E >= 0
    counts = keep.sum(axis=1)
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=ptr[1:])
    return FixedDesign(p=p, ptr=ptr, col=E[keep].astype(np.int32), val=V[keep], names=names)
