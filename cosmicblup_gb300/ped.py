"""Pedigree / ssGBLUP host API mirroring the reference's relationship builder.

Reference interfaces mirrored: ``genmatrix::invertA_henderson(dam, sire)``
(src/core/a_matrix.cpp:392-439) and the ssGBLUP branch of
``MatrixBuilder::build`` (src/io/relationship_builder.cpp:481-633), which
produces the SplitMatrixAdapter H^-1 = A^-1 + S (tau Gb^-1 - omega A22^-1) S^T.
Parent arrays are 0-based indices with -1 for an unknown parent; animals are
listed parents first.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Handle, lib, ptr
from .mme import DeviceMME


def ainv_henderson(handle: Handle, dam, sire, with_inbreeding: bool = False):
    """Return (ptr, col, val[, F, dii]) of A^-1 in CSR form."""
    dam = np.ascontiguousarray(dam, dtype=np.int64)
    sire = np.ascontiguousarray(sire, dtype=np.int64)
    n = dam.size
    nnz = C.c_int64(0)
    handle.check(lib().cbx_ainv_henderson(handle.raw, n, ptr(dam), ptr(sire), C.byref(nnz), None, None,
                                          None, None, None))
    p_ = np.empty(n + 1, dtype=np.int64)
    c_ = np.empty(nnz.value, dtype=np.int32)
    v_ = np.empty(nnz.value, dtype=np.float64)
    F = np.empty(n)
    d = np.empty(n)
    handle.check(lib().cbx_ainv_henderson(handle.raw, n, ptr(dam), ptr(sire), C.byref(nnz), ptr(p_), ptr(c_),
                                          ptr(v_), ptr(F), ptr(d)))
    return (p_, c_, v_, F, d) if with_inbreeding else (p_, c_, v_)


def ssgblup_qinv(mme: DeviceMME, dam, sire, gmap, G=None, alpha=0.05, tune_g=True, tau=1.0,
                 omega=1.0, ridge=0.0, return_blocks=False):
    """Install H^-1 as the Qinv of ``mme`` (q = pedigree size).  G None = device GRM."""
    dam = np.ascontiguousarray(dam, dtype=np.int64)
    sire = np.ascontiguousarray(sire, dtype=np.int64)
    gmap = np.ascontiguousarray(gmap, dtype=np.int32)
    ng = gmap.size
    Gc = None if G is None else np.ascontiguousarray(G, dtype=np.float64)
    A22 = np.empty((ng, ng)) if return_blocks else None
    Gd = np.empty((ng, ng)) if return_blocks else None
    mme.h.check(lib().cbx_ssgblup_qinv(mme.h.raw, dam.size, ptr(dam), ptr(sire), ng, ptr(gmap), ptr(Gc),
                                       float(alpha), 1 if tune_g else 0, float(tau), float(omega),
                                       float(ridge), ptr(A22), ptr(Gd)))
    return (A22, Gd) if return_blocks else None
