"""Multi-trait GBLUP host API mirroring the reference's MvEigenVce and
GSSolve::solveMultiTrait.

Reference interfaces mirrored: ``MvEigenVce::Options`` / ``prepare`` /
``runNullModel`` / ``getVg`` / ``getVe`` (src/core/eigen_vce.h,
src/core/eigen_vce.cpp:106-266) with the settings GSVce uses
(src/variance/variance_estimator.cpp:289-298), and
``GSSolve::solveMultiTrait`` (src/solve/mixed_model_solver.cpp:425-524).
Both run in libcbx (``cbx_mt_vce`` / ``cbx_mt_solve``).  Matrices are numpy
arrays: Y (n x t complete cases), X (n x p dense fixed-effect design),
G / Ginv (n x n) or None for the handle's device G^-1 (cbx_invert_psd).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import Handle, lib, ptr


def _cm(a):
    """Column-major copy of a 2-D array, as a C-contiguous buffer (its transpose)."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)


@dataclass
class MvOptions:
    max_iter: int = 500        # max(500, 25 * vce_max_iter) with the default vce_max_iter = 20
    tol: float = 1e-4          # vce_tol
    use_projection: bool = True


class MvEigenVce:
    """Exact multi-trait LMM by eigen-EM (projection onto the null space of X')."""

    def __init__(self, handle: Handle, options: MvOptions | None = None):
        self.h = handle
        self.options = options or MvOptions()
        self.Vg = self.Ve = None
        self.iterations = 0
        self.converged = False
        self._args = None

    def prepare(self, Y, X, G=None) -> None:
        if not self.options.use_projection:
            raise ValueError("only the projected form (the reference's GSVce setting) is provided")
        Y = np.asarray(Y, dtype=np.float64)
        has_x = X is not None and np.asarray(X).size > 0
        self._dims = (Y.shape[0], Y.shape[1], np.asarray(X).shape[1] if has_x else 0)
        self._args = (_cm(Y), _cm(X) if has_x else None, None if G is None else _cm(G))

    def runNullModel(self) -> bool:
        Y, X, G = self._args
        n, t, p = self._dims
        Vg, Ve = np.zeros((t, t)), np.zeros((t, t))
        it, conv = C.c_int32(0), C.c_int32(0)
        self.h.check(lib().cbx_mt_vce(self.h.raw, n, t, p, ptr(Y), ptr(X) if X is not None else None,
                                      ptr(G) if G is not None else None, int(self.options.max_iter),
                                      float(self.options.tol), ptr(Vg), ptr(Ve), C.byref(it), C.byref(conv)))
        self.Vg, self.Ve = Vg, Ve
        self.iterations, self.converged = it.value, bool(conv.value)
        return self.converged

    def getVg(self) -> np.ndarray:
        return self.Vg

    def getVe(self) -> np.ndarray:
        return self.Ve


def solve_multi_trait(handle: Handle, Y, X, Vg, Ve, Ginv=None) -> dict:
    """Multi-trait MME solve; beta (p x t) and u (n x t), trait-major as the reference."""
    Y = np.asarray(Y, dtype=np.float64)
    n, t = Y.shape
    has_x = X is not None and np.asarray(X).size > 0
    p = np.asarray(X).shape[1] if has_x else 0
    Y = _cm(Y)
    X = _cm(X) if has_x else None
    beta = np.zeros(max(1, p * t))
    u = np.zeros(n * t)
    # keep every buffer referenced until the call returns
    Gi = _cm(Ginv) if Ginv is not None else None
    vg, ve = _cm(Vg), _cm(Ve)
    handle.check(lib().cbx_mt_solve(handle.raw, n, t, p, ptr(Y), ptr(X) if X is not None else None,
                                    ptr(Gi), ptr(vg), ptr(ve), ptr(beta), ptr(u)))
    return {"beta": beta[:p * t], "u": u, "beta_mat": beta[:p * t].reshape(t, p).T if p else np.zeros((0, t)),
            "u_mat": u.reshape(t, n).T}
