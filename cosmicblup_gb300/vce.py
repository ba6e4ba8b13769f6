"""AI-REML host API mirroring the reference's VCESolver / AI_REML.

Reference interfaces mirrored: ``VCEConfig`` (src/core/vce.h:140-165),
``VCESolver::solve`` / ``getVarE`` / ``getVarsU`` / ``getSolution`` /
``setInitialVars`` (src/core/vce.h:223-390), ``invert_psd_matrix``
(src/core/matrix_io.cpp:488-501).  The iteration runs in libcbx
(``cbx_reml_iterate`` / ``cbx_reml_solve``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Handle, lib, ptr
from .mme import DeviceMME


class RemlConfig(C.Structure):
    _fields_ = [("max_iter", C.c_int32), ("tol", C.c_double), ("mc_samples", C.c_int32),
                ("pcg_max_iter", C.c_int32), ("pcg_tol", C.c_double), ("precision", C.c_int32),
                ("mode", C.c_int32), ("seed", C.c_int32)]

    @classmethod
    def default(cls, **kw) -> "RemlConfig":
        c = cls()
        lib().cbx_reml_config_default(C.byref(c))
        for k, v in kw.items():
            setattr(c, k, v)
        return c


class RemlIterInfo(C.Structure):
    _fields_ = [("kind", C.c_int32), ("var_u", C.c_double), ("var_e", C.c_double),
                ("logL", C.c_double), ("trace", C.c_double), ("probes", C.c_int32),
                ("pcg_iters", C.c_int64), ("matvecs", C.c_int64), ("e_sse", C.c_double),
                ("uQu", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


MODE_AUTO, MODE_EM, MODE_DENSE, MODE_AI = 0, 1, 2, 3


class AIREML:
    """Single-component AI-REML on a DeviceMME."""

    def __init__(self, mme: DeviceMME, var_u: float = 1.0, var_e: float = 1.0,
                 config: RemlConfig | None = None):
        self.mme = mme
        self.config = config or RemlConfig.default()
        self.var_u, self.var_e = float(var_u), float(var_e)
        self.history: list[dict] = []
        self.iterations = 0
        self.converged = False
        self.solution = None

    def setInitialVars(self, var_e: float, vars_u) -> None:
        self.var_e = float(var_e)
        self.var_u = float(vars_u[0] if np.ndim(vars_u) else vars_u)

    def run_iteration(self, grad_probes: int = 0, solution: bool = False) -> dict:
        """One REML iteration.  grad_probes > 0 also returns the REML gradient at
        the iteration's starting point from that many probes (cbx_reml_iterate_grad:
        one block solve serves both) as d["grad"], d["grad_trace"], d["grad_pcg_iters"],
        and with solution=True the data solve as self.solution."""
        vu, ve = C.c_double(self.var_u), C.c_double(self.var_e)
        info = RemlIterInfo()
        if grad_probes > 0:
            g = np.zeros(2)
            tr, it = C.c_double(0), C.c_int64(0)
            sol = np.zeros(self.mme.dim) if solution else None
            self.mme.h.check(lib().cbx_reml_iterate_grad(self.mme.h.raw, C.byref(self.config), int(grad_probes),
                                                         C.byref(vu), C.byref(ve), C.byref(info), ptr(g),
                                                         C.byref(tr), C.byref(it), ptr(sol)))
            if solution:
                self.solution = sol
        else:
            self.mme.h.check(lib().cbx_reml_iterate(self.mme.h.raw, C.byref(self.config), C.byref(vu),
                                                    C.byref(ve), C.byref(info)))
        self.var_u, self.var_e = vu.value, ve.value
        d = info.as_dict()
        if grad_probes > 0:
            d.update(grad=g, grad_trace=tr.value, grad_pcg_iters=it.value)
        self.history.append(d)
        return d

    def solve(self) -> tuple[float, float]:
        vu, ve = C.c_double(self.var_u), C.c_double(self.var_e)
        it, conv = C.c_int32(0), C.c_int32(0)
        sol = np.zeros(self.mme.dim)
        hist = (RemlIterInfo * max(1, self.config.max_iter))()
        self.mme.h.check(lib().cbx_reml_solve(self.mme.h.raw, C.byref(self.config), C.byref(vu),
                                              C.byref(ve), C.byref(it), C.byref(conv), ptr(sol), hist))
        self.var_u, self.var_e = vu.value, ve.value
        self.iterations, self.converged = it.value, bool(conv.value)
        self.history = [hist[i].as_dict() for i in range(it.value)]
        self.solution = sol
        return self.var_u, self.var_e

    def getVarE(self) -> float:
        return self.var_e

    def getVarsU(self) -> list[float]:
        return [self.var_u]

    def getSolution(self) -> np.ndarray:
        return self.solution


def invert_psd(handle: Handle, M=None, n: int | None = None, ridge: float = 0.0,
               download: bool = True):
    """Eigen-bending inverse (device result kept on the handle); M None = device GRM."""
    if M is not None:
        M = np.ascontiguousarray(M, dtype=np.float64)
        n = M.shape[0]
    out = np.empty((n, n), dtype=np.float64) if download else None
    handle.check(lib().cbx_invert_psd(handle.raw, ptr(M), int(n), float(ridge), ptr(out)))
    return out


def reml_gradient(mme: DeviceMME, var_u: float, var_e: float, nprobe: int = 256, seed: int = 42,
                  exact: bool = False, precision: int = 0, pcg_tol: float = 1e-10,
                  pcg_maxit: int = 10000) -> dict:
    """d logL / d(var_u, var_e) (the reference's AI-REML score) -- cbx_reml_gradient."""
    g = np.zeros(2)
    tr = C.c_double(0)
    it = C.c_int64(0)
    mme.h.check(lib().cbx_reml_gradient(mme.h.raw, float(var_u), float(var_e), int(nprobe), int(seed),
                                        1 if exact else 0, int(precision), float(pcg_tol), int(pcg_maxit),
                                        ptr(g), C.byref(tr), C.byref(it)))
    return {"grad": g, "trace": tr.value, "pcg_iters": it.value}


def reml_logl_dense(mme: DeviceMME, var_u: float, var_e: float) -> float:
    out = C.c_double(0)
    mme.h.check(lib().cbx_reml_logl_dense(mme.h.raw, float(var_u), float(var_e), C.byref(out)))
    return out.value


def final_solve(mme: DeviceMME, var_u: float, var_e: float, solver: int = 0, tol: float = 1e-10,
                maxit: int = 10000, precision: int = 0, calc_se: bool = True) -> dict:
    """GSSolve::solve: BLUE / BLUP solution and fixed-effect SEs (cbx_final_solve)."""
    sol = np.zeros(mme.dim)
    se = np.zeros(mme.p)
    ci = np.zeros((mme.p, mme.p))
    mme.h.check(lib().cbx_final_solve(mme.h.raw, float(var_u), float(var_e), int(solver), float(tol), int(maxit),
                                      int(precision), 1 if calc_se else 0, ptr(sol), ptr(se), ptr(ci)))
    return {"beta": sol[:mme.p], "u": sol[mme.p:], "sol": sol, "beta_se": se, "Cinv_beta": ci}
