"""Text result files, mirroring GSOutput::writeResults
(src/solve/result_writer.cpp:64-430) for one genetic component: ``.vars``,
``.beta`` and ``.rand`` (the C ABI's cbx_write_vars / cbx_write_beta /
cbx_write_rand; host formatting only, no GPU)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import CbxError, lib, ptr
from .mme import rows_to_csr


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise CbxError(rc, what)


def _cstrings(items):
    arr = (C.c_char_p * len(items))(*[s.encode() for s in items])
    return arr


def write_vars(prefix: str, var_u: float, se_u: float, var_e: float, se_e: float, tag: str = "GA") -> str:
    path = prefix + ".vars"
    _check(lib().cbx_write_vars(path.encode(), tag.encode(), float(var_u), float(se_u), float(var_e),
                                float(se_e)), path)
    return path


def write_beta(prefix: str, names, beta, beta_se=None) -> str:
    path = prefix + ".beta"
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    se = None if beta_se is None else np.ascontiguousarray(beta_se, dtype=np.float64)
    nm = _cstrings(list(names))
    _check(lib().cbx_write_beta(path.encode(), beta.size, C.cast(nm, C.c_void_p), ptr(beta), ptr(se)), path)
    return path


def write_rand(prefix: str, y, aid, rows, p: int, beta, u, ids=None, tag: str = "GA") -> str:
    """rows: FixedDesignG rows (list of (col, val) lists) or an (fx_ptr, fx_col, fx_val) tuple."""
    path = prefix + ".rand"
    y = np.ascontiguousarray(y, dtype=np.float64)
    aid = np.ascontiguousarray(aid, dtype=np.int32)
    fp, fc, fv = rows if isinstance(rows, tuple) else rows_to_csr(rows)
    fp = np.ascontiguousarray(fp, dtype=np.int64)
    fc = np.ascontiguousarray(fc, dtype=np.int32)
    fv = np.ascontiguousarray(fv, dtype=np.float64)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    idarr = None if ids is None else _cstrings(list(ids))
    _check(lib().cbx_write_rand(path.encode(), tag.encode(), y.size, ptr(y), ptr(aid), ptr(fp), ptr(fc), ptr(fv),
                                int(p), ptr(beta), u.size, ptr(u),
                                None if idarr is None else C.cast(idarr, C.c_void_p)), path)
    return path
