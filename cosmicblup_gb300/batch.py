"""Batched independent GBLUP problems (``cbx_batch_reml``).

Each problem is one reference run -- ``GrmBuilder::compute`` (src/core/
grm_builder.cpp:63-405), ``invert_psd_matrix`` (src/core/matrix_io.cpp:488-501)
and ``AI_REML::solve`` (src/core/vce.cpp:741-837) -- and the batch shares one
GPU through worker handles whose streams overlap.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import CbxError, lib
from .mme import rows_to_csr
from .vce import RemlConfig


class _Problem(C.Structure):
    _fields_ = [("bed", C.c_void_p), ("bed_bytes", C.c_int64), ("n", C.c_int64), ("m", C.c_int64),
                ("n_rec", C.c_int64), ("p", C.c_int64), ("y", C.c_void_p), ("aid", C.c_void_p),
                ("fx_ptr", C.c_void_p), ("fx_col", C.c_void_p), ("fx_val", C.c_void_p),
                ("var_u", C.c_double), ("var_e", C.c_double)]


class _Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("converged", C.c_int32),
                ("var_u", C.c_double), ("var_e", C.c_double), ("pcg_iters", C.c_int64),
                ("seconds", C.c_double), ("solution", C.c_void_p)]


@dataclass
class BatchProblem:
    """One GBLUP problem: BED bytes (with header) for n animals x m SNPs, one
    record list (y, 1-based aid), the fixed-effect design with p columns as a
    CSR triple (ptr, col, val) or as FixedDesignG rows, and starting variances."""
    bed: bytes
    n: int
    m: int
    y: np.ndarray
    aid: np.ndarray
    rows: tuple
    p: int
    var_u: float = 0.5
    var_e: float = 0.5


@dataclass
class BatchResult:
    status: int
    iterations: int
    converged: bool
    var_u: float
    var_e: float
    pcg_iters: int
    seconds: float
    solution: np.ndarray


def batch_reml(problems: list[BatchProblem], cfg: RemlConfig | None = None, device: int = 0,
               workers: int = 8, min_maf: float = 0.01, check: bool = True) -> list[BatchResult]:
    cfg = cfg or RemlConfig.default()
    keep = []
    arr = (_Problem * len(problems))()
    res = (_Result * len(problems))()
    sols = []
    for i, pb in enumerate(problems):
        bed = np.frombuffer(pb.bed, dtype=np.uint8)
        y = np.ascontiguousarray(pb.y, dtype=np.float64)
        aid = np.ascontiguousarray(pb.aid, dtype=np.int32)
        # the design as a CSR triple, or as FixedDesignG rows (per-record (col, val) lists)
        fp, fc, fv = pb.rows if isinstance(pb.rows, tuple) else rows_to_csr(pb.rows)
        fp = np.ascontiguousarray(fp, dtype=np.int64)
        fc = np.ascontiguousarray(fc, dtype=np.int32)
        fv = np.ascontiguousarray(fv, dtype=np.float64)
        if fp.size != y.size + 1 or fp[0] != 0 or fc.size != fp[-1] or fv.size != fp[-1] or aid.size != y.size:
            raise ValueError(f"problem {i}: inconsistent record / design arrays")
        sol = np.zeros(pb.p + pb.n)
        keep += [bed, y, aid, fp, fc, fv]
        sols.append(sol)
        arr[i] = _Problem(bed.ctypes.data, bed.size, pb.n, pb.m, y.size, pb.p, y.ctypes.data, aid.ctypes.data,
                          fp.ctypes.data, fc.ctypes.data, fv.ctypes.data, pb.var_u, pb.var_e)
        res[i].solution = sol.ctypes.data
    rc = lib().cbx_batch_reml(device, len(problems), C.cast(arr, C.c_void_p), C.c_float(min_maf),
                              C.cast(C.pointer(cfg), C.c_void_p), workers, C.cast(res, C.c_void_p))
    out = [BatchResult(r.status, r.iterations, bool(r.converged), r.var_u, r.var_e, r.pcg_iters, r.seconds,
                       sols[i]) for i, r in enumerate(res)]
    if check and rc != 0:
        raise CbxError(rc, f"batch problem failed with status {rc}")
    return out
