"""Oracle: Rademacher probe vectors of the reference (test infrastructure).

Restates src/core/rng.h:19-53 and the probe schedule of
AdaptiveTraceEstimator::estimate (src/core/adaptive_trace_estimator.cpp:11-81)
for one OpenMP thread: probes come in batches of 16; the batch that starts
after ``done`` samples uses a fresh engine seeded ``seed + done`` and draws its
probes consecutively.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB):
            _build.build()
        L = C.CDLL(_build.LIB)
        L.oracle_rademacher.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_void_p]
        L.oracle_mt64_raw.argtypes = [C.c_uint64, C.c_int64, C.c_void_p]
        _lib = L
    return _lib


def rademacher(seed: int, n: int, count: int = 1) -> np.ndarray:
    """(count, n) probes drawn consecutively from mt19937_64(seed)."""
    out = np.empty((count, n), dtype=np.float64)
    lib().oracle_rademacher(seed, n, count, out.ctypes.data)
    return out


def mt64_raw(seed: int, count: int) -> np.ndarray:
    out = np.empty(count, dtype=np.uint64)
    lib().oracle_mt64_raw(seed, count, out.ctypes.data)
    return out


def probe_batches(dim: int, min_samples: int, max_samples: int, seed: int = 42,
                  threads: int = 1):
    """Yield (done, probes) per batch in the reference's order (threads = 1)."""
    if threads != 1:
        raise NotImplementedError("only the single-thread probe schedule is restated")
    batch = max(16, 4 * threads)
    done = 0
    while done < max_samples:
        cur = min(batch, max_samples - done)
        yield done, rademacher(seed + done, dim, cur)
        done += cur


def adaptive_trace(dim: int, op, min_samples: int = 30, max_samples: int = 300,
                   tol: float = 0.05, seed: int = 42) -> tuple[float, int, list]:
    """Restatement of AdaptiveTraceEstimator::estimate (one thread).

    ``op`` maps a probe z (dim,) to A z.  Returns (trace, samples, values)."""
    if dim <= 0:
        return 0.0, 0, []
    if min_samples <= 0:
        min_samples = 10
    if max_samples < min_samples:
        max_samples = min_samples
    tsum = tsq = 0.0
    done = 0
    vals = []
    for start, probes in probe_batches(dim, min_samples, max_samples, seed):
        bs = bq = 0.0
        for z in probes:
            v = float(z @ op(z))
            vals.append(v)
            bs += v
            bq += v * v
        tsum += bs
        tsq += bq
        done += len(probes)
        if done >= min_samples:
            mean = tsum / done
            var = (tsq - tsum * tsum / done) / (done - 1.0)
            se = np.sqrt(max(0.0, var) / done)
            if abs(mean) > 1e-12 and se / abs(mean) < tol:
                break
    return tsum / done, done, vals
