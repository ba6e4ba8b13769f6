"""CPU tests pinning the oracle's probe stream and adaptive trace schedule to the
reference's own code: oracle/_ref/libref_trace.so is compiled from the reference
tree's src/core/rng.h and src/core/adaptive_trace_estimator.cpp (recipe in
oracle/ref_trace, built by oracle/build.py where the reference checkout exists).
Skipped where that library was not built."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import build as ob
from oracle.rng import adaptive_trace, rademacher


def ref_lib():
    if not os.path.exists(ob.REF_LIB):
        try:
            ob.build()
        except Exception:
            pass
    if not os.path.exists(ob.REF_LIB):
        pytest.skip("the reference's rng / trace estimator is not built here")
    try:
        L = C.CDLL(ob.REF_LIB)
    except OSError:
        pytest.skip("the reference's rng / trace estimator library does not load here")
    L.ref_rademacher.argtypes = [C.c_ulong, C.c_int, C.c_void_p]
    L.ref_trace_estimate.restype = C.c_double
    return L


CB = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int)


@pytest.mark.parametrize("seed", [0, 42, 58, 74, 12345, 2**40 + 7])
@pytest.mark.parametrize("n", [1, 7, 1000])
def test_rademacher_bit_exact(seed, n):
    L = ref_lib()
    ref = np.empty(n)
    L.ref_rademacher(seed, n, ref.ctypes.data)
    assert np.array_equal(rademacher(seed, n, 1)[0], ref)


@pytest.mark.parametrize("dim,tol", [(40, 0.05), (200, 0.02), (25, 1e-6)])
def test_adaptive_trace_matches_reference(dim, tol):
    L = ref_lib()
    rng = np.random.default_rng(dim)
    B = rng.standard_normal((dim, dim))
    A = B @ B.T / dim + np.eye(dim)

    def op(z_ptr, out_ptr, d):
        z = np.ctypeslib.as_array(z_ptr, shape=(d,))
        out = np.ctypeslib.as_array(out_ptr, shape=(d,))
        out[:] = A @ z

    cb = CB(op)
    ref = L.ref_trace_estimate(dim, cb, 30, 100, C.c_double(tol), 42)
    got, samples, _ = adaptive_trace(dim, lambda z: A @ z, 30, 100, tol, 42)
    assert 30 <= samples <= 100
    assert abs(got - ref) <= 1e-12 * abs(ref)
