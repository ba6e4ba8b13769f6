"""The fixed-point tensor-core refinement product (dense_fx.cu) against exact dot
products: each row of the block and each column of the vectors cut into six
balanced 8-bit digits, digit products summed exactly on tcgen05 (kind::f16) in
128-element chunks and flushed into int64 totals."""
import ctypes as C
import math

import numpy as np
import pytest

from cosmicblup_gb300._lib import lib, ptr

pytestmark = pytest.mark.gpu


def fx(handle, Q, V, reps=0):
    """Y = Q[:, :ng] V[:, :ng]^T: the product runs over k < ng (the genotyped
    rows); the block's columns ng .. ld are its zero row padding."""
    ng, ld = Q.shape
    S = V.shape[0]
    Y = np.zeros((ng, S))
    ms = C.c_double(0)
    handle.check(lib().cbx_selftest_dense_fx(handle.raw, ptr(np.ascontiguousarray(Q)), ng, ld,
                                             ptr(np.ascontiguousarray(V)), S, reps, ptr(Y), C.byref(ms)))
    return Y, ms.value


def xdot(a, b):
    """Exact dot product of two FP64 vectors (math.fsum over exactly split products)."""
    ah = a.astype(np.float32).astype(np.float64)
    bh = b.astype(np.float32).astype(np.float64)
    parts = [ah * bh, ah * (b - bh), (a - ah) * bh, (a - ah) * (b - bh)]
    return math.fsum(np.concatenate(parts))


def planes(Q):
    """The block as the product sees it: FP32 hi + lo (about 48 bits)."""
    hi = Q.astype(np.float32).astype(np.float64)
    lo = (Q - hi).astype(np.float32).astype(np.float64)
    return hi + lo


@pytest.mark.parametrize("S", [32, 16, 20, 1])
def test_fx_product_on_an_offset_block(handle, S):
    """A block with a large common offset against centred vectors (the
    cancellation of an eigen-bent G^-1): error below 2^-42 of sum |Q||V|."""
    rng = np.random.default_rng(300 + S)
    ng, ld = 2001, 2004
    Q = np.zeros((ng, ld))
    Q[:, :ng] = rng.standard_normal((ng, ng)) + 150.0
    V = np.zeros((S, ld))
    V[:, :ng] = rng.standard_normal((S, ng))
    V[:, :ng] -= V[:, :ng].mean(axis=1, keepdims=True)
    Y, _ = fx(handle, Q, V)
    Qp = planes(Q)
    scale = np.abs(Q) @ np.abs(V).T
    for i in list(range(0, ng, 37)) + [ng - 1]:
        for c in range(S):
            err = abs(Y[i, c] - xdot(Qp[i], V[c])) / scale[i, c]
            assert err < 2.0 ** -42, (i, c, err)


def test_fx_product_fixed_point_bound(handle):
    """Entries spanning e^-6 .. e^6 within each row, ragged rows and K tail: the
    error stays within the fixed-point bound 2^-42 (max_k |q_ik| sum_k |v_kc| +
    max_k |v_kc| sum_k |q_ik|), and the zero columns of a partial piece are 0."""
    rng = np.random.default_rng(310)
    ng, ld, S = 1003, 1004, 24
    Q = np.zeros((ng, ld))
    Q[:, :ng] = rng.standard_normal((ng, ng)) * np.exp(rng.uniform(-6, 6, (ng, ng)))
    Q[5] = 0.0                                          # an all-zero row
    V = np.zeros((S, ld))
    V[:, :ng] = rng.standard_normal((S, ng)) * np.exp(rng.uniform(-3, 3, (S, 1)))
    V[3] = 0.0                                          # an all-zero column
    Y, _ = fx(handle, Q, V)
    Qp = planes(Q)
    aQ, aV = np.abs(Qp), np.abs(V)
    bound = 2.0 ** -42 * (aQ.max(axis=1)[:, None] * aV.sum(axis=1)[None, :]
                          + aV.max(axis=1)[None, :] * aQ.sum(axis=1)[:, None])
    assert np.all(Y[5] == 0.0) and np.all(Y[:, 3] == 0.0)
    for i in list(range(0, ng, 53)) + [ng - 1]:
        for c in range(S):
            err = abs(Y[i, c] - xdot(Qp[i], V[c]))
            assert err <= bound[i, c] + 1e-300, (i, c, err, bound[i, c])


def test_fx_agrees_with_the_float_float_product(handle):
    """Both FP64-accurate products agree to ~2^-40 of sum |Q||V| on a G^-1-like
    symmetric block."""
    rng = np.random.default_rng(320)
    ng = ld = 1024
    Z = rng.standard_normal((ng, 3 * ng)) / np.sqrt(3 * ng)
    G = Z @ Z.T + 0.05 * np.eye(ng)
    Q = np.linalg.inv(G)
    V = rng.standard_normal((32, ld))
    Yf, _ = fx(handle, Q, V)
    Yff = np.zeros((ng, 32))
    ms = C.c_double(0)
    handle.check(lib().cbx_selftest_dense_ff(handle.raw, ptr(Q), ng, ld, ptr(V), 32, 1, 0, ptr(Yff), C.byref(ms)))
    scale = np.abs(Q) @ np.abs(V).T
    assert (np.abs(Yf - Yff) / scale).max() < 2.0 ** -40


def test_fx_product_timing(handle):
    """Times the product at block order 8,192 (32 columns) beside the float-float
    kernel, for the record."""
    rng = np.random.default_rng(330)
    ng = ld = 8192
    Q = rng.standard_normal((ng, ld))
    V = rng.standard_normal((32, ld))
    Y, ms = fx(handle, Q, V, reps=5)
    Yff = np.zeros((ng, 32))
    ms_ff = C.c_double(0)
    handle.check(lib().cbx_selftest_dense_ff(handle.raw, ptr(Q), ng, ld, ptr(V), 32, 1, 3, ptr(Yff),
                                             C.byref(ms_ff)))
    scale = np.abs(Q) @ np.abs(V).T
    assert (np.abs(Y - Yff) / scale).max() < 2.0 ** -40
    print(f"n=8192, 32 columns: fixed-point tensor product {ms:.3f} ms, float-float {ms_ff.value:.3f} ms")
