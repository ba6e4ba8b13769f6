"""GPU tests of the failure paths, each made without faulting or hanging the GPU.

* A bounded device-side wait that runs out: the self-test kernel waits on an
  mbarrier that nothing arrives at, with a 10 ms limit; the call returns
  CBX_ERR_TIMEOUT (as every bounded wait of the library reports a timeout) and
  the handle keeps working.
* The iteration limit: PCGSolver::solve (src/core/pcg_solver.h:530-534) returns
  its last iterate and reports max_iter iterations and the true relative
  residual, raising nothing; so does cbx_pcg_solve (the FP64 iterate equals the
  oracle's after the same number of iterations).
* Breakdown and restart (src/core/pcg_solver.h:482-495): a zero right-hand
  side, and a right-hand side along a singular direction of the LHS (an animal
  without records, lambda = 0: p'Ap = 0 with r != 0), restart once from p = z,
  break down again and return the iterate with the true residual, as the
  oracle's restatement does; other columns of the same block are unaffected.
"""
import ctypes as C

import numpy as np
import pytest

from cosmicblup_gb300 import DeviceMME
from cosmicblup_gb300._lib import CBX_OK, lib
from cosmicblup_gb300.mme import FP64, MIXED
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from oracle.grm import vanraden_grm
from oracle.mme import MME, BlockJacobi, build_fixed_design, invert_psd_matrix, pcg

pytestmark = pytest.mark.gpu
CBX_ERR_TIMEOUT = 4


@pytest.fixture(scope="module")
def prob():
    n, m = 200, 1500
    bed, _ = simulate_bed(n, m, seed=900, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, n, m)["G"]
    Gi = invert_psd_matrix(G)
    # a well-conditioned Qinv for comparing iterates after a few iterations: with
    # the eigen-bent G^-1 (condition ~1e10) the iterates of two FP64 CG runs that
    # round differently part after a handful of iterations
    Qwc = np.linalg.inv(0.8 * G + 0.2 * np.eye(n))
    g = genetic_values(bed, n, m, seed=901, var_a=0.4)
    rec = simulate_gblup_records(n, 3, g, seed=902, var_e=0.6)
    p, rows, _ = build_fixed_design(rec["cats"])
    return {"n": n, "Gi": Gi, "Qwc": Qwc, "rec": rec, "p": p, "rows": rows}


def test_bounded_wait_times_out_and_handle_survives(handle, prob):
    ms = C.c_double(0)
    rc = lib().cbx_selftest_wait_timeout(handle.raw, 10_000_000, C.byref(ms))
    assert rc == CBX_ERR_TIMEOUT
    assert b"timed out" in lib().cbx_last_error(handle.raw)
    assert 9.0 <= ms.value < 1000.0
    # the context is still usable: a solve on the same handle matches the oracle
    d = prob
    dm = DeviceMME(handle, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    dm.set_qinv_dense(d["Gi"])
    om = MME(d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    x, _, rr = dm.pcg_solve(1.5, om.rhs())
    xe = np.linalg.solve(om.lhs(d["Gi"], 1.5), om.rhs())
    assert np.abs(x - xe).max() <= 1e-8 * np.abs(xe).max()
    # and a second timeout is reported the same way (the status word was reset)
    assert lib().cbx_selftest_wait_timeout(handle.raw, 1_000_000, C.byref(ms)) == CBX_ERR_TIMEOUT
    assert lib().cbx_sync(handle.raw) == CBX_OK


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_iteration_limit_returns_iterate_and_true_residual(handle, prob, precision):
    d = prob
    dm = DeviceMME(handle, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    dm.set_qinv_dense(d["Qwc"])
    om = MME(d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    A, b = om.lhs(d["Qwc"], 1.5), om.rhs()
    maxit = 8
    x, it, rr = dm.pcg_solve(1.5, b, maxit=maxit, precision=precision)  # raises on an error status
    true_rel = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    assert rr[0] > 1e-10 and abs(rr[0] - true_rel) <= 1e-6 * true_rel
    if precision == FP64:
        assert it[0] == maxit
        xo, ito, relo, _ = pcg(lambda v: A @ v, b, BlockJacobi(A, om.p), tol=1e-10, maxit=maxit)
        assert ito == maxit and abs(rr[0] - relo) <= 1e-6 * relo
        assert np.abs(x - xo).max() <= 1e-9 * np.abs(xo).max()
    else:
        assert it[0] <= maxit


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_breakdown_restart_returns_iterate(handle, prob, precision):
    d = prob
    n, p = d["n"], d["p"]
    k = 17  # this animal keeps no record: its row and column of W'W are zero
    keep = d["rec"]["aid"] != k + 1
    y, aid = d["rec"]["y"][keep], d["rec"]["aid"][keep]
    rows = [r for r, kp in zip(d["rows"], keep) if kp]
    dm = DeviceMME(handle, y, aid, rows, p, n)
    dm.set_qinv_dense(d["Gi"])
    om = MME(y, aid, rows, p, n)
    A = om.lhs(d["Gi"], 0.0)  # lambda = 0: the LHS is W'W, singular along e_(p+k)
    B = np.zeros((om.dim, 3))
    B[:, 0] = om.rhs()
    B[p + k, 1] = 1.0         # column 1: along the singular direction; column 2: zero
    maxit = 50
    X, it, rr = dm.pcg_solve(0.0, B, maxit=maxit, precision=precision)
    for c in (1, 2):
        xo, ito, relo, restarts = pcg(lambda v: A @ v, B[:, c], BlockJacobi(A, p), tol=1e-10, maxit=maxit)
        assert restarts == 1 and ito == maxit
        assert np.array_equal(X[:, c], xo) and np.all(xo == 0.0)
        assert rr[c] == relo  # 1 along the singular direction, 0 for b = 0
        if precision == FP64:
            assert it[c] == maxit
    # column 0 in the same block runs its own recurrence: it converges as a solve
    # alone does (same iterations; the block and single-column products sum in
    # different orders, and this LHS is singular, so the iterates are compared
    # through their true residuals)
    x0, it0, rr0 = dm.pcg_solve(0.0, B[:, 0], maxit=maxit, precision=precision)
    b0 = B[:, 0]
    assert it[0] == it0[0]
    for x in (X[:, 0], x0):
        assert np.linalg.norm(b0 - A @ x) <= 1e-9 * np.linalg.norm(b0)
