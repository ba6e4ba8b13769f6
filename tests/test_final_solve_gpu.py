"""GPU tests of the final MME solve with fixed-effect standard errors
(cbx_final_solve, the reference's GSSolve::solve): direct Cholesky and both
PCG forms against the oracle's dense solve and inverse."""
import numpy as np
import pytest

from cosmicblup_gb300 import DeviceMME
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from cosmicblup_gb300.vce import final_solve
from oracle.grm import vanraden_grm
from oracle.mme import MME, build_fixed_design, invert_psd_matrix

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob():
    n, m = 300, 1200
    bed, _ = simulate_bed(n, m, seed=600, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, n, m)["G"]
    Gi = invert_psd_matrix(G)
    g = genetic_values(bed, n, m, seed=601, var_a=0.4)
    rec = simulate_gblup_records(n, 3, g, seed=602, var_e=0.6)
    p, rows, _ = build_fixed_design(rec["cats"])
    return {"n": n, "Gi": Gi, "rec": rec, "p": p, "rows": rows, "mme": MME(rec["y"], rec["aid"], rows, p, n)}


def oracle_final(d, vu, ve):
    om = d["mme"]
    A = om.lhs(d["Gi"], ve / vu)
    sol = np.linalg.solve(A, om.rhs())
    Ci = np.linalg.inv(A)[:d["p"], :d["p"]]
    return sol, np.sqrt(np.maximum(0.0, ve * np.diag(Ci))), Ci


@pytest.mark.parametrize("solver,tol", [(0, 0.0), (1, 1e-11), (2, 1e-10)])
def test_final_solve_and_se(handle, prob, solver, tol):
    dm = DeviceMME(handle, prob["rec"]["y"], prob["rec"]["aid"], prob["rows"], prob["p"], prob["n"])
    dm.set_qinv_dense(prob["Gi"])
    vu, ve = 0.4, 0.6
    res = final_solve(dm, vu, ve, solver=solver, tol=tol if tol else 1e-10)
    sol, se, Ci = oracle_final(prob, vu, ve)
    rt = 1e-10 if solver == 0 else 1e-6
    np.testing.assert_allclose(res["sol"], sol, rtol=rt, atol=rt * np.abs(sol).max())
    np.testing.assert_allclose(res["beta_se"], se, rtol=rt)
    np.testing.assert_allclose(res["Cinv_beta"], Ci, rtol=rt, atol=rt * np.abs(Ci).max())


def test_final_solve_without_se(handle, prob):
    dm = DeviceMME(handle, prob["rec"]["y"], prob["rec"]["aid"], prob["rows"], prob["p"], prob["n"])
    dm.set_qinv_dense(prob["Gi"])
    res = final_solve(dm, 0.4, 0.6, solver=0, calc_se=False)
    sol, _, _ = oracle_final(prob, 0.4, 0.6)
    np.testing.assert_allclose(res["sol"], sol, rtol=1e-10, atol=1e-10 * np.abs(sol).max())
    assert not res["beta_se"].any()
