"""GPU parity tests of the REML path against the oracle restatement of AI_REML.

Bar: variance components within 1e-6 relative of the FP64
oracle; the Hutchinson probe count identical (same probe vectors, same adaptive
stop); the eigen-bending inverse within 1e-9 of the oracle's.
"""
import numpy as np
import pytest

from cosmicblup_gb300 import AIREML, DeviceMME, RemlConfig, invert_psd
from cosmicblup_gb300.mme import FP64, MIXED
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from cosmicblup_gb300.vce import MODE_DENSE, MODE_EM
from oracle.grm import vanraden_grm
from oracle.mme import MME, build_fixed_design, invert_psd_matrix
from oracle.reml import AIREML as OracleREML

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob():
    n, m = 300, 2000
    bed, _ = simulate_bed(n, m, seed=1000, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, n, m)["G"]
    Gi = invert_psd_matrix(G)
    g = genetic_values(bed, n, m, seed=1002, var_a=0.4)
    rec = simulate_gblup_records(n, 2, g, seed=1003, var_e=0.6)
    p, rows, _ = build_fixed_design(rec["cats"])
    return {"n": n, "G": G, "Gi": Gi, "rec": rec, "p": p, "rows": rows,
            "mme": MME(rec["y"], rec["aid"], rows, p, n)}


def dev(handle, d):
    dm = DeviceMME(handle, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    dm.set_qinv_dense(d["Gi"])
    return dm


def relerr(a, b):
    return abs(a - b) / abs(b)


def test_invert_psd_matches_oracle(handle, prob):
    Gi = invert_psd(handle, prob["G"])
    ref = prob["Gi"]
    assert np.abs(Gi - ref).max() <= 1e-9 * np.abs(ref).max()
    # ridge path
    Gr = invert_psd(handle, prob["G"], ridge=0.01)
    refr = invert_psd_matrix(prob["G"], 0.01)
    assert np.abs(Gr - refr).max() <= 1e-9 * np.abs(refr).max()


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_em_iteration_matches_oracle(handle, prob, precision):
    o = OracleREML(prob["mme"], prob["Gi"], 1.0, 1.0)
    ores = o.em_iteration()
    r = AIREML(dev(handle, prob), 1.0, 1.0, RemlConfig.default(mode=MODE_EM, precision=precision))
    info = r.run_iteration()
    assert info["kind"] == 0
    assert info["probes"] == ores["samples"]
    assert relerr(info["trace"], ores["trace"]) < 1e-8
    assert relerr(info["e_sse"], ores["e_sse"]) < 1e-8
    assert relerr(info["uQu"], ores["uQu"]) < 1e-8
    assert relerr(r.var_u, o.var_u) < 1e-6
    assert relerr(r.var_e, o.var_e) < 1e-6


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_em_solve_three_iterations(handle, prob, precision):
    """Consecutive EM iterations: from the second on, the data and probe
    solves are warm-started from the previous iteration and (mixed precision)
    their residuals are carried to the new lambda."""
    o = OracleREML(prob["mme"], prob["Gi"], 1.0, 1.0, max_iter=3)
    o.solve(dense_exact=False)
    r = AIREML(dev(handle, prob), 1.0, 1.0, RemlConfig.default(mode=MODE_EM, max_iter=3, precision=precision))
    r.solve()
    assert r.iterations == o.iterations
    assert relerr(r.var_u, o.var_u) < 1e-6
    assert relerr(r.var_e, o.var_e) < 1e-6


def test_dense_exact_solve_matches_oracle(handle, prob):
    o = OracleREML(prob["mme"], prob["Gi"], 1.0, 1.0)
    o.solve(dense_exact=True)
    r = AIREML(dev(handle, prob), 1.0, 1.0, RemlConfig.default(mode=MODE_DENSE))
    r.solve()
    assert r.converged == o.converged
    assert r.iterations == o.iterations
    assert relerr(r.var_u, o.var_u) < 1e-6
    assert relerr(r.var_e, o.var_e) < 1e-6
    assert all(h["kind"] == 1 for h in r.history)
    assert np.isfinite(r.history[-1]["logL"])


def test_dense_exact_step_logl(handle, prob):
    o = OracleREML(prob["mme"], prob["Gi"], 0.5, 0.8)
    assert o.dense_exact_step()
    r = AIREML(dev(handle, prob), 0.5, 0.8, RemlConfig.default(mode=MODE_DENSE))
    info = r.run_iteration()
    assert relerr(r.var_u, o.var_u) < 1e-6 and relerr(r.var_e, o.var_e) < 1e-6
    assert relerr(info["logL"], o.history[-1][1]) < 1e-9
