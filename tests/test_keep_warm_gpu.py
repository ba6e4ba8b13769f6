"""Warm starts across MME rebuilds (cbx_mme_keep_warm): a REML run whose records
are uploaded again at every iteration, as the reference keeps last_solution
across the iterations of one run (src/core/vce.cpp:1226-1235).

With the option on, the iteration on a rebuilt MME starts from the previous
MME's solutions and reaches the same variance components as the same iteration
on one MME; with it off (the default), a rebuilt MME starts cold and repeats a
fresh handle's iteration exactly."""
import numpy as np
import pytest

from cosmicblup_gb300 import AIREML, DeviceMME, Handle, RemlConfig
from cosmicblup_gb300.mme import MIXED
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from cosmicblup_gb300.vce import MODE_EM
from oracle.grm import vanraden_grm
from oracle.mme import build_fixed_design, invert_psd_matrix

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob():
    n, m = 400, 2500
    bed, _ = simulate_bed(n, m, seed=1400, p_lo=0.05, miss=0.01)
    Gi = invert_psd_matrix(vanraden_grm(bed, n, m)["G"])
    g = genetic_values(bed, n, m, seed=1401, var_a=0.4)
    rec = simulate_gblup_records(n, 2, g, seed=1402, var_e=0.6)
    p, rows, _ = build_fixed_design(rec["cats"])
    return {"n": n, "Gi": Gi, "rec": rec, "p": p, "rows": rows}


def rebuild(h, d):
    dm = DeviceMME(h, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    dm.set_qinv_dense(d["Gi"])
    return dm


def iterate(dm, theta):
    r = AIREML(dm, *theta, RemlConfig.default(mode=MODE_EM, precision=MIXED, max_iter=1))
    info = r.run_iteration(grad_probes=32)
    return (r.var_u, r.var_e), info["pcg_iters"] + info["grad_pcg_iters"], info["grad"]


def test_rebuilt_mme_warm_start(handle, prob):
    theta0 = (0.5, 0.5)
    # the run on one MME: two iterations, the second warm
    dm = rebuild(handle, prob)
    r = AIREML(dm, *theta0, RemlConfig.default(mode=MODE_EM, precision=MIXED, max_iter=1))
    r.run_iteration(grad_probes=32)
    theta1 = (r.var_u, r.var_e)
    i2 = r.run_iteration(grad_probes=32)
    theta2_one = (r.var_u, r.var_e)
    # a cold iteration from theta1 on a fresh MME (option off)
    _, cold_its, _ = iterate(rebuild(handle, prob), theta1)
    try:
        # the run with the MME rebuilt at every iteration, warm starts kept
        t1, _, _ = iterate(rebuild(handle, prob), theta0)
        assert t1 == theta1
        handle.keep_warm(True)
        t2, warm_its, grad = iterate(rebuild(handle, prob), t1)
    finally:
        handle.keep_warm(False)
    for a, b in zip(t2, theta2_one):
        assert abs(a - b) <= 1e-7 * abs(b)
    assert np.abs(grad - i2["grad"]).max() <= 1e-6 * np.abs(i2["grad"]).max()
    assert warm_its < cold_its


def test_rebuilt_mme_starts_cold_by_default(prob):
    # a fresh handle's iteration ...
    with Handle(0) as h1:
        t_ref, its_ref, g_ref = iterate(rebuild(h1, prob), (0.5, 0.5))
    # ... equals the same iteration on an MME rebuilt after a finished run
    with Handle(0) as h2:
        dm = rebuild(h2, prob)
        iterate(dm, (0.7, 0.3))
        t, its, g = iterate(rebuild(h2, prob), (0.5, 0.5))
    assert its == its_ref
    assert t == t_ref
    assert np.array_equal(g, g_ref)
