"""GPU tests of the REML gradient entry (cbx_reml_gradient): exact traces against
central finite differences of the REML log-likelihood (relative step 1e-4), and
the 256-probe Hutchinson gradient against the oracle's restatement of the
reference's AI-REML score with the same probe vectors."""
import numpy as np
import pytest

from cosmicblup_gb300 import DeviceMME
from cosmicblup_gb300.mme import MIXED
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from cosmicblup_gb300.vce import reml_gradient, reml_logl_dense
from oracle.grm import vanraden_grm
from oracle.mme import MME, build_fixed_design, invert_psd_matrix
from oracle.reml import AIREML as OracleREML
from oracle.rng import adaptive_trace

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob():
    n, m = 250, 1500
    bed, _ = simulate_bed(n, m, seed=500, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, n, m)["G"]
    Gi = invert_psd_matrix(G)
    g = genetic_values(bed, n, m, seed=501, var_a=0.5)
    rec = simulate_gblup_records(n, 3, g, seed=502, var_e=0.5)
    p, rows, _ = build_fixed_design(rec["cats"])
    return {"n": n, "Gi": Gi, "rec": rec, "p": p, "rows": rows, "mme": MME(rec["y"], rec["aid"], rows, p, n)}


def dev(handle, d):
    dm = DeviceMME(handle, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    dm.set_qinv_dense(d["Gi"])
    return dm


def oracle_score(om, Gi, vu, ve, probes=None):
    lam = ve / vu
    A = om.lhs(Gi, lam)
    sol = np.linalg.solve(A, om.rhs())
    p, q, n = om.p, om.q, om.n
    u = sol[p:]
    e = om.y - om.mult_design(sol[:p], u)
    Cuu = np.linalg.inv(A)[p:, p:]
    if probes is None:
        tr = np.trace(Gi @ Cuu)
    else:
        tr = np.mean([z @ (Gi @ (Cuu @ z)) for z in probes])
    ltr = min(lam * tr, q - 1e-6)
    return np.array([0.5 * (u @ Gi @ u + tr * ve - q * vu) / vu**2,
                     0.5 * (e @ e - ve * (n - p - q + ltr)) / ve**2])


def test_exact_gradient_matches_finite_differences(handle, prob):
    dm = dev(handle, prob)
    vu, ve = 0.45, 0.55
    g = reml_gradient(dm, vu, ve, exact=True)["grad"]
    fd = []
    for k, (a, b) in enumerate([(vu, ve), (vu, ve)]):
        h = 1e-4 * (vu if k == 0 else ve)
        if k == 0:
            lp, lm = reml_logl_dense(dm, vu + h, ve), reml_logl_dense(dm, vu - h, ve)
        else:
            lp, lm = reml_logl_dense(dm, vu, ve + h), reml_logl_dense(dm, vu, ve - h)
        fd.append((lp - lm) / (2 * h))
    fd = np.array(fd)
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())
    np.testing.assert_allclose(g, oracle_score(prob["mme"], prob["Gi"], vu, ve), rtol=1e-8)
    # the oracle's dense log-likelihood agrees with the device one
    o = OracleREML(prob["mme"], prob["Gi"], vu, ve)
    o._init_dense()
    assert abs(o.logL(vu, ve) - reml_logl_dense(dm, vu, ve)) < 1e-8 * abs(o.logL(vu, ve))


@pytest.mark.parametrize("precision", [0, MIXED])
def test_hutchinson_gradient_matches_oracle(handle, prob, precision):
    dm = dev(handle, prob)
    vu, ve = 0.45, 0.55
    res = reml_gradient(dm, vu, ve, nprobe=256, seed=42, precision=precision)
    probes = []
    adaptive_trace(prob["n"], lambda z: (probes.append(z.copy()), np.zeros_like(z))[1], 256, 256, 0.0, 42)
    ref = oracle_score(prob["mme"], prob["Gi"], vu, ve, probes=probes)
    np.testing.assert_allclose(res["grad"], ref, rtol=1e-6)


@pytest.mark.parametrize("precision", [0, MIXED])
def test_gradient_after_iteration_reuses_forward_solves(handle, prob, precision):
    """The gradient right after an EM iteration at the same point takes the
    iteration's data-solve terms and probe solves (no PCG iteration when it
    needs no more probes than the iteration solved) and equals the standalone
    gradient; more probes than the iteration solved cost only the extra ones."""
    from cosmicblup_gb300 import AIREML, RemlConfig
    from cosmicblup_gb300.vce import MODE_EM
    vu, ve = 0.45, 0.55
    dm = dev(handle, prob)
    r = AIREML(dm, vu, ve, RemlConfig.default(mode=MODE_EM, precision=precision))
    k = r.run_iteration()["probes"]
    g_reuse = reml_gradient(dm, vu, ve, nprobe=k, seed=42, precision=precision)
    assert g_reuse["pcg_iters"] == 0
    g_more = reml_gradient(dm, vu, ve, nprobe=96, seed=42, precision=precision)
    assert g_more["pcg_iters"] > 0
    again = reml_gradient(dm, vu, ve, nprobe=96, seed=42, precision=precision)
    assert again["pcg_iters"] == 0 and np.array_equal(again["grad"], g_more["grad"])
    dm2 = dev(handle, prob)  # a fresh MME: no forward state
    g_alone = reml_gradient(dm2, vu, ve, nprobe=k, seed=42, precision=precision)
    assert g_alone["pcg_iters"] > 0
    # Each score component is a difference of terms of order q / (2 var_u) and
    # n / (2 var_e) (u'Qinv u + var_e tr against q var_u, and so on): the two
    # gradients come from different solves to relres 1e-10, so they agree to
    # 1e-8 of those terms.
    scale = max(prob["n"] / (2 * vu), prob["n"] / (2 * ve))
    np.testing.assert_allclose(g_reuse["grad"], g_alone["grad"], rtol=1e-8, atol=1e-8 * scale)
    g_alone96 = reml_gradient(dm2, vu, ve, nprobe=96, seed=42, precision=precision)
    np.testing.assert_allclose(g_more["grad"], g_alone96["grad"], rtol=1e-8, atol=1e-8 * scale)
    probes = []
    adaptive_trace(prob["n"], lambda z: (probes.append(z.copy()), np.zeros_like(z))[1], 96, 96, 0.0, 42)
    np.testing.assert_allclose(g_more["grad"], oracle_score(prob["mme"], prob["Gi"], vu, ve, probes=probes),
                               rtol=1e-6)


def test_exact_gradient_matches_finite_differences_ssgblup(handle):
    """The gradient with exact traces against central finite differences (relative
    step 1e-4) of the REML log-likelihood on a scaled single-step problem: 6
    generations x 500 animals, the last 500 genotyped (gene-dropped, m = 3,000),
    H^-1 from the device GRM, A22 recursion, tuneG and blend."""
    from cosmicblup_gb300 import GrmBuilder, GrmOptions, PlinkReader, ssgblup_qinv
    from cosmicblup_gb300.synth import simulate_bed_gene_drop, simulate_pedigree
    sire, dam = simulate_pedigree(6, 500, 20, 250, seed=3201, p_unknown=0.05)
    q, ng, m = sire.size, 500, 3000
    gmap = np.arange(q - ng, q, dtype=np.int32)
    bed, _ = simulate_bed_gene_drop(sire, dam, 500, m, seed=3200)
    GrmBuilder(GrmOptions(), handle=handle).compute(PlinkReader.from_bytes(bed, ng, m))
    rec = simulate_gblup_records(q, 20, np.random.default_rng(3202).normal(0, 0.6, q), seed=3203, var_e=0.65)
    p, rows, _ = build_fixed_design(rec["cats"])
    dm = DeviceMME(handle, rec["y"], rec["aid"], rows, p, q)
    ssgblup_qinv(dm, dam, sire, gmap, G=None)
    vu, ve = 0.4, 0.6
    g = reml_gradient(dm, vu, ve, exact=True, precision=MIXED)["grad"]
    fd = []
    for k in range(2):
        hk = 1e-4 * (vu if k == 0 else ve)
        if k == 0:
            lp, lm = reml_logl_dense(dm, vu + hk, ve), reml_logl_dense(dm, vu - hk, ve)
        else:
            lp, lm = reml_logl_dense(dm, vu, ve + hk), reml_logl_dense(dm, vu, ve - hk)
        fd.append((lp - lm) / (2 * hk))
    fd = np.array(fd)
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())


@pytest.mark.parametrize("precision", [0, MIXED])
def test_iteration_with_gradient_in_one_block(handle, prob, precision):
    """cbx_reml_iterate_grad: in mixed precision the gradient's 64 probes join the
    iteration's data + probe block (65 columns, the 128-wide solver), so the
    gradient solves nothing; the iteration (same probes selected by its
    estimator) and the gradient equal those of the separate calls to the
    tolerance of their solves, and the iteration matches the oracle."""
    from cosmicblup_gb300 import AIREML, RemlConfig
    from cosmicblup_gb300.vce import MODE_EM
    vu, ve = 0.45, 0.55
    scale = max(prob["n"] / (2 * vu), prob["n"] / (2 * ve))
    r1 = AIREML(dev(handle, prob), vu, ve, RemlConfig.default(mode=MODE_EM, precision=precision))
    d1 = r1.run_iteration(grad_probes=64)
    if precision == MIXED:
        assert d1["grad_pcg_iters"] == 0
    dm2 = dev(handle, prob)
    r2 = AIREML(dm2, vu, ve, RemlConfig.default(mode=MODE_EM, precision=precision))
    d2 = r2.run_iteration()
    g2 = reml_gradient(dm2, vu, ve, nprobe=64, seed=42, precision=precision)
    assert d1["probes"] == d2["probes"]
    assert abs(r1.var_u - r2.var_u) <= 1e-9 * r2.var_u and abs(r1.var_e - r2.var_e) <= 1e-9 * r2.var_e
    np.testing.assert_allclose(d1["grad"], g2["grad"], rtol=1e-8, atol=1e-8 * scale)
    assert abs(d1["grad_trace"] - g2["trace"]) <= 1e-8 * abs(g2["trace"])
    o = OracleREML(prob["mme"], prob["Gi"], vu, ve)
    o.em_iteration()
    assert abs(r1.var_u - o.var_u) <= 1e-6 * o.var_u and abs(r1.var_e - o.var_e) <= 1e-6 * o.var_e
    # a second combined call continues warm from the 65-column block
    d3 = r1.run_iteration(grad_probes=64)
    if precision == MIXED:
        assert d3["grad_pcg_iters"] == 0
    assert np.all(np.isfinite(d3["grad"]))
