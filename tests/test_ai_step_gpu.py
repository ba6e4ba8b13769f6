"""GPU parity of the data-driven AI-REML step (mode 3: run_aireml_step,
src/core/vce.cpp:2414-2857, on its direct-solver branch) against the oracle's
restatement: three consecutive iterations from the same start on a GBLUP
(dense eigen-bent G^-1) and on a single-step GBLUP (split H^-1), with the same
outcome per iteration (AI step accepted, or EM after a failed step), variance
components within 1e-6, the exact trace and logL within 1e-9."""
import numpy as np
import pytest

from cosmicblup_gb300 import AIREML, DeviceMME, RemlConfig, ssgblup_qinv
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records, simulate_pedigree
from cosmicblup_gb300.vce import MODE_AI
from oracle.grm import vanraden_grm
from oracle.mme import MME, build_fixed_design, invert_psd_matrix
from oracle.ped import a_columns, ainv_henderson as o_ainv, csr_to_dense, tune_g
from oracle.reml import AIREML as OracleREML

pytestmark = pytest.mark.gpu


def gblup_case():
    n, m = 300, 2000
    bed, _ = simulate_bed(n, m, seed=700, p_lo=0.05, miss=0.01)
    Gi = invert_psd_matrix(vanraden_grm(bed, n, m)["G"])
    g = genetic_values(bed, n, m, seed=701, var_a=0.4)
    rec = simulate_gblup_records(n, 3, g, seed=702, var_e=0.6)
    p, rows, _ = build_fixed_design(rec["cats"])
    return {"q": n, "Q": Gi, "rec": rec, "p": p, "rows": rows, "set": lambda dm: dm.set_qinv_dense(Gi)}


def ssgblup_case():
    sire, dam = simulate_pedigree(4, 150, 10, 60, seed=731, p_unknown=0.05)
    q, ng = len(sire), 150
    gmap = np.arange(q - ng, q, dtype=np.int32)
    bed, _ = simulate_bed(ng, 1500, seed=732, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, ng, 1500)["G"]
    ptr, col, val, F, dii = o_ainv(dam, sire)
    A22 = a_columns(dam, sire, dii, gmap)[gmap]
    Gt, _, _ = tune_g(G, A22)
    H = csr_to_dense(ptr, col, val, q)
    H[np.ix_(gmap, gmap)] += invert_psd_matrix(0.95 * Gt + 0.05 * A22) - np.linalg.inv(A22)
    rng = np.random.default_rng(733)
    rec = simulate_gblup_records(q, 5, rng.normal(0, 0.6, q), seed=734, var_e=0.65)
    p, rows, _ = build_fixed_design(rec["cats"])
    return {"q": q, "Q": H, "rec": rec, "p": p, "rows": rows,
            "set": lambda dm: ssgblup_qinv(dm, dam, sire, gmap, G=G)}


@pytest.mark.parametrize("case", [gblup_case, ssgblup_case])
def test_ai_data_step_three_iterations(handle, case):
    d = case()
    om = MME(d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["q"])
    o = OracleREML(om, d["Q"], 1.0, 1.0)
    dm = DeviceMME(handle, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["q"])
    d["set"](dm)
    r = AIREML(dm, 1.0, 1.0, RemlConfig.default(mode=MODE_AI))
    kinds = []
    for _ in range(3):
        ok = o.ai_data_step()
        if not ok:
            o.em_iteration()
        info = r.run_iteration()
        kinds.append(info["kind"])
        assert info["kind"] == (2 if ok else 0)
        if ok:
            assert abs(info["trace"] - o.last_ai_step["trace"]) <= 1e-9 * abs(o.last_ai_step["trace"])
            assert abs(info["logL"] - o.last_ai_step["logL"]) <= 1e-9 * abs(o.last_ai_step["logL"])
        assert abs(r.var_u - o.var_u) <= 1e-6 * o.var_u
        assert abs(r.var_e - o.var_e) <= 1e-6 * o.var_e
    assert 2 in kinds  # the AI step itself ran
