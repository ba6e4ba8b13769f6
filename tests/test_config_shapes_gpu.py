"""GPU parity at the shapes of the benchmark configurations.

* The plain GBLUP configuration in full (n = 2,000 animals, m = 10,000 SNPs,
  allele frequencies U(0.05, 0.5), 1 % missing calls, mean + 2-level sex
  effect): GRM integer cross-products bit-exact, G within 1e-13 of the oracle's
  FP64 GEMM, the eigen-bent G^-1 within 1e-9, dense exact AI-REML to
  convergence with variance components within 1e-6 and the same iteration
  count, and the final EBVs within 1e-8.
* Single-step GBLUP at a tenth of the ssGBLUP configuration's pedigree (10
  generations x 1,000 animals, 25 sires x 500 dams per generation, 5 % unknown
  parents, the last 1,000 genotyped at m = 5,000 by gene dropping): three EM +
  Hutchinson REML iterations on the device H^-1 (device GRM, A22 recursion,
  tuneG, blend, inverses) against the oracle's sparse-direct EM, variance
  components within 1e-6 and identical probe counts after every iteration.
* The large GBLUP configuration's GRM (n = 20,000, m = 50,000, 2 % missing):
  integer cross-products bit-exact and G within its exact-rounding bound on
  sampled 128 x 128 tiles (diagonal, off-diagonal and the ragged last rows).
"""
import numpy as np
import pytest

from cosmicblup_gb300 import (AIREML, DeviceMME, GrmBuilder, GrmOptions, PlinkReader, RemlConfig,
                              ssgblup_qinv)
from cosmicblup_gb300.mme import FP64, MIXED
from cosmicblup_gb300.synth import (genetic_values, simulate_bed, simulate_bed_gene_drop,
                                    simulate_gblup_records, simulate_pedigree)
from cosmicblup_gb300.vce import MODE_DENSE, MODE_EM, final_solve, invert_psd
from oracle.grm import grm_tiles_exact, snp_stats, vanraden_grm
from oracle.mme import MME, build_fixed_design, invert_psd_matrix, sparse_data_part
from oracle.plink import decode_bed
from oracle.ped import a_columns, ainv_henderson as o_ainv, tune_g
from oracle.reml import AIREML as OracleREML, SparseEM, hinv_sparse

pytestmark = pytest.mark.gpu


def gpu_grm(handle, bed, n, m):
    b = GrmBuilder(GrmOptions(), handle=handle)
    b.compute(PlinkReader.from_bytes(bed, n, m), keep_xx_counts=True)
    return b


@pytest.fixture(scope="module")
def c1(handle):
    n, m = 2000, 10000
    bed, _ = simulate_bed(n, m, seed=1000, p_lo=0.05, miss=0.01)
    g = genetic_values(bed, n, m, seed=1002, var_a=0.4)
    rec = simulate_gblup_records(n, 2, g, seed=1003, var_e=0.6)
    p, rows, _ = build_fixed_design(rec["cats"])
    ref = vanraden_grm(bed, n, m)
    return {"n": n, "m": m, "bed": bed, "rec": rec, "p": p, "rows": rows, "ref": ref,
            "Gi": invert_psd_matrix(ref["G"])}


def test_c1_grm_counts_and_inverse(handle, c1):
    n, m = c1["n"], c1["m"]
    b = gpu_grm(handle, c1["bed"], n, m)
    geno = decode_bed(c1["bed"], n, m)
    st = snp_stats(geno)
    x = np.where(geno[st["valid"]] >= 0, geno[st["valid"]], 0).astype(np.float64)
    xx = np.rint(x.T @ x).astype(np.int64)  # exact: integer sums below 2^53
    np.testing.assert_array_equal(b.getXXCounts(), xx)
    ref = c1["ref"]
    assert b.getSum2pq() == ref["sum2pq"] and b.getTotalSnps() == ref["n_valid"]
    assert np.abs(b.getGrm() - ref["G"]).max() <= 1e-13 * np.abs(ref["G"]).max()
    Gi = invert_psd(handle, None, n)  # the device GRM left by the builder
    assert np.abs(Gi - c1["Gi"]).max() <= 1e-9 * np.abs(c1["Gi"]).max()


def test_c1_dense_exact_reml_to_convergence(handle, c1):
    n, p = c1["n"], c1["p"]
    rec = c1["rec"]
    om = MME(rec["y"], rec["aid"], c1["rows"], p, n)
    o = OracleREML(om, c1["Gi"], 1.0, 1.0)
    o.solve(dense_exact=True)
    dm = DeviceMME(handle, rec["y"], rec["aid"], c1["rows"], p, n)
    dm.set_qinv_dense(c1["Gi"])
    r = AIREML(dm, 1.0, 1.0, RemlConfig.default(mode=MODE_DENSE))
    r.solve()
    assert r.converged == o.converged and r.iterations == o.iterations
    assert abs(r.var_u - o.var_u) <= 1e-6 * o.var_u
    assert abs(r.var_e - o.var_e) <= 1e-6 * o.var_e
    # final EBVs at the device's estimates (dense Cholesky, as the reference's LDLT)
    fs = final_solve(dm, r.var_u, r.var_e, solver=0, calc_se=False)
    xe = np.linalg.solve(om.lhs(c1["Gi"], r.var_e / r.var_u), om.rhs())
    assert np.abs(fs["u"] - xe[p:]).max() <= 1e-8 * np.abs(xe[p:]).max()


@pytest.fixture(scope="module")
def c3s():
    n_gen, per_gen, ng, m = 10, 1000, 1000, 5000
    sire, dam = simulate_pedigree(n_gen, per_gen, 25, 500, seed=3101, p_unknown=0.05)
    q = sire.size
    gmap = np.arange(q - ng, q, dtype=np.int32)
    bed, _ = simulate_bed_gene_drop(sire, dam, per_gen, m, seed=3100, p_lo=0.01, miss=0.02)
    G = vanraden_grm(bed, ng, m)["G"]
    ptr, col, val, F, dii = o_ainv(dam, sire)
    A22 = a_columns(dam, sire, dii, gmap)[gmap]
    Gt, _, _ = tune_g(G, A22)
    Gd = invert_psd_matrix(0.95 * Gt + 0.05 * A22) - np.linalg.inv(A22)
    rng = np.random.default_rng(3102)
    rec = simulate_gblup_records(q, 50, rng.normal(0, 0.6, q), seed=3103, var_e=0.65)
    p, rows, _ = build_fixed_design(rec["cats"])
    _, W = sparse_data_part(rec["aid"], rows, p, q)
    # three oracle iterations from (0.5, 0.5), shared by both precisions
    o = SparseEM(W, rec["y"], hinv_sparse((ptr, col, val), Gd, gmap), p, 0.5, 0.5)
    its = []
    for _ in range(3):
        r = o.em_iteration()
        its.append({"samples": r["samples"], "trace": r["trace"], "var_u": o.var_u, "var_e": o.var_e})
    return dict(sire=sire, dam=dam, q=q, ng=ng, m=m, gmap=gmap, bed=bed, rec=rec, p=p, rows=rows, oracle=its)


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_scaled_ssgblup_em_three_iterations(handle, c3s, precision):
    d = c3s
    gpu_grm(handle, d["bed"], d["ng"], d["m"])  # the GRM stays on the device
    dm = DeviceMME(handle, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["q"])
    ssgblup_qinv(dm, d["dam"], d["sire"], d["gmap"], G=None)
    r = AIREML(dm, 0.5, 0.5, RemlConfig.default(mode=MODE_EM, precision=precision))
    for o in d["oracle"]:
        info = r.run_iteration()
        assert info["probes"] == o["samples"]
        assert abs(info["trace"] - o["trace"]) <= 1e-7 * abs(o["trace"])
        assert abs(r.var_u - o["var_u"]) <= 1e-6 * o["var_u"]
        assert abs(r.var_e - o["var_e"]) <= 1e-6 * o["var_e"]


def test_grm_tiles_at_n20000(handle):
    n, m = 20000, 50000
    bed, _ = simulate_bed(n, m, seed=2000, p_lo=0.01, miss=0.02)
    b = gpu_grm(handle, bed, n, m)
    xx, G = b.getXXCounts(), b.getGrm()
    t = np.arange(128)
    tiles = [(t + 0, t + 0), (t + 6400, t + 13056), (t + 19872, t + 2048), (t + 19872, t + 19872)]
    ex = grm_tiles_exact(bed, n, m, tiles)
    assert b.getSum2pq() == ex["sum2pq"] and b.getTotalSnps() == ex["n_valid"]
    for (r, c), x, g in zip(tiles, ex["xx"], ex["G"]):
        np.testing.assert_array_equal(xx[np.ix_(r, c)], x)
        bound = ex["n_valid"] * 2.0**-46 / ex["sum2pq"] + 4 * np.spacing(np.abs(g))
        assert np.all(np.abs(G[np.ix_(r, c)] - g) <= bound)
