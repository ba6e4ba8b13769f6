"""GPU tests of the batched GBLUP entry (cbx_batch_reml): every problem of a
batch of uneven sizes gets exactly the single-problem result (GRM, eigen-bent
G^-1, AI-REML), whatever the number of workers; one problem also against the
oracle's REML restatement."""
import numpy as np
import pytest

from cosmicblup_gb300 import AIREML, BatchProblem, DeviceMME, Handle, RemlConfig, batch_reml, invert_psd
from cosmicblup_gb300.mme import MIXED
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from cosmicblup_gb300.vce import MODE_EM
from oracle.grm import vanraden_grm
from oracle.mme import MME, build_fixed_design, invert_psd_matrix
from oracle.reml import AIREML as OracleREML

pytestmark = pytest.mark.gpu

SIZES = [(180, 900), (260, 1500), (120, 700), (330, 2000), (220, 1100), (150, 1300)]


@pytest.fixture(scope="module")
def problems():
    out = []
    for i, (n, m) in enumerate(SIZES):
        bed, _ = simulate_bed(n, m, seed=700 + i, p_lo=0.05, miss=0.01)
        g = genetic_values(bed, n, m, seed=710 + i, var_a=0.3 + 0.05 * i)
        rec = simulate_gblup_records(n, 3 + i, g, seed=720 + i, var_e=0.6)
        p, rows, _ = build_fixed_design(rec["cats"])
        out.append(dict(pb=BatchProblem(bed=bed, n=n, m=m, y=rec["y"], aid=rec["aid"], rows=rows, p=p),
                        rec=rec, rows=rows, p=p, bed=bed, n=n, m=m))
    return out


def single(d, cfg):
    import ctypes as C
    from cosmicblup_gb300._lib import lib, ptr
    with Handle(0) as h:
        arr = np.frombuffer(d["bed"], dtype=np.uint8)
        s2, nv = C.c_double(0), C.c_int64(0)
        h.check(lib().cbx_grm_bed(h.raw, ptr(arr), arr.size, d["n"], d["m"], C.c_float(0.01), 1, 2048, None,
                                  None, None, C.byref(s2), C.byref(nv)))
        invert_psd(h, None, d["n"], download=False)
        dm = DeviceMME(h, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
        dm.set_qinv_dense(None)
        r = AIREML(dm, 0.5, 0.5, cfg)
        r.solve()
        return r.var_u, r.var_e, r.iterations


@pytest.mark.parametrize("workers", [1, 4])
def test_batch_equals_single(problems, workers):
    cfg = RemlConfig.default(mode=MODE_EM, precision=MIXED, max_iter=4)
    res = batch_reml([d["pb"] for d in problems], cfg, workers=workers)
    for d, r in zip(problems, res):
        assert r.status == 0
        vu, ve, it = single(d, cfg)
        assert r.iterations == it
        assert abs(r.var_u - vu) <= 1e-12 * vu and abs(r.var_e - ve) <= 1e-12 * ve
        assert r.solution.shape == (d["p"] + d["n"],) and np.isfinite(r.solution).all()


def test_batch_problem_against_oracle(problems):
    d = problems[1]
    cfg = RemlConfig.default(mode=MODE_EM, max_iter=2)
    r = batch_reml([d["pb"]], cfg, workers=1)[0]
    G = vanraden_grm(d["bed"], d["n"], d["m"])["G"]
    o = OracleREML(MME(d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"]), invert_psd_matrix(G), 0.5, 0.5,
                   max_iter=2)
    o.solve(dense_exact=False)
    assert abs(r.var_u - o.var_u) <= 1e-6 * o.var_u
    assert abs(r.var_e - o.var_e) <= 1e-6 * o.var_e
