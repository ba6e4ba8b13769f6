"""GPU parity tests of the ssGBLUP path: Henderson A^-1, the H^-1 blocks
(A22, tuneG, blend, eigen-bent inverse, A22^-1), PCG and an EM REML iteration
on the split H^-1, against the oracle."""
import numpy as np
import pytest

from cosmicblup_gb300 import AIREML, DeviceMME, RemlConfig, ainv_henderson, ssgblup_qinv
from cosmicblup_gb300.synth import simulate_bed, simulate_gblup_records, simulate_pedigree
from cosmicblup_gb300.vce import MODE_EM
from oracle.grm import vanraden_grm
from oracle.mme import MME, build_fixed_design, invert_psd_matrix
from oracle.ped import a_columns, ainv_henderson as o_ainv, csr_to_dense, tune_g
from oracle.reml import AIREML as OracleREML

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ss():
    sire, dam = simulate_pedigree(4, 150, 10, 60, seed=31, p_unknown=0.05)
    n = len(sire)
    ng = 150
    gmap = np.arange(n - ng, n, dtype=np.int32)  # last generation genotyped
    bed, _ = simulate_bed(ng, 1500, seed=32, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, ng, 1500)["G"]
    ptr, col, val, F, dii = o_ainv(dam, sire)
    Ainv = csr_to_dense(ptr, col, val, n)
    A22 = a_columns(dam, sire, dii, gmap)[gmap]
    Gt, a, b = tune_g(G, A22)
    Gb = 0.95 * Gt + 0.05 * A22
    Gd = invert_psd_matrix(Gb) - np.linalg.inv(A22)
    H = Ainv.copy()
    H[np.ix_(gmap, gmap)] += Gd
    rng = np.random.default_rng(33)
    rec = simulate_gblup_records(n, 5, rng.normal(0, 0.6, n), seed=34, var_e=0.65)
    p, rows, _ = build_fixed_design(rec["cats"])
    return dict(sire=sire, dam=dam, n=n, ng=ng, gmap=gmap, G=G, Ainv=(ptr, col, val), F=F, dii=dii,
                A22=A22, Gd=Gd, H=H, rec=rec, p=p, rows=rows, mme=MME(rec["y"], rec["aid"], rows, p, n))


def test_ainv_henderson_bit_exact(handle, ss):
    p_, c_, v_, F, d = ainv_henderson(handle, ss["dam"], ss["sire"], with_inbreeding=True)
    op, oc, ov = ss["Ainv"]
    np.testing.assert_array_equal(p_, op)
    np.testing.assert_array_equal(c_, oc)
    np.testing.assert_array_equal(v_, ov)
    np.testing.assert_array_equal(F, ss["F"])
    np.testing.assert_array_equal(d, ss["dii"])


def test_hinv_blocks(handle, ss):
    dm = DeviceMME(handle, ss["rec"]["y"], ss["rec"]["aid"], ss["rows"], ss["p"], ss["n"])
    A22, Gd = ssgblup_qinv(dm, ss["dam"], ss["sire"], ss["gmap"], G=ss["G"], return_blocks=True)
    assert np.abs(A22 - ss["A22"]).max() < 1e-12
    assert np.abs(Gd - ss["Gd"]).max() <= 1e-9 * np.abs(ss["Gd"]).max()
    X = np.random.default_rng(1).normal(size=(ss["n"], 2))
    Y = dm.qinv_apply(X)
    assert np.abs(Y - ss["H"] @ X).max() <= 1e-9 * np.abs(ss["H"] @ X).max()


def test_pcg_and_em_on_hinv(handle, ss):
    dm = DeviceMME(handle, ss["rec"]["y"], ss["rec"]["aid"], ss["rows"], ss["p"], ss["n"])
    ssgblup_qinv(dm, ss["dam"], ss["sire"], ss["gmap"], G=ss["G"])
    om = ss["mme"]
    lam = 1.4
    A = om.lhs(ss["H"], lam)
    b = om.rhs()
    x, it, rr = dm.pcg_solve(lam, b)
    xe = np.linalg.solve(A, b)
    assert np.abs(x - xe).max() <= 1e-8 * np.abs(xe).max()
    o = OracleREML(om, ss["H"], 0.5, 0.7)
    ores = o.em_iteration()
    r = AIREML(dm, 0.5, 0.7, RemlConfig.default(mode=MODE_EM))
    info = r.run_iteration()
    assert info["probes"] == ores["samples"]
    assert abs(r.var_u - o.var_u) <= 1e-6 * o.var_u
    assert abs(r.var_e - o.var_e) <= 1e-6 * o.var_e


def test_split_with_device_block_equals_host_block(handle, ss):
    """A later MME of the handle takes the dense H^-1 block that ssgblup_qinv left on
    the device (Gd omitted): the same operator as the block passed from the host."""
    dm = DeviceMME(handle, ss["rec"]["y"], ss["rec"]["aid"], ss["rows"], ss["p"], ss["n"])
    _, Gd = ssgblup_qinv(dm, ss["dam"], ss["sire"], ss["gmap"], G=ss["G"], return_blocks=True)
    Ainv = ainv_henderson(handle, ss["dam"], ss["sire"])
    X = np.random.default_rng(2).normal(size=(ss["n"], 3))
    dm_host = DeviceMME(handle, ss["rec"]["y"], ss["rec"]["aid"], ss["rows"], ss["p"], ss["n"])
    dm_host.set_qinv_split(*Ainv, Gd=Gd, gmap=ss["gmap"])
    Y_host = dm_host.qinv_apply(X)
    x_host, _, _ = dm_host.pcg_solve(1.4, ss["mme"].rhs())
    dm_dev = DeviceMME(handle, ss["rec"]["y"], ss["rec"]["aid"], ss["rows"], ss["p"], ss["n"])
    dm_dev.set_qinv_split(*Ainv, gmap=ss["gmap"])
    np.testing.assert_array_equal(dm_dev.qinv_apply(X), Y_host)
    x_dev, _, _ = dm_dev.pcg_solve(1.4, ss["mme"].rhs())
    np.testing.assert_array_equal(x_dev, x_host)
