"""GPU parity tests of the multi-trait path: eigen-EM variance estimation
(cbx_mt_vce) and the Kronecker multi-trait MME solve (cbx_mt_solve) against
the oracle's restatement of MvEigenVce and GSSolve::solveMultiTrait."""
import numpy as np
import pytest

from cosmicblup_gb300 import MvEigenVce, MvOptions, invert_psd, solve_multi_trait
from cosmicblup_gb300.synth import simulate_bed, simulate_mt_records
from oracle.grm import vanraden_grm
from oracle.mme import invert_psd_matrix
from oracle.mt import mt_solve, mv_eigen_vce

pytestmark = pytest.mark.gpu

RG = np.array([[1.0, 0.5, -0.3], [0.5, 1.0, 0.2], [-0.3, 0.2, 1.0]])
SD_G = np.sqrt([0.3, 0.4, 0.5])
VG = RG * np.outer(SD_G, SD_G)
SD_E = np.sqrt([0.7, 0.6, 0.5])
VE = (np.full((3, 3), 0.1) + 0.9 * np.eye(3)) * np.outer(SD_E, SD_E)


@pytest.fixture(scope="module")
def mtp():
    n, m = 400, 2000
    bed, _ = simulate_bed(n, m, seed=700, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, n, m)["G"]
    Ginv = invert_psd_matrix(G)
    Grec = np.linalg.inv(Ginv)          # the reference recovers G from G^-1
    Grec = 0.5 * (Grec + Grec.T)
    rec = simulate_mt_records(bed, n, m, seed=701, Vg=VG, Ve=VE)
    return {"n": n, "G": G, "Ginv": Ginv, "Grec": Grec, "Y": rec["Y"], "X": rec["X"]}


def test_mt_vce_matches_oracle(handle, mtp):
    o = mv_eigen_vce(mtp["Y"], mtp["X"], mtp["Grec"], max_iter=500, tol=1e-4)
    v = MvEigenVce(handle, MvOptions(max_iter=500, tol=1e-4))
    v.prepare(mtp["Y"], mtp["X"], mtp["Grec"])
    conv = v.runNullModel()
    assert conv == o["converged"]
    assert v.iterations == o["iterations"]
    np.testing.assert_allclose(v.getVg(), o["Vg"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(v.getVe(), o["Ve"], rtol=1e-8, atol=1e-10)


def test_mt_vce_tight_tolerance(handle, mtp):
    o = mv_eigen_vce(mtp["Y"], mtp["X"], mtp["Grec"], max_iter=3000, tol=1e-9)
    v = MvEigenVce(handle, MvOptions(max_iter=3000, tol=1e-9))
    v.prepare(mtp["Y"], mtp["X"], mtp["Grec"])
    v.runNullModel()
    assert abs(v.iterations - o["iterations"]) <= 1
    np.testing.assert_allclose(v.getVg(), o["Vg"], rtol=1e-7, atol=1e-10)
    np.testing.assert_allclose(v.getVe(), o["Ve"], rtol=1e-7, atol=1e-10)


def test_mt_vce_from_device_ginv(handle, mtp):
    invert_psd(handle, mtp["G"])        # leaves G^-1 on the device
    o = mv_eigen_vce(mtp["Y"], mtp["X"], mtp["Grec"], max_iter=500, tol=1e-4)
    v = MvEigenVce(handle)
    v.prepare(mtp["Y"], mtp["X"], None)
    v.runNullModel()
    np.testing.assert_allclose(v.getVg(), o["Vg"], rtol=1e-6)
    np.testing.assert_allclose(v.getVe(), o["Ve"], rtol=1e-6)


def test_mt_solve_matches_oracle(handle, mtp):
    o = mt_solve(mtp["Y"], mtp["X"], mtp["Ginv"], VG, VE)
    r = solve_multi_trait(handle, mtp["Y"], mtp["X"], VG, VE, Ginv=mtp["Ginv"])
    np.testing.assert_allclose(r["beta"], o["beta"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(r["u"], o["u"], rtol=1e-8, atol=1e-8 * np.abs(o["u"]).max())
    assert r["u_mat"].shape == (mtp["n"], 3)


def test_mt_rejects_bad_sizes(handle, mtp):
    from cosmicblup_gb300 import CbxError
    v = MvEigenVce(handle)
    v.prepare(mtp["Y"][:, :1].repeat(9, axis=1), mtp["X"], mtp["Grec"])
    with pytest.raises(CbxError):
        v.runNullModel()
