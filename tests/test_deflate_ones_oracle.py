"""The one-null-direction path of the eigen-bending inverse, as a numpy model of
its steps, against the oracle's invert_psd_matrix (CPU, oracle only).

invert_psd_matrix (reference src/core/matrix_io.cpp:488-501) raises every
eigenvalue of M below eps = 1e-6 to eps and inverts.  A VanRaden G has exactly
one such eigenvalue when it has fewer animals than SNPs: its centred columns sum
to zero, so the all-ones direction is (nearly) null.  The device path
(reml.cu, deflate_ones) finds that eigenpair by inverse iteration with the
Cholesky factor of M + eps I, checks with a second Cholesky factor that every
other eigenvalue is above 100 eps, and inverts M + (eps - u'Mu) u u^T by
Cholesky.  With more animals than SNPs there are many small eigenvalues; the
check fails there and the device takes its syevdx path.
"""
import numpy as np
import pytest
import scipy.linalg as sl

from cosmicblup_gb300.synth import simulate_bed
from oracle.grm import vanraden_grm
from oracle.mme import invert_psd_matrix

EPS = 1e-6


def deflate_ones(M):
    """The device path's steps; None where it would fall back."""
    n = M.shape[0]
    v = np.full(n, 1.0 / np.sqrt(n))
    if not v @ M @ v < EPS:
        return None
    F = np.linalg.cholesky(M + EPS * np.eye(n))
    u = v.copy()
    for _ in range(8):
        u = sl.cho_solve((F, True), u)
        u /= np.linalg.norm(u)
    rho = u @ M @ u
    if not rho < EPS:
        return None
    c = np.abs(M).sum(axis=1).max() + 1.0
    try:
        np.linalg.cholesky(M + c * np.outer(u, u) - 100 * EPS * np.eye(n))
    except np.linalg.LinAlgError:
        return None
    return np.linalg.inv(M + (EPS - rho) * np.outer(u, u))


@pytest.mark.parametrize("n,m,seed", [(300, 2000, 1000), (500, 4000, 1001)])
def test_matches_the_eigen_bending_inverse(n, m, seed):
    bed, _ = simulate_bed(n, m, seed=seed, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, n, m)["G"]
    assert (np.linalg.eigvalsh(G) < EPS).sum() == 1
    got = deflate_ones(G)
    ref = invert_psd_matrix(G)
    assert got is not None
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_more_animals_than_snps_falls_back():
    bed, _ = simulate_bed(400, 300, seed=1002, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, 400, 300)["G"]
    assert (np.linalg.eigvalsh(G) < EPS).sum() > 1
    assert deflate_ones(G) is None
