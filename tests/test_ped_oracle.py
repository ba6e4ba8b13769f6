"""CPU tests of the pedigree oracle: Henderson A^-1 against the inverse of the
tabular A, and the A = T D T^T column recursion against the same A."""
import numpy as np

from cosmicblup_gb300.synth import simulate_pedigree
from oracle.ped import a_columns, ainv_henderson, csr_to_dense, ml


def tabular_A(dam, sire):
    n = len(dam)
    A = np.zeros((n, n))
    for i in range(n):
        s, d = sire[i], dam[i]
        A[i, i] = 1.0 + (0.5 * A[s, d] if s >= 0 and d >= 0 else 0.0)
        for j in range(i):
            v = 0.0
            if s >= 0:
                v += A[j, s]
            if d >= 0:
                v += A[j, d]
            A[i, j] = A[j, i] = 0.5 * v
    return A


def test_toy_pedigree_inbreeding():
    # sample1..6 of the reference's inline test pedigree (tests/run_case.py): 5 and 6 are full-sib matings
    sire = np.array([-1, -1, 0, 0, 2, 2])
    dam = np.array([-1, -1, 1, 1, 3, 3])
    F, dii = ml(dam, sire)
    A = tabular_A(dam, sire)
    np.testing.assert_allclose(F, np.diag(A) - 1.0, atol=1e-15)
    assert F[4] == 0.25 and F[5] == 0.25


def test_henderson_inverse_matches_tabular():
    sire, dam = simulate_pedigree(4, 60, 6, 20, seed=3, p_unknown=0.1)
    n = len(sire)
    ptr, col, val, F, dii = ainv_henderson(dam, sire)
    Ainv = csr_to_dense(ptr, col, val, n)
    A = tabular_A(dam, sire)
    np.testing.assert_allclose(Ainv @ A, np.eye(n), atol=1e-9)
    np.testing.assert_allclose(F, np.diag(A) - 1.0, atol=1e-12)


def test_a_column_recursion():
    sire, dam = simulate_pedigree(5, 40, 5, 15, seed=4)
    n = len(sire)
    _, _, _, F, dii = ainv_henderson(dam, sire)
    cols = np.arange(n - 40, n)
    A = tabular_A(dam, sire)
    np.testing.assert_allclose(a_columns(dam, sire, dii, cols), A[:, cols], atol=1e-12)
