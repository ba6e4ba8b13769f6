"""CPU tests of the multi-trait oracle: the vectorised EM update against a
per-sample restatement of MvEigenVce::updateEM (src/core/eigen_vce.cpp:163-237),
invariance of Vg / Ve to the null-space basis, and the Kronecker MME ordering
against the equivalent V-matrix (GLS + BLUP) solution."""
import numpy as np

from oracle.mt import em_update, mt_solve, mv_eigen_vce, mv_prepare


def _data(n=120, t=3, p=2, seed=0):
    rng = np.random.default_rng(seed)
    Z = rng.standard_normal((n, 3 * n))
    G = Z @ Z.T / (3 * n) + 0.05 * np.eye(n)
    X = np.zeros((n, p))
    X[:, 0] = 1.0
    if p > 1:
        X[rng.random(n) < 0.5, 1] = 1.0
    Vg = np.array([[0.4, 0.1, -0.05], [0.1, 0.5, 0.04], [-0.05, 0.04, 0.3]])[:t, :t]
    Ve = np.array([[0.6, 0.05, 0.05], [0.05, 0.5, 0.05], [0.05, 0.05, 0.7]])[:t, :t]
    L = np.linalg.cholesky(np.kron(Vg, G) + np.kron(Ve, np.eye(n)))
    y = L @ rng.standard_normal(n * t)
    Y = y.reshape(t, n).T + 3.0
    return Y, X, G, Vg, Ve


def update_em_loop(D, Uty, Vg, Ve):
    """updateEM as written: per-sample V_i solve, S_g / S_e accumulation (no covariates)."""
    n, t = Uty.shape
    Sg = np.zeros((t, t))
    Se = np.zeros((t, t))
    for i in range(n):
        Vi = Vg * D[i] + Ve
        P = np.linalg.solve(Vi, np.eye(t))
        r = Uty[i]
        Wg = Vg * D[i] @ P
        uh = Wg @ r
        if D[i] > 1e-12:
            Sg += np.outer(uh, uh) / D[i] + Vg - Wg @ Vg
        else:
            Sg += Vg
        We = Ve @ P
        eh = We @ r
        Se += np.outer(eh, eh) + Ve - We @ Ve
    return Sg / n, Se / n


def test_em_update_matches_per_sample_loop():
    Y, X, G, Vg, Ve = _data()
    D, Uty, n_eff, Vg0, Ve0 = mv_prepare(Y, X, G)
    D = D.copy()
    D[:3] = 0.0  # exercise the d_i ~ 0 branch
    a = em_update(D, Uty, Vg0, Ve0)
    b = update_em_loop(D, Uty, Vg0, Ve0)
    np.testing.assert_allclose(a[0], b[0], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(a[1], b[1], rtol=1e-12, atol=1e-14)


def test_vce_invariant_to_null_space_basis():
    Y, X, G, _, _ = _data(seed=1)
    ref = mv_eigen_vce(Y, X, G, max_iter=200, tol=1e-8)
    # a different orthonormal basis of null(X'): rotate the QR basis
    n, p = X.shape
    Q, _ = np.linalg.qr(X, mode="complete")
    A = Q[:, p:] @ np.linalg.qr(np.random.default_rng(5).standard_normal((n - p, n - p)))[0]
    D, U = np.linalg.eigh(A.T @ G @ A)
    D = np.where(D < 0, 0.0, D)
    Uty = U.T @ (A.T @ Y)
    Yc = Y - Y.mean(0)
    Vg = Ve = 0.5 * (Yc.T @ Yc) / (n - p - 1)
    for _ in range(ref["iterations"]):
        Vg, Ve = em_update(D, Uty, Vg, Ve)
    np.testing.assert_allclose(Vg, ref["Vg"], rtol=1e-9)
    np.testing.assert_allclose(Ve, ref["Ve"], rtol=1e-9)


def test_kronecker_mme_matches_gls_blup():
    Y, X, G, Vg, Ve = _data(n=60, seed=2)
    n, t = Y.shape
    p = X.shape[1]
    res = mt_solve(Y, X, np.linalg.inv(G), Vg, Ve)
    y = Y.reshape(-1, order="F")
    XX = np.kron(np.eye(t), X)
    V = np.kron(Vg, G) + np.kron(Ve, np.eye(n))
    Vi = np.linalg.inv(V)
    beta = np.linalg.solve(XX.T @ Vi @ XX, XX.T @ Vi @ y)
    u = np.kron(Vg, G) @ Vi @ (y - XX @ beta)
    np.testing.assert_allclose(res["beta"], beta, rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(res["u"], u, rtol=1e-8, atol=1e-10 * np.abs(u).max())
    assert res["beta"].shape == (p * t,)
