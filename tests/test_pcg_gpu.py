"""GPU parity tests of the MME operator and the multi-RHS PCG against the oracle.

Bar: solutions within 1e-8 relative of the oracle's FP64 PCG (the EBV parity
target); mixed precision must reach a TRUE relative residual < 1e-10.
"""
import numpy as np
import pytest

from cosmicblup_gb300 import CbxError, DeviceMME
from cosmicblup_gb300.mme import ABS, FP64, MIXED
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from oracle.grm import vanraden_grm
from oracle.mme import MME, BlockJacobi, build_fixed_design, invert_psd_matrix, matrix_free_pcg, pcg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gblup():
    n, m = 300, 2000
    bed, _ = simulate_bed(n, m, seed=1000, p_lo=0.05, miss=0.01)
    G = vanraden_grm(bed, n, m)["G"]
    Gi = invert_psd_matrix(G)
    g = genetic_values(bed, n, m, seed=1002, var_a=0.4)
    rec = simulate_gblup_records(n, 7, g, seed=1003, var_e=0.6)
    p, rows, _ = build_fixed_design(rec["cats"])
    return {"n": n, "G": G, "Gi": Gi, "rec": rec, "p": p, "rows": rows,
            "mme": MME(rec["y"], rec["aid"], rows, p, n)}


def dev_mme(handle, d):
    dm = DeviceMME(handle, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    dm.set_qinv_dense(d["Gi"])
    return dm


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def true_relres(A, x, b):
    """||b - A x|| / ||b|| in extended precision: an FP64 product with an
    eigen-bent G^-1 (every entry offset by clamp^-1 / n) carries rounding of
    order 1e-12 relative, too coarse to check a 1e-10 stop."""
    Al = A.astype(np.longdouble)
    bl = b.astype(np.longdouble)
    r = bl - Al @ x.astype(np.longdouble)
    return float(np.sqrt((r * r).sum() / (bl * bl).sum()))


def test_single_rhs_fp64_matches_oracle(handle, gblup):
    om, lam = gblup["mme"], 1.5
    A = om.lhs(gblup["Gi"], lam)
    b = om.rhs()
    x_ref, it_ref, rr_ref, _ = pcg(lambda v: A @ v, b, BlockJacobi(A, om.p), 1e-10, 10000)
    dm = dev_mme(handle, gblup)
    x, it, rr = dm.pcg_solve(lam, b)
    assert rel(x, x_ref) < 1e-8
    assert rel(x, np.linalg.solve(A, b)) < 1e-8
    assert rr[0] < 1e-10
    assert abs(int(it[0]) - it_ref) <= 2, (it, it_ref)


def test_multi_rhs_probes(handle, gblup):
    om, lam = gblup["mme"], 2.0
    A = om.lhs(gblup["Gi"], lam)
    rng = np.random.default_rng(3)
    k = 5
    B = np.zeros((om.dim, k))
    B[om.p:, :] = rng.choice([-1.0, 1.0], size=(om.q, k))
    B[:, 2] = om.rhs()
    dm = dev_mme(handle, gblup)
    X, it, rr = dm.pcg_solve(lam, B)
    Xe = np.linalg.solve(A, B)
    for c in range(k):
        assert rel(X[:, c], Xe[:, c]) < 1e-8, c
        assert rr[c] < 1e-10
    # 32 and 40 columns: one full block, and a block of 32 plus one of 8
    B2 = np.zeros((om.dim, 40))
    B2[om.p:, :] = rng.choice([-1.0, 1.0], size=(om.q, 40))
    X2, it2, rr2 = dm.pcg_solve(lam, B2)
    assert rel(X2, np.linalg.solve(A, B2)) < 1e-8
    assert np.all(rr2 < 1e-10)


def test_mixed_precision_true_residual(handle, gblup):
    """Mixed mode stops on the TRUE residual.  Forward error: 1e-8 for the data
    and probe right-hand sides; the all-ones u vector lies along the eigenvector
    that eigen-bending clamps (G^-1 eigenvalue 1e6), where any solver at relres
    1e-10 -- FP64 included -- is only accurate to cond * 1e-10, so that column
    is checked on its residual."""
    om, lam = gblup["mme"], 1.5
    A = om.lhs(gblup["Gi"], lam)
    rng = np.random.default_rng(12)
    B = np.stack([om.rhs(), np.r_[np.zeros(om.p), rng.choice([-1.0, 1.0], om.q)],
                  np.r_[np.zeros(om.p), np.ones(om.q)]], axis=1)
    dm = dev_mme(handle, gblup)
    X, it, rr = dm.pcg_solve(lam, B, precision=MIXED)
    for c in range(3):
        true = true_relres(A, X[:, c], B[:, c])
        assert true < 1e-10 and rr[c] < 1e-10
    for c in range(2):
        assert rel(X[:, c], np.linalg.solve(A, B[:, c])) < 1e-8


def test_warm_start_and_abs_tol(handle, gblup):
    om, lam = gblup["mme"], 1.5
    A = om.lhs(gblup["Gi"], lam)
    b = om.rhs()
    dm = dev_mme(handle, gblup)
    x0 = np.linalg.solve(A, b) * (1 + 1e-4)
    x, it, rr = dm.pcg_solve(lam, b, X0=x0)
    assert rel(x, np.linalg.solve(A, b)) < 1e-8
    xa, ita, rra = dm.pcg_solve(lam, b, tol=1e-8, tol_mode=ABS)
    d = np.diag(A)
    xo, ito = matrix_free_pcg(lambda v: A @ v, b, d, tol=1e-8, maxit=10000)
    assert rra[0] < 1e-8
    assert np.linalg.norm(b - A @ xa) < 1e-7


def test_qinv_apply(handle, gblup):
    dm = dev_mme(handle, gblup)
    rng = np.random.default_rng(5)
    X = rng.normal(size=(gblup["n"], 3))
    Y = dm.qinv_apply(X)
    assert rel(Y, gblup["Gi"] @ X) < 1e-12


def test_split_qinv_equals_dense(handle, gblup):
    """A sparse + S Gd S^T with a scattered genotyped map equals the dense sum."""
    om, lam = gblup["mme"], 1.2
    q = om.q
    rng = np.random.default_rng(8)
    # a sparse SPD tridiagonal "A^-1" and a dense block on a random subset
    main = 2.0 + rng.random(q)
    off = -0.4 * rng.random(q - 1)
    Adense = np.diag(main) + np.diag(off, 1) + np.diag(off, -1)
    ng = 120
    gmap = np.sort(rng.choice(q, size=ng, replace=False)).astype(np.int32)
    Wm = rng.normal(size=(ng, ng)) / np.sqrt(ng)
    Gd = Wm @ Wm.T + 0.5 * np.eye(ng)
    Q = Adense.copy()
    Q[np.ix_(gmap, gmap)] += Gd
    a_ptr = [0]
    a_col, a_val = [], []
    for i in range(q):
        for j in range(max(0, i - 1), min(q, i + 2)):
            a_col.append(j)
            a_val.append(Adense[i, j])
        a_ptr.append(len(a_col))
    dm = DeviceMME(handle, gblup["rec"]["y"], gblup["rec"]["aid"], gblup["rows"], gblup["p"], q)
    dm.set_qinv_split(np.array(a_ptr), np.array(a_col), np.array(a_val), Gd, gmap)
    A = om.lhs(Q, lam)
    b = om.rhs()
    x, it, rr = dm.pcg_solve(lam, b)
    assert rel(x, np.linalg.solve(A, b)) < 1e-8
    X = rng.normal(size=(q, 2))
    assert rel(dm.qinv_apply(X), Q @ X) < 1e-12


def test_input_errors(handle, gblup):
    y = gblup["rec"]["y"].copy()
    y[3] = np.nan
    with pytest.raises(CbxError, match="NONFINITE"):
        DeviceMME(handle, y, gblup["rec"]["aid"], gblup["rows"], gblup["p"], gblup["n"])
    dm = DeviceMME(handle, gblup["rec"]["y"], gblup["rec"]["aid"], gblup["rows"], gblup["p"], gblup["n"])
    with pytest.raises(CbxError, match="STATE"):
        dm.pcg_solve(1.0, np.ones(dm.dim))


@pytest.mark.parametrize("k", [16, 32, 33, 64])
def test_mixed_probe_block_tensor_cores(handle, gblup, k):
    """Blocks of 16 / 32 / 64 probes use the tcgen05 3xTF32 block product in the
    FP32 bulk (33 columns: a 64-wide block whose FP64-class refinement products
    run in a 32 + 1 column split)."""
    om, lam = gblup["mme"], 2.0
    A = om.lhs(gblup["Gi"], lam)
    rng = np.random.default_rng(40 + k)
    B = np.zeros((om.dim, k))
    B[om.p:, :] = rng.choice([-1.0, 1.0], size=(om.q, k))
    dm = dev_mme(handle, gblup)
    X, it, rr = dm.pcg_solve(lam, B, precision=MIXED)
    Xe = np.linalg.solve(A, B)
    for c in range(k):
        true = true_relres(A, X[:, c], B[:, c])
        assert true < 1e-10 and rr[c] < 1e-10, (c, true, rr[c])
        assert rel(X[:, c], Xe[:, c]) < 1e-8, c


@pytest.mark.parametrize("S", [16, 32, 64])
def test_dense_tc_product_accuracy(handle, S):
    """The tcgen05 3xTF32 block product alone against an FP64 product: its
    error must be at FP32 level (a few 2^-24 of sum |Q||V| per entry), far
    below what plain TF32 (2^-11) would give."""
    from cosmicblup_gb300._lib import lib, ptr
    rng = np.random.default_rng(70 + S)
    ng, ld = 1000, 3000
    Q = rng.standard_normal((ng, ld)).astype(np.float32)
    Q[:, ::7] *= 1e3                      # wide dynamic range along K
    V = rng.standard_normal((S, ld)).astype(np.float32)
    Y = np.zeros((ng, S), dtype=np.float32)
    handle.check(lib().cbx_selftest_dense_tc(handle.raw, ptr(Q), ng, ld, ptr(V), S, ptr(Y)))
    exact = Q.astype(np.float64) @ V.astype(np.float64).T
    scale = np.abs(Q).astype(np.float64) @ np.abs(V).astype(np.float64).T
    err = np.abs(Y - exact) / scale
    assert err.max() < 2e-6, err.max()


@pytest.mark.parametrize("S,rpw", [(32, 1), (32, 2), (16, 4), (1, 8)])
def test_dense_ff_product_accuracy(handle, S, rpw):
    """The float-float block product alone against an exact (integer-checked)
    reference: error within ~2^-44 of sum |Q||V| per entry, on a block with a
    large common offset (the cancellation an eigen-bent G^-1 produces)."""
    import ctypes as C
    from cosmicblup_gb300._lib import lib, ptr
    rng = np.random.default_rng(80 + S + rpw)
    ng, ld = 700, 2048
    Q = rng.standard_normal((ng, ld)) + 150.0
    V = rng.standard_normal((S, ld))
    V -= V.mean(axis=1, keepdims=True)   # strong cancellation against the offset
    Y = np.zeros((ng, S))
    ms = C.c_double(0)
    handle.check(lib().cbx_selftest_dense_ff(handle.raw, ptr(Q), ng, ld, ptr(V), S, rpw, 0, ptr(Y), C.byref(ms)))
    import math

    # exact dot products of FP64 inputs: math.fsum over exactly split products
    def xdot(a, b):
        ah = a.astype(np.float32).astype(np.float64)
        bh = b.astype(np.float32).astype(np.float64)
        parts = [ah * bh, ah * (b - bh), (a - ah) * bh, (a - ah) * (b - bh)]
        return math.fsum(np.concatenate(parts))
    rows = range(0, ng, 37)
    scale = np.abs(Q) @ np.abs(V).T
    for i in rows:
        for c in range(S):
            err = abs(Y[i, c] - xdot(Q[i], V[c])) / scale[i, c]
            assert err < 6e-14, (i, c, err)


@pytest.mark.parametrize("S,rpw,packed", [(16, 2, -2), (16, 2, -1), (32, 1, -1)])
def test_packed_ff_product_is_bit_identical(handle, S, rpw, packed):
    """The f32x2 float-float product gives the scalar kernel's bits (same per-lane
    rounding, same accumulation order), including ragged rows and a K tail."""
    import ctypes as C
    from cosmicblup_gb300._lib import lib, ptr
    rng = np.random.default_rng(90 + S)
    ng, ld = 1003, 2308
    Q = rng.standard_normal((ng, ld)) * np.exp(rng.uniform(-5, 5, (ng, ld))) + 40.0
    V = rng.standard_normal((S, ld))
    Y1, Y2 = np.zeros((ng, S)), np.zeros((ng, S))
    ms1, ms2 = C.c_double(0), C.c_double(0)
    handle.check(lib().cbx_selftest_dense_ff(handle.raw, ptr(Q), ng, ld, ptr(V), S, rpw, 3, ptr(Y1), C.byref(ms1)))
    handle.check(lib().cbx_selftest_dense_ff(handle.raw, ptr(Q), ng, ld, ptr(V), S, packed, 3, ptr(Y2), C.byref(ms2)))
    assert np.array_equal(Y1, Y2)
    print(f"S={S}: scalar rpw {rpw} {ms1.value:.4f} ms, packed rpw {-packed} {ms2.value:.4f} ms")


def test_fused_iteration_matches_separate_kernels(handle, gblup, monkeypatch):
    """The persistent cooperative PCG iteration (CBX_FUSED=1) runs the same
    per-column recurrences as the separate kernels (its sums are ordered
    differently): solutions agree to 1e-8, true relres < 1e-10."""
    om, lam = gblup["mme"], 2.0
    A = om.lhs(gblup["Gi"], lam)
    rng = np.random.default_rng(91)
    k = 33
    B = np.zeros((om.dim, k))
    B[om.p:, :] = rng.choice([-1.0, 1.0], size=(om.q, k))
    B[:, 0] = om.rhs()
    dm = dev_mme(handle, gblup)
    X0, it0, rr0 = dm.pcg_solve(lam, B, precision=MIXED)
    monkeypatch.setenv("CBX_FUSED", "1")
    dm1 = dev_mme(handle, gblup)
    X1, it1, rr1 = dm1.pcg_solve(lam, B, precision=MIXED)
    monkeypatch.delenv("CBX_FUSED")
    for c in range(k):
        assert true_relres(A, X1[:, c], B[:, c]) < 1e-10, c
        assert rel(X1[:, c], X0[:, c]) < 1e-8, c



def test_overlapped_sparse_part_matches(handle, gblup, monkeypatch):
    """The FP32 operator with its sparse part on the second stream beside the
    block product and the block term added afterwards (CBX_OVERLAP=1): the same
    operator with its sums in another order, so the solutions agree to 1e-8 and
    reach true relres < 1e-10."""
    om, lam = gblup["mme"], 2.0
    A = om.lhs(gblup["Gi"], lam)
    rng = np.random.default_rng(92)
    k = 17
    B = np.zeros((om.dim, k))
    B[om.p:, :] = rng.choice([-1.0, 1.0], size=(om.q, k))
    B[:, 0] = om.rhs()
    dm = dev_mme(handle, gblup)
    X0, _, _ = dm.pcg_solve(lam, B, precision=MIXED)
    monkeypatch.setenv("CBX_OVERLAP", "1")
    dm1 = dev_mme(handle, gblup)
    X1, _, _ = dm1.pcg_solve(lam, B, precision=MIXED)
    monkeypatch.delenv("CBX_OVERLAP")
    for c in range(k):
        assert true_relres(A, X1[:, c], B[:, c]) < 1e-10, c
        assert rel(X1[:, c], X0[:, c]) < 1e-8, c
