"""GPU parity tests of the genotype matrix-free products (cbx_geno_*, cbx_snp_effects)
against the oracle (oracle/geno.py).

Bar: per-SNP means and inv_stds bit-exact (the same IEEE operations as
PlinkReader::computeStats).  Z^T v: the device sums are exact in 64-bit fixed point
after one rounding of each input below 2^-62 sum|v|, so it may differ from the oracle's
FP64 sums only by their rounding: |dy_j| <= 1e-13 (2 + mean_j) sum|v| inv_std_j.  Z v:
the float-rounded terms are summed exactly, |dy_i| <= 1e-13 sum_j max_c |w_cj|.
"""
import numpy as np
import pytest

from cosmicblup_gb300 import CbxError, DeviceGenotypes, GrmBuilder, GrmOptions, PlinkReader, invert_psd
from cosmicblup_gb300.synth import encode_bed, simulate_bed
from oracle.geno import compute_stats, multiply_z_v, multiply_zt_v, snp_effects, val_maps
from oracle.plink import decode_bed

pytestmark = pytest.mark.gpu


def case(n, m, seed, miss=0.05):
    bed, _ = simulate_bed(n, m, seed=seed, miss=miss)
    g = decode_bed(bed, n, m).copy()
    g[0, :] = 1            # monomorphic: inv_std = 0
    g[1, :] = -1           # nothing observed
    g[2, : n // 2] = -1
    g[3, :] = 2
    g[3, 0] = 1            # nearly monomorphic
    return encode_bed(g), g


def zt_tol(v, mean, inv):
    return 1e-13 * np.abs(v).sum(axis=0) * ((2 + mean) * inv)[:, None] + 1e-300


def z_tol(u, mean, inv):
    return 1e-13 * np.abs(val_maps(mean, inv, u)).max(axis=1).astype(np.float64).sum() + 1e-300


def test_stats_bit_exact_toy(handle, toy_golden):
    bed = bytes.fromhex(toy_golden["bed_hex"])
    d = DeviceGenotypes(bed, 6, 4, handle)
    mean, inv = compute_stats(decode_bed(bed, 6, 4))
    np.testing.assert_array_equal(d.getMeans(), mean)
    np.testing.assert_array_equal(d.getInvStds(), inv)


@pytest.mark.parametrize("n,m", [(1, 5), (7, 9), (17, 33), (1003, 257), (4099, 1500)])
def test_products_vs_oracle(handle, n, m):
    bed, g = case(n, m, seed=n + m) if n >= 4 else (simulate_bed(n, m, seed=1)[0], None)
    g = decode_bed(bed, n, m) if g is None else g
    d = DeviceGenotypes(bed, n, m, handle)
    mean, inv = compute_stats(g)
    np.testing.assert_array_equal(d.getMeans(), mean)
    np.testing.assert_array_equal(d.getInvStds(), inv)
    rng = np.random.default_rng(n * 7 + m)
    V = rng.standard_normal((n, 3)) * np.exp(rng.uniform(-8, 4, (n, 3)))
    Y = d.multiply_Zt_v(V)
    for c in range(3):
        ref = multiply_zt_v(g, mean, inv, V[:, c])
        assert np.all(np.abs(Y[:, c] - ref) <= zt_tol(V[:, c:c + 1], mean, inv)[:, 0])
    U = rng.standard_normal((m, 2))
    X = d.multiply_Z_v(U)
    for c in range(2):
        ref = multiply_z_v(g, mean, inv, U[:, c])
        assert np.abs(X[:, c] - ref).max() <= z_tol(U[:, c], mean, inv)


def test_deterministic_and_edge_vectors(handle):
    n, m = 2053, 301
    bed, g = case(n, m, seed=17)
    d = DeviceGenotypes(bed, n, m, handle)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(n)
    a, b = d.multiply_Zt_v(v), d.multiply_Zt_v(v)
    assert np.array_equal(a, b)
    u = rng.standard_normal(m)
    assert np.array_equal(d.multiply_Z_v(u), d.multiply_Z_v(u))
    assert not np.any(d.multiply_Zt_v(np.zeros(n)))
    assert not np.any(d.multiply_Z_v(np.zeros(m)))
    # Z^T 1 = 0: sum_obs x = mean * n_obs for every SNP
    assert np.abs(d.multiply_Zt_v(np.ones(n))).max() <= 1e-12 * n * d.getInvStds().max()
    # huge dynamic range: tiny entries round into the fixed point, within the bound
    w = v * np.exp(rng.uniform(-300, 300, n))
    mean, inv = compute_stats(g)
    ref = multiply_zt_v(g, mean, inv, w)
    assert np.all(np.abs(d.multiply_Zt_v(w) - ref) <= zt_tol(w[:, None], mean, inv)[:, 0])
    bad = v.copy()
    bad[5] = np.nan
    with pytest.raises(CbxError) as e:
        d.multiply_Zt_v(bad)
    assert e.value.code == 6
    with pytest.raises(ValueError):
        d.multiply_Z_v(v)  # wrong length
    # the handle stays usable after the error
    assert np.array_equal(d.multiply_Zt_v(v), a)


def test_attach_rejects_bad_bytes(handle):
    bed, _ = simulate_bed(10, 4, seed=2)
    with pytest.raises(CbxError) as e:
        DeviceGenotypes(b"\x6c\x1b\x00" + bed[3:], 10, 4, handle)
    assert e.value.code == 3
    with pytest.raises(CbxError) as e:
        DeviceGenotypes(bed[:-1], 10, 4, handle)
    assert e.value.code == 3


def test_reader_methods_mirror_reference(handle):
    n, m = 517, 140
    bed, g = case(n, m, seed=23)
    r = PlinkReader.from_bytes(bed, n, m)
    r.computeStats(handle)
    mean, inv = compute_stats(g)
    np.testing.assert_array_equal(r.getMeans(), mean)
    v = np.linspace(-1, 1, n)
    assert np.all(np.abs(r.multiply_Zt_v(v) - multiply_zt_v(g, mean, inv, v)) <= zt_tol(v[:, None], mean, inv)[:, 0])


def test_snp_effects_vs_oracle(handle):
    n, m = 611, 900
    bed, g = case(n, m, seed=29)
    rng = np.random.default_rng(4)
    A = rng.standard_normal((n, n))
    Ginv = A @ A.T / n + np.eye(n)
    u = rng.standard_normal(n)
    d = DeviceGenotypes(bed, n, m, handle)
    eff, freq, t2 = d.snp_effects(u, Ginv)
    re, rf, rt2 = snp_effects(g, Ginv, u)
    assert abs(t2 - rt2) <= 1e-13 * rt2
    np.testing.assert_array_equal(freq, rf)
    mean, inv = compute_stats(g)
    q = Ginv @ u
    # effect = (Z^T q)_j / inv_std_j / t2: the bound of Z^T q divided through, plus the G^-1 product
    tol = (1e-13 * np.abs(q).sum() * (2 + mean) + 1e-12 * np.abs(re)) / rt2 + 1e-300
    assert np.all(np.abs(eff - re) <= tol)
    assert eff[0] == 0.0 and eff[1] == 0.0


def test_snp_effects_with_device_inverse(handle):
    # the workflow of the result writer: GRM -> G^-1 on the device -> back-solve
    n, m = 300, 2000
    bed, _ = simulate_bed(n, m, seed=31, p_lo=0.05)
    g = decode_bed(bed, n, m)
    b = GrmBuilder(GrmOptions(), handle=handle)
    b.compute(PlinkReader.from_bytes(bed, n, m))
    Gi = invert_psd(handle, None, n)
    u = np.random.default_rng(5).standard_normal(n)
    d = DeviceGenotypes(bed, n, m, handle)
    eff, _, t2 = d.snp_effects(u)
    re, _, rt2 = snp_effects(g, Gi, u)
    # Z^T q cancels the eigen-bent G^-1's large component of q (Z^T 1 = 0): the
    # bound scales with the FP64 rounding of q = G^-1 u
    mean, _ = compute_stats(g)
    qbound = 1e-12 * (np.abs(Gi) @ np.abs(u)).sum()
    assert np.all(np.abs(eff - re) <= (2 + mean) * qbound / rt2 + 1e-300)
    with pytest.raises(CbxError) as e:
        d.snp_effects(np.ones(n - 1))
    assert e.value.code == 1


def test_large_properties(handle):
    # size-independent properties at a production-like shape
    n, m = 8192, 16384
    bed, _ = simulate_bed(n, m, seed=41, miss=0.02)
    d = DeviceGenotypes(bed, n, m, handle)
    rng = np.random.default_rng(8)
    v1, v2 = rng.standard_normal(n), rng.standard_normal(n)
    y1, y2 = d.multiply_Zt_v(v1), d.multiply_Zt_v(v2)
    y3 = d.multiply_Zt_v(2.0 * v1 + v2)
    inv = d.getInvStds()
    bound = 1e-13 * (np.abs(v1).sum() * 3 + np.abs(v2).sum()) * 4 * inv + 1e-300
    assert np.all(np.abs(y3 - (2.0 * y1 + y2)) <= bound)
    assert np.abs(d.multiply_Zt_v(np.ones(n))).max() <= 1e-12 * n * inv.max()
    # adjoint identity u.(Z w) = (Z^T u).w, up to the float rounding of Z w's terms
    w = rng.standard_normal(m)
    lhs = v1 @ d.multiply_Z_v(w)
    rhs = y1 @ w
    assert abs(lhs - rhs) <= 1e-6 * np.abs(v1).sum() * np.abs(w).max() * 4
