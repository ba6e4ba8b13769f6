"""CPU tests of the genotype-product oracle (oracle/geno.py) against a loop-for-loop
restatement of the reference's PlinkReader code, on the reference's toy fixture and
small random BEDs."""
import math

import numpy as np

from cosmicblup_gb300.synth import encode_bed, simulate_bed
from oracle.geno import (compute_stats, multiply_z_v, multiply_zt_v, multiply_zt_v_c, snp_effects, total_2pq,
                         val_maps)
from oracle.plink import decode_bed

LUT = {0: 2.0, 2: 1.0, 3: 0.0}  # PlinkReader::lookup_table (plink_reader.cpp:17-20), 1 = missing


def codes(bed: bytes, n: int, m: int):
    """Byte-walk of the payload as PlinkReader does it: codes[j][i]."""
    bps = (n + 3) // 4
    out = []
    for j in range(m):
        row = bed[3 + j * bps: 3 + (j + 1) * bps]
        out.append([(row[i // 4] >> (2 * (i % 4))) & 3 for i in range(n)])
    return out


def loop_stats(cs):
    """plink_reader.cpp:192-236, one SNP at a time."""
    means, inv = [], []
    for col in cs:
        s, count = 0.0, 0
        for c in col:
            if c != 1:
                s += LUT[c]
                count += 1
        if count > 0:
            mean = s / count
            p = mean / 2.0
            var = 2.0 * p * (1.0 - p)
            means.append(mean)
            inv.append(0.0 if var < 1e-9 else 1.0 / math.sqrt(var))
        else:
            means.append(0.0)
            inv.append(0.0)
    return np.array(means), np.array(inv)


def loop_zt(cs, means, inv, v):
    """plink_reader.cpp:341-392, sequential FP64 sums."""
    y = []
    for j, col in enumerate(cs):
        if inv[j] == 0.0:
            y.append(0.0)
            continue
        sxv = svo = 0.0
        for i, c in enumerate(col):
            if c != 1:
                sxv += LUT[c] * v[i]
                svo += v[i]
        y.append((sxv - means[j] * svo) * inv[j])
    return np.array(y)


def loop_z(cs, means, inv, v, n):
    """plink_reader.cpp:239-293 with float val_map, sequential FP64 sums."""
    y = [0.0] * n
    for j, col in enumerate(cs):
        if inv[j] == 0.0:
            continue
        w = v[j] * inv[j]
        vm = {0: float(np.float32((2.0 - means[j]) * w)), 1: 0.0,
              2: float(np.float32((1.0 - means[j]) * w)), 3: float(np.float32((0.0 - means[j]) * w))}
        for i, c in enumerate(col):
            y[i] += vm[c]
    return np.array(y)


def small_case(n, m, seed):
    bed, _ = simulate_bed(n, m, seed=seed, miss=0.1)
    g = decode_bed(bed, n, m).copy()
    g[0, :] = 1           # monomorphic SNP: inv_std = 0
    g[1, :] = -1          # nothing observed
    if m > 2:
        g[2, : n // 2] = -1
    return encode_bed(g), g


def test_stats_bit_exact_vs_loop(toy_golden):
    for bed, n, m in [(bytes.fromhex(toy_golden["bed_hex"]), 6, 4), (*small_case(37, 11, 3)[:1], 37, 11)]:
        g = decode_bed(bed, n, m)
        mean, inv = compute_stats(g)
        lm, li = loop_stats(codes(bed, n, m))
        np.testing.assert_array_equal(mean, lm)
        np.testing.assert_array_equal(inv, li)


def test_toy_stats_known_answer(toy_golden):
    # toy.bed genotypes (the reference's own fixture): SNP means straight from the calls
    g = np.array(toy_golden["genotypes_snp_major"])
    mean, inv = compute_stats(g.astype(np.int8))
    for j in range(g.shape[0]):
        obs = g[j][g[j] >= 0]
        assert mean[j] == obs.sum() / obs.size
        p = mean[j] / 2.0
        assert inv[j] == 1.0 / math.sqrt(2.0 * p * (1.0 - p))


def test_products_vs_loop():
    n, m = 37, 11
    bed, g = small_case(n, m, 4)
    cs = codes(bed, n, m)
    mean, inv = compute_stats(g)
    rng = np.random.default_rng(9)
    v = rng.standard_normal(n)
    ref = loop_zt(cs, mean, inv, v)
    got = multiply_zt_v(g, mean, inv, v)
    tol = 1e-13 * np.abs(v).sum() * (2 + mean) * inv + 1e-300
    assert np.all(np.abs(got - ref) <= tol)
    u = rng.standard_normal(m)
    ref = loop_z(cs, mean, inv, u, n)
    got = multiply_z_v(g, mean, inv, u)
    scale = np.abs(val_maps(mean, inv, u)).max(axis=1).sum()
    assert np.abs(got - ref).max() <= 1e-13 * scale


def test_zt_of_ones_vanishes():
    # sum_obs x - mean * n_obs = 0 for every SNP: Z^T 1 = 0 up to rounding
    n, m = 203, 17
    bed, g = small_case(n, m, 5)
    mean, inv = compute_stats(g)
    y = multiply_zt_v(g, mean, inv, np.ones(n))
    assert np.abs(y).max() <= 1e-12 * n * inv.max()


def test_snp_effects_formula():
    n, m = 41, 13
    bed, g = small_case(n, m, 6)
    rng = np.random.default_rng(2)
    A = rng.standard_normal((n, n))
    Ginv = A @ A.T / n + np.eye(n)
    u = rng.standard_normal(n)
    eff, freq, t2 = snp_effects(g, Ginv, u)
    mean, inv = compute_stats(g)
    assert t2 == total_2pq(mean)
    np.testing.assert_array_equal(freq, mean / 2.0)
    assert eff[0] == 0.0 and eff[1] == 0.0  # monomorphic / unobserved SNPs
    q = Ginv @ u
    ref = loop_zt(codes(bed, n, m), mean, inv, q)
    ok = inv > 0
    np.testing.assert_allclose(eff[ok], ref[ok] / inv[ok] / t2, rtol=1e-12, atol=1e-14)


def test_c_restatement_matches_loop():
    # the C restatement follows the reference's per-SNP sample order: the loop
    # restatement above gives the same bits
    n, m = 203, 29
    bed, g = small_case(n, m, 11)
    mean, inv = compute_stats(g)
    v = np.random.default_rng(12).standard_normal(n)
    ref = loop_zt(codes(bed, n, m), mean, inv, v)
    for threads in (1, 3):
        assert np.array_equal(multiply_zt_v_c(bed, n, m, mean, inv, v, threads=threads), ref)
    assert np.array_equal(multiply_zt_v_c(bed, n, m, mean, inv, v, threads=2, j0=5, j1=20), ref[5:20])

