"""Oracle: VanRaden genomic relationship matrix from PLINK BED (test infrastructure).

Restates ``GrmBuilder::compute(const PlinkReader&)`` for the configuration the
hot path uses (src/core/grm_builder.cpp:63-405): one population, no SNP
weights, no HWE filter (``min_hwe`` defaults to 0, src/core/grm_builder.h:18),
algorithm 1 (VanRaden).  Float semantics are kept exactly:

* ``freq = sum_x / (2 n_obs)`` in double; ``maf = min(freq, 1-freq)``; a SNP
  is dropped when ``maf < (double)min_maf`` or ``|maf| < 1e-8`` (:219-224);
* ``snp_2pq = (float)(2 freq (1-freq))`` (:238-240), ``allele_freqs =
  (float)freq`` (:242), ``snp_means = (float)(2 freq)`` (:246);
* Z = (x - mean) for observed calls and 0 for missing ones, in double (:291-312);
* Sum 2pq is accumulated per ``block_size`` SNP block in double, then added to
  the running total (:267-277, :353);
* ``G = Z Z^T / sum_2pq`` (:351, :399-401).
"""
from __future__ import annotations

import numpy as np

from .plink import decode_bed, snp_counts


def snp_stats(geno_snp_major: np.ndarray, min_maf=np.float32(0.01)) -> dict:
    """Per-SNP validity, mean (f32), 2pq (f32) and allele frequency (f32)."""
    c = snp_counts(geno_snp_major)
    n_obs, sum_x = c["n_obs"], c["sum_x"]
    m = n_obs.shape[0]
    valid = np.zeros(m, dtype=bool)
    mean = np.zeros(m, dtype=np.float32)
    two_pq = np.zeros(m, dtype=np.float32)
    freq_out = np.full(m, -1.0, dtype=np.float32)
    thr = float(np.float32(min_maf))  # float promoted to double in the comparison
    with np.errstate(divide="ignore", invalid="ignore"):
        freq = sum_x.astype(np.float64) / (2.0 * n_obs.astype(np.float64))
    for j in range(m):
        if n_obs[j] == 0:
            continue
        f = float(freq[j])
        maf = min(f, 1.0 - f)
        if maf < thr or abs(maf) < 1e-8:
            continue
        two_pq[j] = np.float32(1.0 * 2.0 * f * (1.0 - f))
        freq_out[j] = np.float32(f)
        mean[j] = np.float32(f * 2.0)
        valid[j] = True
    return {"valid": valid, "mean": mean, "two_pq": two_pq, "freq": freq_out, **c}


def sum_2pq_blocked(two_pq: np.ndarray, valid: np.ndarray, block_size: int = 2048) -> float:
    """Sum 2pq exactly as the reference orders it: per block in double, then total."""
    total = 0.0
    m = two_pq.shape[0]
    for start in range(0, m, block_size):
        blk = 0.0
        for j in range(start, min(start + block_size, m)):
            if valid[j]:
                blk += float(two_pq[j])
        total += blk
    return total


def centred_z(geno_snp_major: np.ndarray, stats: dict) -> np.ndarray:
    """Z (n x n_valid) in double: x - mean if observed, 0 if missing."""
    g = geno_snp_major[stats["valid"]].astype(np.float64)
    mu = stats["mean"][stats["valid"]].astype(np.float64)[:, None]
    z = np.where(g >= 0, g - mu, 0.0)
    return np.ascontiguousarray(z.T)


def vanraden_grm(bed, n: int, m: int, min_maf=np.float32(0.01), block_size: int = 2048) -> dict:
    """FP64 VanRaden G with the reference's rounding model (BLAS GEMM order differs).

    Returns dict(G, sum2pq, n_valid, freq, stats).
    """
    geno = decode_bed(bed, n, m)
    st = snp_stats(geno, min_maf)
    s2pq = sum_2pq_blocked(st["two_pq"], st["valid"], block_size)
    z = centred_z(geno, st)
    G = z @ z.T
    if s2pq > 0:
        G = G / s2pq
    return {"G": G, "sum2pq": s2pq, "n_valid": int(st["valid"].sum()), "freq": st["freq"], "stats": st}


def xx_counts(bed, n: int, m: int) -> np.ndarray:
    """Integer cross-products X X^T over ALL SNPs, missing calls counted as 0."""
    geno = decode_bed(bed, n, m).astype(np.int64)
    x = np.where(geno >= 0, geno, 0)
    return x.T @ x


def xx_counts_valid(bed, n: int, m: int, min_maf=np.float32(0.01)) -> np.ndarray:
    """Integer cross-products X X^T over the SNPs that pass the MAF filter."""
    geno = decode_bed(bed, n, m)
    st = snp_stats(geno, min_maf)
    x = np.where(geno[st["valid"]] >= 0, geno[st["valid"]], 0).astype(np.int64)
    return x.T @ x


def vanraden_grm_exact(bed, n: int, m: int, min_maf=np.float32(0.01), block_size: int = 2048) -> dict:
    """Correctly-rounded G: Z Z^T summed exactly in integers, one rounding at the end.

    Every mean is a float >= 2^-6 (MAF >= 0.01), so mean * 2^29 is an integer
    below 2^30 and each Z entry is an integer multiple of 2^-29.  The products are
    split in 16-bit halves so that int64 sums cannot overflow; the pieces are
    recombined with Python integers.  Meant for small n and m only.
    """
    geno = decode_bed(bed, n, m)
    st = snp_stats(geno, min_maf)
    s2pq = sum_2pq_blocked(st["two_pq"], st["valid"], block_size)
    g = geno[st["valid"]].astype(np.int64)
    a = (st["mean"][st["valid"]].astype(np.float64) * 2.0**29).astype(np.int64)
    assert np.all(a.astype(np.float64) == st["mean"][st["valid"]].astype(np.float64) * 2.0**29)
    U = np.where(g >= 0, (g << 29) - a[:, None], 0)  # (n_valid, n), |U| < 2^31
    U1 = U >> 16
    U0 = U - (U1 << 16)
    hh = U1.T @ U1
    hl = U1.T @ U0
    ll = U0.T @ U0
    out = np.empty((n, n), dtype=np.float64)
    for i in range(n):
        for k in range(n):
            v = (int(hh[i, k]) << 32) + ((int(hl[i, k]) + int(hl[k, i])) << 16) + int(ll[i, k])
            out[i, k] = float(v) * 2.0**-58 if s2pq <= 0 else _div_exact(v, s2pq)
    return {"G": out, "sum2pq": s2pq, "n_valid": int(st["valid"].sum()), "freq": st["freq"], "stats": st}


def _div_exact(v: int, s2pq: float) -> float:
    """round(v * 2^-58) then divide by s2pq in double, as an FP64 GEMM result would be."""
    return (float(v) * 2.0**-58) / s2pq


def grm_tiles_exact(bed, n: int, m: int, tiles, min_maf=np.float32(0.01), block_size: int = 2048) -> dict:
    """Exact X X^T counts and correctly-rounded G on sample tiles of a large GRM.

    ``tiles`` lists (rows, cols) index arrays.  The SNP statistics (validity,
    float means, blocked sum 2pq) come from all n samples; the tiles' counts are
    exact integer sums (float64 products of small integers), and G follows
    vanraden_grm_exact: Z entries are multiples of 2^-29, summed exactly in
    16-bit halves, rounded once.  Returns dict(xx=[...], G=[...], sum2pq, n_valid).
    """
    geno = decode_bed(bed, n, m)
    st = snp_stats(geno, min_maf)
    s2pq = sum_2pq_blocked(st["two_pq"], st["valid"], block_size)
    gv = geno[st["valid"]]
    a = (st["mean"][st["valid"]].astype(np.float64) * 2.0**29).astype(np.int64)
    xx, gg = [], []
    for rows, cols in tiles:
        rows, cols = np.asarray(rows), np.asarray(cols)
        xr = np.where(gv[:, rows] >= 0, gv[:, rows], 0).astype(np.float64)
        xc = np.where(gv[:, cols] >= 0, gv[:, cols], 0).astype(np.float64)
        xx.append(np.rint(xr.T @ xc).astype(np.int64))  # exact: every partial sum < 2^53

        def u(idx):
            g = gv[:, idx].astype(np.int64)
            return np.where(g >= 0, (g << 29) - a[:, None], 0)

        Ur, Uc = u(rows), u(cols)
        Ur1, Uc1 = Ur >> 16, Uc >> 16
        Ur0, Uc0 = Ur - (Ur1 << 16), Uc - (Uc1 << 16)
        hh, hl, lh, ll = Ur1.T @ Uc1, Ur1.T @ Uc0, Ur0.T @ Uc1, Ur0.T @ Uc0
        G = np.empty((rows.size, cols.size))
        for i in range(rows.size):
            for k in range(cols.size):
                v = (int(hh[i, k]) << 32) + ((int(hl[i, k]) + int(lh[i, k])) << 16) + int(ll[i, k])
                G[i, k] = float(v) * 2.0**-58 if s2pq <= 0 else _div_exact(v, s2pq)
        gg.append(G)
    return {"xx": xx, "G": gg, "sum2pq": s2pq, "n_valid": int(st["valid"].sum())}
