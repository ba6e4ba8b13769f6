"""Seeded synthetic inputs with the shapes of the GBLUP/ssGBLUP workloads.

No public dataset is involved: genotypes, pedigrees and phenotypes are drawn
from documented generators so that benchmarks and parity tests are
reproducible.

* Genotypes: per SNP an allele frequency p ~ U(p_lo, 0.5); each call is
  Binomial(2, p) copies of the first ``.bim`` allele (HWE); each call is set
  missing independently with probability ``miss``.  Written SNP-major with the
  PLINK 2-bit code (00 = two copies, 01 = missing, 10 = one, 11 = none).
* Phenotypes: y = mu + fixed-class effect + g + e with g = Z w / sqrt(sum 2pq),
  w ~ N(0, var_a), e ~ N(0, var_e), Z the centred genotype matrix.
* Pedigree (ssGBLUP): discrete generations, founders first, parents drawn from
  the previous generation's sires and dams, each parent unknown w.p. 0.05.
"""
from __future__ import annotations

import numpy as np

BED_MAGIC = bytes([0x6C, 0x1B, 0x01])
_GENO_TO_CODE = np.array([3, 2, 0], dtype=np.uint8)  # 0 copies->11, 1->10, 2->00


def encode_bed(geno_snp_major: np.ndarray) -> bytes:
    """Pack an (m, n) int8 genotype array (-1 = missing) into BED bytes."""
    m, n = geno_snp_major.shape
    bps = (n + 3) // 4
    codes = np.zeros((m, bps * 4), dtype=np.uint8)  # PLINK pads unused slots with 00
    g = geno_snp_major
    codes[:, :n] = np.where(g < 0, 1, _GENO_TO_CODE[np.clip(g, 0, 2)])
    c = codes.reshape(m, bps, 4)
    packed = c[:, :, 0] | (c[:, :, 1] << 2) | (c[:, :, 2] << 4) | (c[:, :, 3] << 6)
    return BED_MAGIC + packed.astype(np.uint8).tobytes()


def simulate_bed(n: int, m: int, seed: int, p_lo: float = 0.05, miss: float = 0.01,
                 chunk: int = 4096) -> tuple[bytes, np.ndarray]:
    """Return (bed_bytes, p) for n samples and m SNPs, generated in SNP chunks."""
    rng = np.random.default_rng(seed)
    p = rng.uniform(p_lo, 0.5, size=m)
    parts = [BED_MAGIC]
    for s in range(0, m, chunk):
        e = min(s + chunk, m)
        g = rng.binomial(2, p[s:e, None], size=(e - s, n)).astype(np.int8)
        if miss > 0:
            g[rng.random((e - s, n)) < miss] = -1
        parts.append(encode_bed(g)[3:])
    return b"".join(parts), p


def genetic_values(bed: bytes, n: int, m: int, seed: int, var_a: float,
                   chunk: int = 2048) -> np.ndarray:
    """g = Z w / sqrt(sum 2pq) with w ~ N(0, var_a); Z centred at the observed 2p."""
    rng = np.random.default_rng(seed)
    bps = (n + 3) // 4
    payload = np.frombuffer(bed, dtype=np.uint8, offset=3)
    lut = np.array([2.0, np.nan, 1.0, 0.0])
    g = np.zeros(n)
    s2pq = 0.0
    for s in range(0, m, chunk):
        e = min(s + chunk, m)
        blk = payload[s * bps:e * bps].reshape(e - s, bps)
        codes = np.stack([(blk >> (2 * k)) & 3 for k in range(4)], axis=2).reshape(e - s, bps * 4)[:, :n]
        x = lut[codes]
        obs = ~np.isnan(x)
        cnt = np.maximum(obs.sum(axis=1), 1)
        mu = np.where(obs, x, 0).sum(axis=1) / cnt
        pf = mu / 2
        s2pq += float((2 * pf * (1 - pf)).sum())
        z = np.where(obs, x - mu[:, None], 0.0)
        w = rng.normal(0.0, np.sqrt(var_a), size=e - s)
        g += w @ z
    return g / np.sqrt(max(s2pq, 1e-12))


def simulate_gblup_records(n: int, n_levels: int, g: np.ndarray, seed: int, var_e: float,
                           mu: float = 10.0) -> dict:
    """One record per animal: y = mu + class effect + g + e.  Levels are strings."""
    rng = np.random.default_rng(seed)
    lvl = rng.integers(0, n_levels, size=n)
    eff = rng.normal(0.0, 1.0, size=n_levels)
    y = mu + eff[lvl] + g + rng.normal(0.0, np.sqrt(var_e), size=n)
    return {"y": y, "aid": np.arange(1, n + 1, dtype=np.int32),
            "cats": [[f"L{int(v):04d}"] for v in lvl]}


def simulate_pedigree(n_gen: int, per_gen: int, n_sires: int, n_dams: int, seed: int,
                      p_unknown: float = 0.05) -> tuple[np.ndarray, np.ndarray]:
    """Return (sire, dam) arrays, 0-based parent index or -1, founders first."""
    rng = np.random.default_rng(seed)
    n = n_gen * per_gen
    sire = np.full(n, -1, dtype=np.int64)
    dam = np.full(n, -1, dtype=np.int64)
    for gen in range(1, n_gen):
        lo = gen * per_gen
        prev = (gen - 1) * per_gen
        ns = min(n_sires, per_gen)
        nd = min(n_dams, per_gen - ns)
        sires = prev + rng.choice(per_gen, size=ns, replace=False)
        pool = np.setdiff1d(np.arange(prev, prev + per_gen), sires)
        dams = rng.choice(pool, size=nd, replace=False)
        s = rng.choice(sires, size=per_gen)
        d = rng.choice(dams, size=per_gen)
        s[rng.random(per_gen) < p_unknown] = -1
        d[rng.random(per_gen) < p_unknown] = -1
        sire[lo:lo + per_gen] = s
        dam[lo:lo + per_gen] = d
    return sire, dam
