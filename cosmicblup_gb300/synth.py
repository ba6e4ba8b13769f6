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


def _bed_chunk(n: int, p: np.ndarray, miss: float, seed) -> bytes:
    """SNP-major BED payload for the SNPs with frequencies p (one uint16 draw per call)."""
    rng = np.random.default_rng(seed)
    k = p.shape[0]
    scale = 65536.0
    tm = np.uint32(round(miss * scale))
    q2 = (1.0 - miss) * scale
    t2 = (tm + np.round(q2 * p * p)).astype(np.uint32)[:, None]                 # two copies
    t1 = (t2[:, 0] + np.round(q2 * 2 * p * (1 - p))).astype(np.uint32)[:, None]  # one copy
    bps = (n + 3) // 4
    u = rng.integers(0, 65536, size=(k, bps * 4), dtype=np.uint16).astype(np.uint32)
    # code: 01 missing, 00 two copies, 10 one copy, 11 none
    code = ((u < tm).astype(np.uint8) + 2 * ((u >= t2) & (u < t1)).astype(np.uint8)
            + 3 * (u >= t1).astype(np.uint8))
    code[:, n:] = 0  # PLINK pads unused slots with 00
    c = code.reshape(k, bps, 4)
    packed = c[:, :, 0] | (c[:, :, 1] << 2) | (c[:, :, 2] << 4) | (c[:, :, 3] << 6)
    return packed.astype(np.uint8).tobytes()


def simulate_bed(n: int, m: int, seed: int, p_lo: float = 0.05, miss: float = 0.01,
                 chunk: int = 1024, threads: int | None = None) -> tuple[bytes, np.ndarray]:
    """Return (bed_bytes, p) for n samples and m SNPs.

    Chunks of SNPs are generated in parallel threads from independent child
    seeds of ``seed``, so the result depends only on (n, m, seed, p_lo, miss, chunk).
    """
    import concurrent.futures as cf
    import os
    ss = np.random.SeedSequence(seed)
    p_seed, *chunk_seeds = ss.spawn(1 + (m + chunk - 1) // chunk)
    p = np.random.default_rng(p_seed).uniform(p_lo, 0.5, size=m)
    starts = list(range(0, m, chunk))
    threads = threads or min(16, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        parts = list(ex.map(lambda a: _bed_chunk(n, p[a[1]:a[1] + chunk], miss, a[0]),
                            zip(chunk_seeds, starts)))
    return BED_MAGIC + b"".join(parts), p


def _g_chunk(payload, n, bps, s, e, w):
    lut = np.array([2.0, np.nan, 1.0, 0.0])
    blk = payload[s * bps:e * bps].reshape(e - s, bps)
    codes = np.stack([(blk >> (2 * k)) & 3 for k in range(4)], axis=2).reshape(e - s, bps * 4)[:, :n]
    x = lut[codes]
    obs = ~np.isnan(x)
    cnt = np.maximum(obs.sum(axis=1), 1)
    mu = np.where(obs, x, 0).sum(axis=1) / cnt
    pf = mu / 2
    z = np.where(obs, x - mu[:, None], 0.0)
    return w @ z, float((2 * pf * (1 - pf)).sum())


def genetic_values(bed: bytes, n: int, m: int, seed: int, var_a: float,
                   chunk: int = 1024, threads: int | None = None) -> np.ndarray:
    """g = Z w / sqrt(sum 2pq) with w ~ N(0, var_a); Z centred at the observed 2p."""
    import concurrent.futures as cf
    import os
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, np.sqrt(var_a), size=m)
    bps = (n + 3) // 4
    payload = np.frombuffer(bed, dtype=np.uint8, offset=3)
    threads = threads or min(16, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(lambda s: _g_chunk(payload, n, bps, s, min(s + chunk, m), w[s:min(s + chunk, m)]),
                          range(0, m, chunk)))
    g = np.zeros(n)
    s2pq = 0.0
    for gv, sp in res:
        g += gv
        s2pq += sp
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


def simulate_bed_gene_drop(sire: np.ndarray, dam: np.ndarray, per_gen: int, m: int, seed: int,
                           p_lo: float = 0.01, miss: float = 0.02, chunk: int = 4096,
                           threads: int | None = None) -> tuple[bytes, np.ndarray]:
    """Genotypes of a pedigree's last generation by gene dropping.

    The pedigree lists ``per_gen`` animals per discrete generation, founders
    first, every known parent in the previous generation (simulate_pedigree).
    Per SNP a base frequency p ~ U(p_lo, 0.5) of the counted allele; founder
    haplotypes and the haplotype passed by an unknown parent are drawn from
    it, and each known parent passes one of its two alleles with probability
    1/2, independently per SNP (no linkage).  Only the last generation is
    kept; each of its calls is then set missing with probability ``miss``.
    Returns (bed_bytes, p) with samples in pedigree order.  Chunks of SNPs are
    independent (child seeds of ``seed``) and run in parallel threads, so the
    result depends only on the arguments."""
    import concurrent.futures as cf
    import os
    sire = np.asarray(sire, dtype=np.int64)
    dam = np.asarray(dam, dtype=np.int64)
    n_all = sire.size
    n_gen = n_all // per_gen
    assert n_gen * per_gen == n_all, "pedigree size must be a whole number of generations"
    for gen in range(1, n_gen):
        lo, prev = gen * per_gen, (gen - 1) * per_gen
        for par in (sire[lo:lo + per_gen], dam[lo:lo + per_gen]):
            k = par[par >= 0]
            assert np.all((k >= prev) & (k < lo)), "parents must come from the previous generation"
    ss = np.random.SeedSequence(seed)
    p_seed, *chunk_seeds = ss.spawn(1 + (m + chunk - 1) // chunk)
    p = np.random.default_rng(p_seed).uniform(p_lo, 0.5, size=m)
    tmiss = np.uint16(round(miss * 65536))

    def drop(arg):
        cs, j0 = arg
        k = min(m, j0 + chunk) - j0
        kb = (k + 7) // 8
        rng = np.random.default_rng(cs)
        thr = np.round(p[j0:j0 + k] * 65536.0).astype(np.uint32)

        def fresh(rows):  # haplotypes from the base frequencies, bit-packed per SNP
            u = rng.integers(0, 65536, size=(rows, k), dtype=np.uint16)
            return np.packbits(u < thr, axis=1, bitorder="little")

        hA, hB = fresh(per_gen), fresh(per_gen)
        for gen in range(1, n_gen):
            lo, prev = gen * per_gen, (gen - 1) * per_gen

            def gamete(par):
                known = par >= 0
                idx = np.where(known, par - prev, 0)
                mask = rng.integers(0, 256, size=(per_gen, kb), dtype=np.uint8)
                g = (hA[idx] & mask) | (hB[idx] & ~mask)
                nu = int((~known).sum())
                if nu:
                    g[~known] = fresh(nu)
                return g

            hA, hB = gamete(sire[lo:lo + per_gen]), gamete(dam[lo:lo + per_gen])
        x = (np.unpackbits(hA, axis=1, count=k, bitorder="little")
             + np.unpackbits(hB, axis=1, count=k, bitorder="little"))
        g = np.ascontiguousarray(x.T).astype(np.int8)
        g[rng.integers(0, 65536, size=(k, per_gen), dtype=np.uint16) < tmiss] = -1
        return encode_bed(g)[len(BED_MAGIC):]

    starts = list(range(0, m, chunk))
    threads = threads or min(16, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        parts = list(ex.map(drop, zip(chunk_seeds, starts)))
    return BED_MAGIC + b"".join(parts), p


def simulate_mt_records(bed: bytes, n: int, m: int, seed: int, Vg: np.ndarray, Ve: np.ndarray,
                        n_levels: int = 2) -> dict:
    """Multi-trait records y_i = mu + level effect + g_i + e_i (one row per animal).

    g = [g_1 .. g_t] L_g' with g_k independent genetic values of variance 1
    (Cov(vec g) = Vg (x) G), e_i ~ N(0, Ve); a 2-level class (sex) plus the mean
    as fixed effects.  Returns Y (n x t) and the dense design X (n x (1 + levels - 1)).
    """
    Vg, Ve = np.asarray(Vg, dtype=np.float64), np.asarray(Ve, dtype=np.float64)
    t = Vg.shape[0]
    rng = np.random.default_rng(seed)
    g0 = np.stack([genetic_values(bed, n, m, seed=seed * 1000 + k + 1, var_a=1.0) for k in range(t)], axis=1)
    g = g0 @ np.linalg.cholesky(Vg).T
    e = rng.standard_normal((n, t)) @ np.linalg.cholesky(Ve).T
    lvl = rng.integers(0, n_levels, size=n)
    eff = rng.normal(0.0, 1.0, size=(n_levels, t))
    Y = 10.0 + eff[lvl] + g + e
    X = np.zeros((n, n_levels))
    X[:, 0] = 1.0
    for k in range(1, n_levels):
        X[lvl == k, k] = 1.0
    return {"Y": Y, "X": X, "level": lvl}


def pedigree_breeding_values(sire: np.ndarray, dam: np.ndarray, var_a: float, seed: int) -> np.ndarray:
    """Breeding values down a pedigree listed parents first:
    a_i = (a_sire + a_dam) / 2 + m_i, m_i ~ N(0, d_i var_a) with the Mendelian
    sampling fraction d_i = 1/2, 3/4 or 1 for two, one or no known parents
    (inbreeding ignored).  Unknown parents contribute 0."""
    rng = np.random.default_rng(seed)
    n = sire.size
    known = (sire >= 0).astype(np.int64) + (dam >= 0).astype(np.int64)
    d = np.where(known == 2, 0.5, np.where(known == 1, 0.75, 1.0))
    m = rng.normal(0.0, 1.0, size=n) * np.sqrt(d * var_a)
    a = np.zeros(n)
    for i in range(n):
        pa = (a[sire[i]] if sire[i] >= 0 else 0.0) + (a[dam[i]] if dam[i] >= 0 else 0.0)
        a[i] = 0.5 * pa + m[i]
    return a

