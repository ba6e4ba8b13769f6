"""Oracle: PLINK BED decoding and per-SNP statistics (test infrastructure).

Restates the 2-bit lookup of ``PlinkReader`` (src/core/plink_reader.cpp:17-20):
code 00 -> 2 copies of the first .bim allele, 01 -> missing, 10 -> 1, 11 -> 0,
four samples per byte, least-significant bit pair first, SNP-major payload after
the 3-byte magic ``6C 1B 01`` (src/core/plink_reader.cpp:66-91).
"""
from __future__ import annotations

import numpy as np

BED_MAGIC = bytes([0x6C, 0x1B, 0x01])

# code -> genotype (copies of allele 1); -1 marks a missing call.
CODE_TO_GENO = np.array([2, -1, 1, 0], dtype=np.int8)


def bytes_per_snp(n: int) -> int:
    """ceil(n/4), src/core/plink_reader.cpp:83."""
    return (n + 3) // 4


def check_bed(bed: bytes | np.ndarray, n: int, m: int) -> np.ndarray:
    """Validate magic + size like PlinkReader::openBed and return the payload."""
    buf = np.frombuffer(bed, dtype=np.uint8) if not isinstance(bed, np.ndarray) else bed
    if buf.size < 3:
        raise ValueError("Invalid .bed file (too small)")
    if buf[0] != 0x6C or buf[1] != 0x1B:
        raise ValueError("Invalid .bed file magic number")
    if buf[2] != 0x01:
        raise ValueError("Only SNP-major mode (0x01) .bed files are supported")
    bps = bytes_per_snp(n)
    if buf.size < 3 + m * bps:
        raise ValueError("Truncated .bed file")
    return buf[3:3 + m * bps]


def decode_bed(bed: bytes | np.ndarray, n: int, m: int, snp_lo: int = 0,
               snp_hi: int | None = None) -> np.ndarray:
    """Decode SNPs [snp_lo, snp_hi) into an (n_snp, n) int8 array, -1 = missing."""
    payload = check_bed(bed, n, m)
    bps = bytes_per_snp(n)
    snp_hi = m if snp_hi is None else snp_hi
    blk = payload[snp_lo * bps:snp_hi * bps].reshape(snp_hi - snp_lo, bps)
    codes = np.empty((snp_hi - snp_lo, bps, 4), dtype=np.uint8)
    for k in range(4):
        codes[:, :, k] = (blk >> (2 * k)) & 3
    codes = codes.reshape(snp_hi - snp_lo, bps * 4)[:, :n]
    return CODE_TO_GENO[codes]


def snp_counts(geno_snp_major: np.ndarray) -> dict:
    """Integer per-SNP tallies of the stats pass (src/core/grm_builder.cpp:191-217).

    Returns n_obs, sum_x, n_hom1 (code 00), n_het (code 10), n_hom2 (code 11),
    all int64 arrays of length m.
    """
    g = geno_snp_major
    obs = g >= 0
    return {
        "n_obs": obs.sum(axis=1, dtype=np.int64),
        "sum_x": np.where(obs, g, 0).sum(axis=1, dtype=np.int64),
        "n_hom1": (g == 2).sum(axis=1, dtype=np.int64),
        "n_het": (g == 1).sum(axis=1, dtype=np.int64),
        "n_hom2": (g == 0).sum(axis=1, dtype=np.int64),
    }
