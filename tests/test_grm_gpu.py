"""GPU parity tests of the GRM path (cbx_bed_snp_counts, cbx_grm_bed) against the oracle.

Bar: integer cross-products and SNP tallies bit-exact.  G: the GPU forms X X^T
and the centring term exactly and the mu^2 term from mu_j^2 rounded to a
multiple of 2^-45, then rounds once; so |G - G_exact| <= n_valid 2^-46 / sum2pq
+ 4 ulp, and G is within 1e-13 * max|G| of the oracle's FP64 GEMM (the
reference's rounding model).
"""
import ctypes as C

import numpy as np
import pytest

from cosmicblup_gb300 import CbxError, GrmBuilder, GrmOptions, PlinkReader, bed_snp_counts
from cosmicblup_gb300._lib import lib, ptr
from cosmicblup_gb300.synth import encode_bed, simulate_bed
from oracle.grm import vanraden_grm, vanraden_grm_exact, xx_counts_valid
from oracle.plink import decode_bed, snp_counts

pytestmark = pytest.mark.gpu


def exact_bound(G_exact, n_valid, s2pq):
    return n_valid * 2.0**-46 / s2pq + 4 * np.spacing(np.abs(G_exact))


def gpu_grm(handle, bed, n, m, **kw):
    b = GrmBuilder(GrmOptions(**kw), handle=handle)
    b.compute(PlinkReader.from_bytes(bed, n, m), keep_xx_counts=True)
    return b


def test_umma_layout_probe(handle):
    A = ((np.arange(128)[:, None] * 3 + np.arange(32)[None, :] * 5) % 7 - 3).astype(np.float32)
    B = ((np.arange(32)[:, None] * 2 + np.arange(32)[None, :] * 3) % 5 - 2).astype(np.float32)
    D = np.zeros((128, 32), np.float32)
    handle.check(lib().cbx_selftest_umma(handle.raw, ptr(A), ptr(B), ptr(D)))
    np.testing.assert_array_equal(D, A @ B.T)


def test_toy_fixture_bit_exact(handle, toy_golden):
    bed = bytes.fromhex(toy_golden["bed_hex"])
    b = gpu_grm(handle, bed, 6, 4)
    assert b.getXXCounts().tolist() == toy_golden["xx_counts"]
    assert b.getSum2pq() == toy_golden["sum2pq"]
    assert b.getTotalSnps() == toy_golden["n_valid"] == 4
    Gx = np.array(toy_golden["G_exact_rounded"])
    assert np.all(np.abs(b.getGrm() - Gx) <= exact_bound(Gx, 4, b.getSum2pq()))
    Gr = np.array(toy_golden["G_restated"])
    assert np.abs(b.getGrm() - Gr).max() <= 1e-13 * np.abs(Gr).max()
    np.testing.assert_array_equal(b.getAlleleFreqs(), np.array(toy_golden["allele_freqs"], np.float32))


def test_snp_counts_bit_exact(handle):
    bed, _ = simulate_bed(1003, 257, seed=21, miss=0.05)
    got = bed_snp_counts(handle, bed, 1003, 257)
    ref = snp_counts(decode_bed(bed, 1003, 257))
    for k in got:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


@pytest.mark.parametrize("n,m,miss,seed", [
    (37, 100, 0.02, 1),       # single ragged tile, one chunk
    (300, 3000, 0.02, 2),     # two chunks (2048-SNP flush), ragged last tile
    (257, 4100, 0.0, 3),      # no missing calls, three chunks
    (130, 700, 0.2, 4),       # heavy missingness
])
def test_grm_matches_oracle(handle, n, m, miss, seed):
    bed, _ = simulate_bed(n, m, seed=seed, p_lo=0.005, miss=miss)
    b = gpu_grm(handle, bed, n, m)
    np.testing.assert_array_equal(b.getXXCounts(), xx_counts_valid(bed, n, m))
    ex = vanraden_grm_exact(bed, n, m)
    assert b.getSum2pq() == ex["sum2pq"]
    assert b.getTotalSnps() == ex["n_valid"]
    np.testing.assert_array_equal(b.getAlleleFreqs(), ex["freq"])
    G = b.getGrm()
    assert np.array_equal(G, G.T)
    assert np.all(np.abs(G - ex["G"]) <= exact_bound(ex["G"], ex["n_valid"], ex["sum2pq"]))
    ref = vanraden_grm(bed, n, m)
    assert np.abs(G - ref["G"]).max() <= 1e-13 * np.abs(ref["G"]).max()


def test_grm_all_filtered(handle):
    g = np.full((5, 20), 2, np.int8)  # monomorphic everywhere
    b = gpu_grm(handle, encode_bed(g), 20, 5)
    assert b.getTotalSnps() == 0 and b.getSum2pq() == 0.0
    assert not b.getGrm().any()


def test_grm_block_size_changes_only_sum_order(handle):
    bed, _ = simulate_bed(64, 900, seed=9, miss=0.01)
    a = gpu_grm(handle, bed, 64, 900, block_size=2048)
    c = gpu_grm(handle, bed, 64, 900, block_size=100)
    assert abs(a.getSum2pq() - c.getSum2pq()) <= 1e-12 * a.getSum2pq()
    ex = vanraden_grm_exact(bed, 64, 900, block_size=100)
    assert c.getSum2pq() == ex["sum2pq"]


def test_grm_errors(handle):
    bed = encode_bed(np.zeros((2, 8), np.int8))
    with pytest.raises(CbxError, match="CBX_ERR_FORMAT.*magic"):
        gpu_grm(handle, b"\x00\x00\x01" + bed[3:], 8, 2)
    with pytest.raises(CbxError, match="CBX_ERR_FORMAT.*SNP-major"):
        gpu_grm(handle, b"\x6c\x1b\x00" + bed[3:], 8, 2)
    with pytest.raises(CbxError, match="CBX_ERR_FORMAT.*truncated"):
        gpu_grm(handle, bed[:-1], 8, 2)
    with pytest.raises(CbxError, match="CBX_ERR_UNSUPPORTED"):
        gpu_grm(handle, bed, 8, 2, algorithm=3)
    # the handle stays usable after errors
    b = gpu_grm(handle, bytes.fromhex("6c1b01cb023a08e00e8b03"), 6, 4)
    assert b.getTotalSnps() == 4
