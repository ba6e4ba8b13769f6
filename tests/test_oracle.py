"""CPU tests: the oracle against the committed golden vectors, and the BED codec."""
import numpy as np
import pytest

from cosmicblup_gb300.synth import encode_bed, simulate_bed
from oracle.grm import (snp_stats, sum_2pq_blocked, vanraden_grm, vanraden_grm_exact,
                        xx_counts)
from oracle.plink import decode_bed


def test_toy_decode_and_xx(toy_golden):
    bed = bytes.fromhex(toy_golden["bed_hex"])
    g = decode_bed(bed, 6, 4)
    assert g.tolist() == toy_golden["genotypes_snp_major"]
    assert encode_bed(g) == bed
    assert xx_counts(bed, 6, 4).tolist() == toy_golden["xx_counts"]


def test_toy_grm_known_answer(toy_golden):
    # VanRaden G for the reference's toy fixture, restated from grm_builder.cpp:166-404
    bed = bytes.fromhex(toy_golden["bed_hex"])
    r = vanraden_grm(bed, 6, 4)
    assert r["sum2pq"] == toy_golden["sum2pq"] == 1.9861111044883728
    G = np.array(toy_golden["G_restated"])
    np.testing.assert_allclose(r["G"], G, rtol=0, atol=1e-15)
    assert np.diag(G)[0] == 1.5244755228898768
    assert G[0, 5] == -1.496503508162676
    assert G[2, 5] == 1.104895081903202
    e = vanraden_grm_exact(bed, 6, 4)
    np.testing.assert_allclose(e["G"], np.array(toy_golden["G_exact_rounded"]), rtol=0, atol=0)


def test_bed_roundtrip_random():
    rng = np.random.default_rng(5)
    for n in (1, 3, 4, 5, 130):
        g = rng.integers(-1, 3, size=(7, n)).astype(np.int8)
        bed = encode_bed(g)
        assert len(bed) == 3 + 7 * ((n + 3) // 4)
        assert np.array_equal(decode_bed(bed, n, 7), g)


def test_bad_magic_and_truncation():
    bed = bytearray(encode_bed(np.zeros((2, 8), np.int8)))
    with pytest.raises(ValueError, match="magic"):
        decode_bed(bytes([0, 0, 1]) + bytes(bed[3:]), 8, 2)
    with pytest.raises(ValueError, match="SNP-major"):
        decode_bed(bytes([0x6C, 0x1B, 0]) + bytes(bed[3:]), 8, 2)
    with pytest.raises(ValueError, match="Truncated"):
        decode_bed(bytes(bed[:-1]), 8, 2)


def test_maf_filter_float_threshold():
    # freq exactly 0.01 passes (0.01 >= (double)0.01f is false? 0.01 < 0.0099999998 is false)
    n = 100
    g = np.zeros((3, n), np.int8)
    g[0, :2] = 1          # freq 0.01 -> kept
    g[1, :1] = 1          # freq 0.005 -> dropped
    g[2, :] = 2           # monomorphic -> dropped
    st = snp_stats(g)
    assert st["valid"].tolist() == [True, False, False]
    assert st["freq"][1] == -1.0


def test_sum2pq_block_order():
    rng = np.random.default_rng(1)
    bed, _ = simulate_bed(50, 300, seed=3, miss=0.05)
    st = snp_stats(decode_bed(bed, 50, 300))
    a = sum_2pq_blocked(st["two_pq"], st["valid"], 2048)
    b = sum_2pq_blocked(st["two_pq"], st["valid"], 7)
    assert abs(a - b) < 1e-12 * a


def test_exact_vs_fp64_oracle():
    bed, _ = simulate_bed(40, 500, seed=11, miss=0.03)
    r = vanraden_grm(bed, 40, 500)
    e = vanraden_grm_exact(bed, 40, 500)
    scale = np.abs(e["G"]).max()
    assert np.abs(r["G"] - e["G"]).max() < 1e-13 * scale
