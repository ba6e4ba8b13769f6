"""CPU tests of host-side helpers: the FixedDesignG -> CSR conversion, the seeded
generators' determinism and pedigree order (parents before offspring, which the
reference's Meuwissen-Luo pass assumes, src/core/a_matrix.cpp:168-178), and the
page-locking helper's fallback where no GPU is present."""
import numpy as np

from cosmicblup_gb300.mme import rows_to_csr
from cosmicblup_gb300.synth import simulate_bed, simulate_pedigree
from oracle.plink import decode_bed


def test_rows_to_csr():
    rows = [[(0, 1.0), (3, 1.0)], [], [(0, 1.0), (1, 2.5)]]
    ptr, col, val = rows_to_csr(rows)
    assert ptr.tolist() == [0, 2, 2, 4] and ptr.dtype == np.int64
    assert col.tolist() == [0, 3, 0, 1] and col.dtype == np.int32
    assert val.tolist() == [1.0, 1.0, 1.0, 2.5] and val.dtype == np.float64


def test_simulate_bed_independent_of_threads():
    a, pa = simulate_bed(301, 2500, seed=9, threads=1)
    b, pb = simulate_bed(301, 2500, seed=9, threads=7)
    assert a == b and np.array_equal(pa, pb)
    g = decode_bed(a, 301, 2500)
    miss = (g < 0).mean()
    assert 0.002 < miss < 0.03   # 1 % missing calls by default
    c, _ = simulate_bed(301, 2500, seed=10)
    assert c != a


def test_pedigree_parents_precede_offspring():
    sire, dam = simulate_pedigree(5, 400, 20, 150, seed=3, p_unknown=0.05)
    n = sire.size
    idx = np.arange(n)
    for par in (sire, dam):
        known = par >= 0
        assert np.all(par[known] < idx[known])
        # parents come from the previous generation
        assert np.all(par[known] // 400 == idx[known] // 400 - 1)
    assert np.all(sire[:400] < 0) and np.all(dam[:400] < 0)   # founders
    both = (sire >= 0) & (dam >= 0)
    assert not np.any(sire[both] == dam[both])
    unknown = (sire[400:] < 0).mean()
    assert 0.02 < unknown < 0.09


def test_pinned_falls_back_without_a_gpu(built_lib):
    from cosmicblup_gb300._lib import pinned
    a = np.arange(1000.0)
    with pinned(a, None, np.zeros(0)) as p:
        assert len(p.done) <= 1
    assert a[10] == 10.0
