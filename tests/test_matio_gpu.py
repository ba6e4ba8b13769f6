"""GPU tests of the relationship-matrix files written from the device matrices
(cbx_write_upper_packed, cbx_write_grm_gcta): byte-identical to the oracle's writer
fed with the same matrix, readable by the oracle's restatement of the reference reader."""
import os

import numpy as np
import pytest

from cosmicblup_gb300 import CbxError, GrmBuilder, GrmOptions, Handle, PlinkReader, invert_psd, write_matrix_bin
from cosmicblup_gb300.synth import simulate_bed
from oracle.matio import grm_gcta_bytes, read_upper_packed, upper_packed_bytes

pytestmark = pytest.mark.gpu


def grm(handle, n, m, seed):
    bed, _ = simulate_bed(n, m, seed=seed, p_lo=0.05, miss=0.01)
    b = GrmBuilder(GrmOptions(), handle=handle)
    b.compute(PlinkReader.from_bytes(bed, n, m))
    return b


def test_grm_and_inverse_files(handle, tmp_path):
    n = 300
    b = grm(handle, n, 2000, seed=61)
    G = b.getGrm()
    p = str(tmp_path / "G.bin")
    write_matrix_bin(handle, 0, p, str(tmp_path / "G.id"), [f"a{i}" for i in range(n)])
    data = open(p, "rb").read()
    assert data == upper_packed_bytes(G)
    assert np.array_equal(read_upper_packed(data), G)
    assert open(tmp_path / "G.id").read().splitlines()[:2] == ["a0", "a1"]
    Gi = invert_psd(handle, None, n).T  # the C ABI's host matrices are column-major
    pi = str(tmp_path / "Ginv.bin")
    write_matrix_bin(handle, 1, pi)
    assert open(pi, "rb").read() == upper_packed_bytes(Gi)


def test_gcta_save(handle, tmp_path):
    n = 257
    b = grm(handle, n, 1500, seed=62)
    prefix = str(tmp_path / "out")
    b.save(prefix)
    g, nb = grm_gcta_bytes(b.getGrm(), b.getTotalSnps())
    assert open(prefix + ".grm.bin", "rb").read() == g
    assert open(prefix + ".grm.N.bin", "rb").read() == nb
    ids = open(prefix + ".grm.id").read().splitlines()
    assert len(ids) == n and ids[0] == "1\t1"


def test_chunked_large_file(handle, tmp_path):
    # n (n + 1) / 2 above the 32 Mi-value staging pass: written in two passes
    n = 8300
    b = grm(handle, n, 400, seed=63)
    p = str(tmp_path / "big.bin")
    write_matrix_bin(handle, 0, p)
    assert os.path.getsize(p) == 60 + 8 * n * (n + 1) // 2
    assert open(p, "rb").read() == upper_packed_bytes(b.getGrm())


def test_missing_matrix_is_an_error(tmp_path):
    with Handle(0) as h:
        with pytest.raises(CbxError) as e:
            write_matrix_bin(h, 1, str(tmp_path / "x.bin"))
        assert e.value.code == 9
        with pytest.raises(CbxError) as e:
            write_matrix_bin(h, 2, str(tmp_path / "x.bin"))
        assert e.value.code == 1
