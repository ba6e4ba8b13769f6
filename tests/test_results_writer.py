"""CPU tests of the text result writers (cbx_write_vars / cbx_write_beta /
cbx_write_rand, host code in libcbx, no GPU) against the oracle's restatement
of GSOutput::writeResults (src/solve/result_writer.cpp:64-430): byte-identical
files, including animals with several records, animals without records (sorted
by ID after the recorded ones), missing IDs and a missing SE column."""
import numpy as np

from cosmicblup_gb300.results import write_beta, write_rand, write_vars
from oracle.results import beta_text, rand_text, vars_text


def test_vars_file(built_lib, tmp_path):
    for args in [(0.41, 0.05, 0.6, 0.04), (1e-7, 0.0, 2.5, 0.1), (3.5, 1e-13, 1e-3, 2e-4)]:
        for tag in ("GA", "HA"):
            path = write_vars(str(tmp_path / "r"), *args, tag=tag)
            assert open(path).read() == vars_text(*args, tag=tag)


def test_beta_file(built_lib, tmp_path):
    rng = np.random.default_rng(1)
    names = ["mu"] + [f"factor1_L{k:04d}" for k in range(1, 12)]
    beta = rng.normal(0, 3, len(names)) * 10.0 ** rng.integers(-6, 6, len(names))
    se = np.abs(rng.normal(0, 1, len(names)))
    path = write_beta(str(tmp_path / "r"), names, beta, se)
    assert open(path).read() == beta_text(names, beta, se)
    path = write_beta(str(tmp_path / "r2"), names, beta)
    assert open(path).read() == beta_text(names, beta)


def test_rand_file(built_lib, tmp_path):
    rng = np.random.default_rng(2)
    q, n, p = 40, 55, 3
    aid = rng.integers(0, q + 1, n).astype(np.int32)  # 0 = no animal; repeats and unrecorded animals
    y = rng.normal(10, 2, n)
    rows = [[(0, 1.0)] + ([(int(rng.integers(1, p)), 1.0)] if rng.random() < 0.7 else []) for _ in range(n)]
    beta = rng.normal(0, 1, p)
    u = rng.normal(0, 0.5, q)
    ids = [f"A{rng.integers(0, 1000):04d}" if rng.random() < 0.9 else "" for _ in range(q)]
    for tag in ("GA", "HA"):
        path = write_rand(str(tmp_path / tag), y, aid, rows, p, beta, u, ids=ids, tag=tag)
        assert open(path).read() == rand_text(y, aid, rows, p, beta, u, ids=ids, tag=tag)
    path = write_rand(str(tmp_path / "noid"), y, aid, rows, p, beta, u)
    assert open(path).read() == rand_text(y, aid, rows, p, beta, u)
