"""GPU test of the launch-shape autotuner: every candidate shape of every tuned
kernel gives the same bits, so a run with tuning on reproduces one with tuning off
exactly, and the decisions are reported."""
import os

import numpy as np
import pytest

from cosmicblup_gb300 import DeviceGenotypes, DeviceMME
from cosmicblup_gb300._lib import tune_enable, tune_report, tune_reset
from cosmicblup_gb300.mme import MIXED
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from oracle.grm import vanraden_grm
from oracle.mme import build_fixed_design, invert_psd_matrix

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem():
    n, m = 1500, 3000
    bed, _ = simulate_bed(n, m, seed=77, p_lo=0.05, miss=0.02)
    Gi = invert_psd_matrix(vanraden_grm(bed, n, m)["G"])
    g = genetic_values(bed, n, m, seed=78, var_a=0.4)
    rec = simulate_gblup_records(n, 9, g, seed=79, var_e=0.6)
    p, rows, _ = build_fixed_design(rec["cats"])
    rng = np.random.default_rng(80)
    B = np.zeros((p + n, 33))
    B[p:, :] = rng.choice([-1.0, 1.0], size=(n, 33))
    return {"bed": bed, "n": n, "m": m, "Gi": Gi, "rec": rec, "p": p, "rows": rows, "B": B,
            "v": rng.standard_normal(n), "w": rng.standard_normal(m)}


def workload(handle, d):
    dm = DeviceMME(handle, d["rec"]["y"], d["rec"]["aid"], d["rows"], d["p"], d["n"])
    dm.set_qinv_dense(d["Gi"])
    X33, _, _ = dm.pcg_solve(1.7, d["B"], precision=MIXED)          # float-float refinements
    X1, _, _ = dm.pcg_solve(1.7, d["B"][:, :1], precision=MIXED)    # one column: the GEMV
    g = DeviceGenotypes(d["bed"], d["n"], d["m"], handle)
    return [X33, X1, g.multiply_Zt_v(d["v"]), g.multiply_Z_v(d["w"])]


def test_tuning_changes_no_bits(handle, problem):
    try:
        tune_enable(False)
        tune_reset()
        off = workload(handle, problem)
        assert tune_report() == []
        tune_enable(True)
        tune_reset()
        on = workload(handle, problem)
        rep = tune_report()
        again = workload(handle, problem)  # decisions reused
        assert tune_report() == rep
    finally:
        tune_enable(True)
    for a, b, c in zip(off, on, again):
        assert np.array_equal(a, b)
        assert np.array_equal(a, c)
    kernels = {ln.split()[0] for ln in rep}
    # the float-float refinement product is tuned when it takes the 16-column
    # pieces, i.e. with the tensor-core fixed-point product switched off (CBX_FX=0)
    tuned = {"k_gemv", "k_geno_zt", "k_geno_z"} | ({"k_dense_ff"} if os.environ.get("CBX_FX") == "0" else set())
    assert tuned <= kernels, rep
    for ln in rep:
        ms = [float(t) for t in ln.split(" ms ")[1].split()]
        choice = int(ln.split(" choice ")[1].split()[0])
        assert all(t > 0 for t in ms) and 0 <= choice < len(ms)
