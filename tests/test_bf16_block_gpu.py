"""The optional bf16 block product of the FP32 PCG bulk (CBX_BF16=1, read once per
process, so the check runs in a child process): the mixed-precision solve keeps
the FP64-accurate refinement residual, so with the bf16 copy of the block it
reaches the same solution (relres 1e-10) as the oracle's direct solve."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

CHILD = r"""
import numpy as np
from cosmicblup_gb300 import DeviceMME, Handle
from cosmicblup_gb300.mme import MIXED
from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
from oracle.grm import vanraden_grm
from oracle.mme import MME, build_fixed_design, invert_psd_matrix
n, m = 1000, 3000
bed, _ = simulate_bed(n, m, seed=610, p_lo=0.05, miss=0.01)
Gi = invert_psd_matrix(vanraden_grm(bed, n, m)["G"])
g = genetic_values(bed, n, m, seed=611, var_a=0.4)
rec = simulate_gblup_records(n, 4, g, seed=612, var_e=0.6)
p, rows, _ = build_fixed_design(rec["cats"])
om = MME(rec["y"], rec["aid"], rows, p, n)
lam = 1.5
A = om.lhs(Gi, lam)
rng = np.random.default_rng(613)
B = np.zeros((om.dim, 70))
B[:, 0] = om.rhs()
B[p:, 1:] = rng.choice([-1.0, 1.0], size=(n, 69))
h = Handle(0)
dm = DeviceMME(h, rec["y"], rec["aid"], rows, p, n)
dm.set_qinv_dense(Gi)
for k in (33, 70):   # a 64-wide block and the 128-wide one
    X, it, rr = dm.pcg_solve(lam, B[:, :k], precision=MIXED)
    Xe = np.linalg.solve(A, B[:, :k])
    err = np.abs(X - Xe).max(axis=0) / np.abs(Xe).max(axis=0)
    assert err.max() < 1e-8, (k, err.max())
    assert rr.max() < 1e-10, (k, rr.max())
print("ok")
"""


def test_bf16_block_solve_matches_oracle():
    env = dict(os.environ, CBX_BF16="1")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=root, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
