"""W'W assembled on the device (wtw.cu) against the host assembly and the oracle.

Both assemblies sum every (row, column) entry's triplets in record order, so
their CSRs are the same bit for bit: FP64 solves with the two MMEs return the
same bits.  Records with several fixed effects (negative covariates), with no
fixed effect, with no animal and with an out-of-range animal id are covered."""
import os

import numpy as np
import pytest

from cosmicblup_gb300 import DeviceMME
from cosmicblup_gb300.mme import FP64
from oracle.mme import MME

pytestmark = pytest.mark.gpu


def records(n_rec, p, q, seed):
    rng = np.random.default_rng(seed)
    y = rng.normal(10.0, 2.0, n_rec)
    aid = rng.integers(0, q + 2, n_rec).astype(np.int32)  # 0: none, q + 1: out of range
    rows = []
    for i in range(n_rec):
        # distinct columns per record, as FixedDesignG builds them (one column per
        # factor or covariate): the reference emits a record's (c, c) product
        # once per pair a <= b, which equals W'W only for distinct columns
        k = int(rng.integers(0, 4))
        cols = set(int(c) for c in rng.choice(np.arange(1, p), size=min(k, p - 1), replace=False))
        if i < p:
            cols.add(i)  # every fixed column has a record
        r = [(0, 1.0)] if k or i == 0 else []
        r += [(c, float(rng.choice([1.0, rng.normal()]))) for c in sorted(cols) if c != 0]
        rows.append(r)
    return y, aid, rows


def build(handle, y, aid, rows, p, q, host):
    old = os.environ.get("CBX_WTW_HOST")
    os.environ["CBX_WTW_HOST"] = "1" if host else "0"
    try:
        dm = DeviceMME(handle, y, aid, rows, p, q)
    finally:
        if old is None:
            del os.environ["CBX_WTW_HOST"]
        else:
            os.environ["CBX_WTW_HOST"] = old
    Q = np.eye(q) * 2.0 + 0.1
    dm.set_qinv_dense(Q)
    return dm, Q


@pytest.mark.parametrize("n_rec,p,q,seed", [(3000, 7, 500, 1500), (20000, 40, 4000, 1501), (50, 3, 20, 1502)])
def test_device_wtw_equals_host_and_oracle(handle, n_rec, p, q, seed):
    y, aid, rows = records(n_rec, p, q, seed)
    aid_o = np.where(aid <= q, aid, 0)
    om = MME(y, aid_o, rows, p, q)
    b = np.random.default_rng(seed + 1).normal(size=(p + q, 3))
    xs = []
    for host in (True, False):
        dm, Q = build(handle, y, aid, rows, p, q, host)
        x, _, _ = dm.pcg_solve(1.7, b, precision=FP64, tol=1e-12)
        xs.append(x)
    assert np.array_equal(xs[0], xs[1])
    A = om.lhs(Q, 1.7)
    xe = np.linalg.solve(A, b)
    assert np.abs(xs[1] - xe).max() <= 1e-9 * np.abs(xe).max()
