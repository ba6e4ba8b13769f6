"""GPU test of cbx_dense_apply_noalloc, the entry point for callers that cannot
allocate device memory while they run (a host framework that owns the device
memory pool, a latency-critical loop that must not call cudaMalloc).  Its
product must agree within rounding with cbx_qinv_apply's, which allocates its
own buffers, on consecutive calls that reuse its static scratch array.

The file name sorts last so that a stop-at-first-failure run has already run
every other test; it also passes alone in a fresh process."""
import numpy as np
import pytest

from cosmicblup_gb300 import DeviceMME, Handle
from cosmicblup_gb300._lib import lib
from cosmicblup_gb300.synth import simulate_bed, simulate_gblup_records
from oracle.grm import vanraden_grm
from oracle.mme import build_fixed_design, invert_psd_matrix

pytestmark = pytest.mark.gpu


def test_noalloc_matches_qinv_apply_twice():
    torch = pytest.importorskip("torch")
    n, m = 300, 2000
    bed, _ = simulate_bed(n, m, seed=77, p_lo=0.05, miss=0.01)
    Gi = invert_psd_matrix(vanraden_grm(bed, n, m)["G"])
    rec = simulate_gblup_records(n, 3, np.zeros(n), seed=78, var_e=1.0)
    p, rows, _ = build_fixed_design(rec["cats"])
    with Handle(0) as h:
        dm = DeviceMME(h, rec["y"], rec["aid"], rows, p, n)
        dm.set_qinv_dense(Gi)
        rng = np.random.default_rng(79)
        # calls in a row with every pass width (1, 2, 4, 8, 16, 32 columns; 40 and
        # 33 take two passes, the second narrower than the first)
        for k in (5, 40, 1, 2, 3, 12, 33, 5):
            X = rng.normal(size=(n, k))
            ref = dm.qinv_apply(X)
            xd = torch.from_numpy(np.ascontiguousarray(X.T)).to("cuda")  # column-major q x k
            yd = torch.full((k, n), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            h.check(lib().cbx_dense_apply_noalloc(h.raw, k, xd.data_ptr(), yd.data_ptr()))
            h.sync()
            Y = yd.cpu().numpy().T
            assert np.abs(Y - ref).max() <= 1e-12 * np.abs(ref).max()
