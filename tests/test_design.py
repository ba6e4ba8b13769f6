"""CPU test: the package's vectorised fixed-effect design builder equals the
oracle's restatement of buildFixedDesignGeneric (src/core/design.cpp:13-109)."""
import numpy as np

from cosmicblup_gb300.design import fixed_design
from cosmicblup_gb300.mme import rows_to_csr
from oracle.mme import build_fixed_design


def test_fixed_design_matches_oracle():
    rng = np.random.default_rng(1)
    cats = [[f"L{rng.integers(0, 30):03d}", ["M", "F", ""][rng.integers(0, 3)], "b" if rng.random() < .5 else "a"]
            for _ in range(500)]
    nums = rng.standard_normal((500, 2))
    d = fixed_design(cats, nums)
    p, rows, names = build_fixed_design(cats, nums)
    fp, fc, fv = rows_to_csr(rows)
    assert d.p == p and d.names == names
    np.testing.assert_array_equal(d.ptr, fp)
    np.testing.assert_array_equal(d.col, fc)
    np.testing.assert_array_equal(d.val, fv)
    assert d.dense().shape == (500, p)


def test_level_order_is_bytewise():
    d = fixed_design([["b"], ["B"], ["a"], ["10"], ["9"]])
    # std::set order: "10" < "9" < "B" < "a" < "b"; "10" is the base level
    assert d.names == ["mu", "factor1_9", "factor1_B", "factor1_a", "factor1_b"]
