"""Pin the CPU oracle against fields computed by the reference's own code.

The fixtures in tests/golden/ come from running the reference package
(tests/golden/make_golden.py).  These tests need no GPU.
"""

import numpy as np
import pytest

from oracle import nlse_oracle as orc
from tests import golden_cases as gc
from tests.cases import rel_l2


def _tol(name: str) -> float:
    if "cpu" in name:
        # The CPU-path fixture ran the numba kernels as plain Python, whose
        # scalar promotion rounds the potential term in complex64.
        return 1e-6
    return 1e-13 if "c128" in name else 1e-7


@pytest.mark.parametrize("name", gc.FIXTURES)
def test_oracle_matches_reference_output(name):
    got = gc.run(name, "oracle")
    ref = gc.load(name)["out"]
    assert got.shape == ref.shape and got.dtype == ref.dtype
    assert rel_l2(got, ref) <= _tol(name)


@pytest.mark.parametrize("tag", ["c64", "c128"])
def test_oracle_elementwise_kernels_match_reference(tag):
    f = gc.load(f"kernels_{tag}")
    A, B, V = f["A"], f["B"], f["V"]
    rdt = np.float32 if tag == "c64" else np.float64
    sq_a, sq_b = (np.abs(A) ** 2).astype(rdt), (np.abs(B) ** 2).astype(rdt)
    np.testing.assert_array_equal(orc.square_mod(A).astype(rdt), f["square_mod"])
    o = A.copy()
    orc.nl_prop(o, sq_a, 0.3, 0.7, 5.0 * V, 2.5, 1.7)
    np.testing.assert_array_equal(o, f["nl_prop"])
    o = A.copy()
    orc.nl_prop(o, sq_a, 0.3, 0.7, None, 2.5, 1.7)
    np.testing.assert_array_equal(o, f["nl_prop_without_V"])
    o = A.copy()
    orc.nl_prop_c(o, sq_a, sq_b, 0.3, 0.7, 5.0 * V, 2.5, -1.5, 1.7, 0.9)
    np.testing.assert_array_equal(o, f["nl_prop_c"])
    o = A.copy()
    orc.nl_prop_c(o, sq_a, sq_b, 0.3, 0.7, None, 2.5, -1.5, 1.7, 0.9)
    np.testing.assert_array_equal(o, f["nl_prop_without_V_c"])
    r1, r2 = A.copy(), B.copy()
    orc.rabi_coupling(r1, r2, 0.3, 1.3)
    np.testing.assert_array_equal(r1, f["rabi1"])
    np.testing.assert_array_equal(r2, f["rabi2"])


def test_step_counts_match_reference_loop():
    for z, dz, n in gc.load("step_counts")["counts"]:
        assert orc.count_steps(z, dz) == int(n)


def test_benchmark_step_counts():
    assert orc.count_steps(10e-3, 5e-5) == 201
    assert orc.count_steps(10e-3, 2e-5) == 501
    assert orc.count_steps(20e-3, 5e-5) == 400
