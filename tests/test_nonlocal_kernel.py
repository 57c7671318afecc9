"""The K0 nonlocal kernel builder (NLSE/nlse.py:143-155) against the oracle,
including the d = 0 case (nl_length below the grid step), where the
reference's kernel is NaN: same NaN kernel, and a RuntimeWarning at
construction naming the cause."""

import warnings

import numpy as np
import pytest

import nlse_gb300 as ng
from oracle import nlse_oracle as orc


@pytest.mark.parametrize("nl_length", [20e-6, 100e-6, 300e-6])
def test_k0_kernel_equals_oracle(nl_length):
    dx = 4 * 2.23e-3 / 1024
    with warnings.catch_warnings():
        warnings.simplefilter("error", RuntimeWarning)
        got = ng.NLSE._k0_profile(nl_length, dx)
    ref = orc.k0_profile(nl_length, dx)
    assert got.shape == ref.shape and np.array_equal(got, ref)


def test_k0_kernel_below_the_grid_step_is_nan_and_warned():
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        s = ng.NLSE(20, 1.05, 4 * 2.23e-3, -1.6e-9, None, 1e-2, NX=64, NY=64, Isat=1e5,
                    nl_length=1e-6)
    assert any("below the grid step" in str(x.message) for x in w
               if issubclass(x.category, RuntimeWarning))
    with np.errstate(all="ignore"), warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = orc.k0_profile(1e-6, s.delta_X)
    assert np.isnan(s.nl_profile).all() and np.isnan(ref).all()
