"""The callbacks' nonlinear index change (NLSE/callbacks.py:57-112) on the CPU.

* The oracle against the records of the reference's own evaluate_delta_n
  and adapt_delta_z inside out_field (tests/golden/callbacks_*.npz, made by
  tests/golden/make_golden.py): bit-exact, same NumPy evaluation.
* The host logic that maps the parameters onto the kernel's per-segment
  values and precision flags (callbacks.index_change_params): a NumPy model
  of the kernel's arithmetic (nlse_delta_n / nlse_delta_n_max: every
  operation rounded on its own, in the precisions the flags select) fed with
  those values must equal the oracle bit for bit, for every parameter type
  NumPy promotes differently.
"""

import numpy as np
import pytest
from scipy.constants import c, epsilon_0

from nlse_gb300 import callbacks as cb
from oracle import nlse_oracle as o
from tests import golden_cases as gc

N2, ISAT = gc.N2, gc.ISAT


@pytest.mark.parametrize("name", ["callbacks_c64_delta_n", "callbacks_c64_batch_delta_n",
                                  "callbacks_c128_delta_n"])
def test_oracle_delta_n_matches_reference_records(name):
    f = gc.load(name)
    n2 = f["n2"] if f["n2"].ndim else N2  # a Python float in the scalar cases
    got = o.delta_n(f["samples"], n2, ISAT)
    assert got.dtype == f["delta_n"].dtype
    assert np.array_equal(got, f["delta_n"])


@pytest.mark.parametrize("name", ["callbacks_c64_adapt", "callbacks_c128_adapt"])
def test_oracle_adapt_matches_reference_steps(name):
    f = gc.load(name)
    u, k = int(f["meta"][4]), float(f["meta"][5])
    dzs = f["dzs"]
    assert dzs[0] == f["meta"][1] and len(dzs) == int(f["meta"][3])
    # the step set after update m (at step m*u) is the one the next step records
    got = [o.adapt_delta_z(s, N2, ISAT, k) for s in f["samples"]]
    ref = dzs[1::u]
    assert len(ref) in (len(got), len(got) - 1)
    assert np.array_equal(np.array(got[:len(ref)]), ref)
    # between updates the step stays
    for m in range(len(ref)):
        assert np.all(dzs[m * u + 1:(m + 1) * u + 1] == ref[m])


def model(A, params, adapt):
    """The kernel's arithmetic in NumPy for A and the output of index_change_params."""
    pix, coef, isat, flags, out = params
    f32 = A.dtype == np.complex64
    T = np.float32 if f32 else np.float64
    TC = np.float64 if (not f32 or flags & 1) else np.float32
    TD = np.float64 if (not f32 or flags & 2) else np.float32
    TO = np.float64 if np.float64 in (TC, TD) else np.float32
    a = A.reshape(-1, pix)
    re, im = a.real.astype(T), a.imag.astype(T)
    i2 = im * im
    if adapt:
        i2 = ((i2 * T(c)) * T(epsilon_0)) / T(2)
    q = re * re + i2
    num = coef.astype(TC)[:, None] * q.astype(TC)
    den = TD(1) + q.astype(TD) / isat.astype(TD)[:, None]
    r = (num.astype(TO) / den.astype(TO)).reshape(A.shape)
    assert r.dtype == out
    return r


def _field(shape, dtype, seed):
    rng = np.random.default_rng(seed)
    A = 3e3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    return A.astype(dtype)


B3 = np.linspace(-1.6e-9, -4e-10, 3).reshape(3, 1, 1)
CASES = [
    # (n2, I_sat, field shape, spatial axes)
    (N2, ISAT, (16, 16), 2),
    (np.float64(N2), ISAT, (16, 16), 2),
    (N2, np.float64(ISAT), (16, 16), 2),
    (B3, ISAT, (3, 16, 16), 2),
    (N2, np.array([1e5, 2e5, 5e4]).reshape(3, 1, 1), (3, 16, 16), 2),
    (B3.astype(np.float32), ISAT, (3, 16, 16), 2),
    (np.float32(N2), np.float32(ISAT), (16, 16), 2),
    (N2, ISAT, (2, 16, 16), 2),                       # two components
    (B3.reshape(3, 1, 1, 1), ISAT, (3, 2, 16, 16), 2),  # batch of two-component fields
    (N2, ISAT, (4, 64), 1),                           # 1-D
    (B3.reshape(3, 1, 1, 1), ISAT, (3, 4, 8, 8), 3),  # 3-D, per-field n2
]


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_kernel_model_with_host_parameters_equals_oracle(case, dtype):
    n2, isat, shape, na = CASES[case]
    A = _field(shape, dtype, case)
    for adapt in (False, True):
        p = cb.index_change_params(n2, isat, shape, na, dtype == np.complex64, adapt)
        assert p is not None
        got = model(A, p, adapt)
        if adapt:
            assert np.array_equal(got.max(), o.adapt_peak(A, n2, isat))
        else:
            ref = o.delta_n(A, n2, isat)
            assert got.dtype == ref.dtype and np.array_equal(got, ref)


def test_adapt_peak_is_float64_for_a_python_float_n2():
    # np.abs of a Python float is a float64 NumPy scalar: the peak is FP64
    p = cb.index_change_params(N2, ISAT, (16, 16), 2, True, adapt=True)
    assert p[3] == 1 and p[4] == np.float64
    p = cb.index_change_params(N2, ISAT, (16, 16), 2, True, adapt=False)
    assert p[3] == 0 and p[4] == np.float32


@pytest.mark.parametrize("n2,shape", [
    (B3, (16, 16)),                      # broadcasting would grow the field
    (np.full((16, 16), N2), (16, 16)),   # varies across the grid
    (N2 * (1 + 1j), (16, 16)),           # complex
    (np.ones((2, 3, 1, 1)), (3, 16, 16)),
])
def test_parameters_without_a_device_form(n2, shape):
    assert cb.index_change_params(n2, ISAT, shape, 2, True, False) is None


def test_step_from_peak_follows_numpy():
    class S:
        k = 8.055365783e6
    for peak in (np.float32(2.5e-4), np.float64(2.5e-4)):
        z_nl = float(1 / (S.k * peak))
        assert cb._peak_to_delta_z(S, peak) == np.abs(z_nl) / 12
    assert cb._peak_to_delta_z(S, np.float32(0)) == np.inf  # n2 = 0 beyond L: no error
