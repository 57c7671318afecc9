"""The constructors' default step (nlse.py:108-114, nlse_3d.py:105-111)
without the broadcast of n2 and power: bit for bit the minimum over the
broadcast array the reference forms, with the same result type."""

import numpy as np
import pytest

import nlse_gb300 as ng
from nlse_gb300.nlse import nonlinear_length

K = 2 * np.pi / 780e-9
B = 7
rng = np.random.default_rng(4)
N2S = [-1.6e-9, np.float64(-1.6e-9), np.array(-1.6e-9),
       -(10.0 ** rng.uniform(-10, -8.4, B)).reshape(B, 1, 1),
       -(10.0 ** rng.uniform(-10, -8.4, B)), np.zeros((B, 1, 1)),
       (-(10.0 ** rng.uniform(-10, -8.4, B))).astype(np.float32).reshape(B, 1, 1)]
POWERS = [1.05, np.float64(1.05), rng.uniform(0.1, 2.0, B), rng.uniform(0.1, 2.0, (B, 1, 1)),
          rng.uniform(0.1, 2.0, (1, B)).astype(np.float32)]


def _literal(n2, power, w2):
    z = 1 / (K * abs(n2 * power / w2))
    return z.min() if isinstance(z, np.ndarray) else z


@pytest.mark.parametrize("n2", range(len(N2S)))
@pytest.mark.parametrize("power", range(len(POWERS)))
def test_nonlinear_length_equals_the_minimum_over_the_broadcast(n2, power):
    a, b, w2 = N2S[n2], POWERS[power], (4 * 2.23e-3) ** 2
    with np.errstate(divide="ignore"):
        ref = _literal(a, b, w2)
        got = nonlinear_length(K, a, b, w2)
    assert type(got) is type(ref) or isinstance(got, np.floating) and isinstance(ref, np.floating)
    assert np.array_equal(np.asarray(got), np.asarray(ref))


def test_constructor_step_type_and_value():
    n2 = -(10.0 ** rng.uniform(-10, -8.4, 2048)).reshape(2048, 1, 1)
    p = rng.uniform(0.1, 2.0, 2048)
    s = ng.NLSE(20, p, 4 * 2.23e-3, n2, None, 1e-2, NX=16, NY=16, Isat=1e5)
    ref = float((1 / (s.k * abs(n2 * p / (4 * 2.23e-3) ** 2))).min())
    assert type(s.delta_z) is float and s.delta_z == 5e-3 * ref
    s = ng.NLSE(20, np.float64(1.05), 4 * 2.23e-3, np.float64(-1.6e-9), None, 1e-2, NX=16, NY=16)
    assert isinstance(s.delta_z, np.float64)
