"""Host arrays across out_field (nlse.py:309-370 semantics on the device engine).

A potential or propagator given as a NumPy array comes back as a NumPy array
with the same values; when nothing changed the device copy (torch version
counter) it is the caller's own array, when a callback changed it in place
the change comes back.  Results reach the host through the pinned staging
path with the values of a direct copy.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import engine  # noqa: E402
from tests import cases  # noqa: E402


def _sim(N=64):
    s = ng.NLSE(20, 1.05, 4 * 2.23e-3, -1.6e-9, None, 1e-3, NX=N, NY=N, Isat=1e5)
    s.delta_z = 5e-5
    s.V = (-1e-4 * np.exp(-(s.XX**2 + s.YY**2) / (70e-6) ** 2)).astype(np.complex64)
    return s


def test_unchanged_host_arrays_come_back_as_the_same_objects():
    s = _sim()
    V0 = s.V
    V_copy = V0.copy()
    E = cases.gaussian(s.XX, s.YY).astype(np.complex64)
    s.out_field(E, 2e-4, verbose=False)
    P0 = s.propagator
    assert s.V is V0 and np.array_equal(s.V, V_copy)
    assert isinstance(P0, np.ndarray)
    s.out_field(E, 2e-4, verbose=False)
    assert s.V is V0 and s.propagator is P0


def test_a_potential_changed_on_the_device_comes_back_changed():
    s = _sim()
    V0 = s.V.copy()
    E = cases.gaussian(s.XX, s.YY).astype(np.complex64)

    def bump(simu, A, z, i):
        if i == 0:
            simu.V.mul_(2)  # in place on the device copy

    s.out_field(E, 2e-4, verbose=False, callback=bump)
    assert isinstance(s.V, np.ndarray)
    np.testing.assert_array_equal(s.V, 2 * V0)


@pytest.mark.parametrize("shape,dtype", [((8, 1024, 1024), torch.complex64),
                                         ((3, 17), torch.complex128),
                                         ((4, 512, 512), torch.float32)])
def test_to_host_equals_a_direct_copy(shape, dtype):
    g = torch.Generator(device="cuda").manual_seed(3)
    real = torch.float64 if dtype == torch.complex128 else torch.float32
    x = torch.randn(shape, dtype=real, device="cuda", generator=g)
    if dtype.is_complex:
        x = torch.complex(x, torch.randn(shape, dtype=real, device="cuda", generator=g))
    for _ in range(2):  # the second call reuses the staging buffer
        h = engine.to_host(x)
        assert not h.is_cuda and h.dtype == x.dtype and h.shape == x.shape
        assert torch.equal(h, x.cpu())
