"""The project FFT (nlse_fft through the C ABI) against numpy.fft."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _plan(ndim, shape, nf, comps, dt):
    from nlse_gb300.engine import Plan

    return Plan.get(ndim, shape, nf, comps, 0 if dt == np.complex64 else 1, torch.device("cuda", 0))


CASES = [
    (1, (2,), 3), (1, (8,), 5), (1, (16,), 2), (1, (32,), 7), (1, (256,), 4), (1, (2048,), 3),
    (1, (4096,), 2),
    (2, (4, 4), 2), (2, (8, 16), 1), (2, (16, 8), 3), (2, (32, 32), 2), (2, (64, 128), 1),
    (2, (256, 256), 2), (2, (512, 64), 1), (2, (2048, 2048), 1), (2, (4096, 32), 1),
    (3, (8, 8, 8), 2), (3, (16, 32, 8), 1), (3, (32, 16, 64), 1), (3, (64, 64, 32), 1),
]


@pytest.mark.parametrize("dt,tol", [(np.complex64, 2e-6), (np.complex128, 1e-14)])
@pytest.mark.parametrize("ndim,shape,nf", CASES)
def test_fft_roundtrip_vs_numpy(ndim, shape, nf, dt, tol):
    rng = np.random.default_rng(sum(shape) + nf)
    a = (rng.standard_normal((nf, *shape)) + 1j * rng.standard_normal((nf, *shape))).astype(dt)
    plan = _plan(ndim, shape, nf, 1, dt)
    d = torch.from_numpy(a).cuda()
    plan.fft(d)
    ref = np.fft.fftn(a.astype(np.complex128), axes=tuple(range(-ndim, 0)))
    got = d.cpu().numpy()
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < tol, f"forward rel err {err}"
    plan.ifft(d)
    back = d.cpu().numpy()
    err2 = np.linalg.norm(back - a) / np.linalg.norm(a)
    assert err2 < tol, f"roundtrip rel err {err2}"


def test_fft_two_components_are_independent_transforms():
    rng = np.random.default_rng(5)
    a = (rng.standard_normal((3, 2, 32, 64)) + 1j * rng.standard_normal((3, 2, 32, 64))).astype(
        np.complex64)
    plan = _plan(2, (32, 64), 3, 2, np.complex64)
    d = torch.from_numpy(a).cuda()
    plan.fft(d)
    ref = np.fft.fft2(a.astype(np.complex128))
    assert np.linalg.norm(d.cpu().numpy() - ref) / np.linalg.norm(ref) < 2e-6
