"""DDGPE noise from the counter-based generator (nlse_add_noise): matches the
oracle's Philox4x32-10 / Box-Muller draws, is reproducible for a (seed, step),
the same for every field of a batch, has the reference's statistics, and runs
inside the DDGPE loop graph with the fused pump exactly as the host loop does."""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import _lib  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402

H = 0.654


def _noise(A, s0, s1, seed, step):
    lib = _lib.load()
    st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    dt = 0 if A.dtype == torch.complex64 else 1
    _lib.check(lib.nlse_add_noise(A.data_ptr(), dt, A.shape[0], A.shape[-1] * A.shape[-2], s0, s1,
                                  seed, step, st), "noise")


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 2e-6), (torch.complex128, 2e-6)])
def test_noise_matches_oracle_and_is_reproducible(dtype, tol):
    B, N, seed = 3, 32, (7 << 32) + 12345
    A = torch.zeros((B, 2, N, N), dtype=dtype, device="cuda")
    _noise(A, 0.5, 2.0, seed, 9)
    got = A.cpu().numpy()
    n0, n1 = orc.ddgpe_noise(N * N, seed, 9)
    ref = np.stack([0.5 * n0.reshape(N, N), 2.0 * n1.reshape(N, N)])
    for b in range(B):
        assert np.abs(got[b] - ref).max() <= tol * np.abs(ref).max()
        assert np.array_equal(got[b], got[0])
    A2 = torch.zeros_like(A)
    _noise(A2, 0.5, 2.0, seed, 9)
    assert torch.equal(A, A2)
    _noise(A2, 0.5, 2.0, seed, 10)
    assert not torch.equal(A, A2 - A)


def test_noise_statistics():
    A = torch.zeros((1, 2, 256, 256), dtype=torch.complex128, device="cuda")
    _noise(A, 3.0, 0.25, 1, 0)
    a = A.cpu().numpy()
    for k, s in ((0, 3.0), (1, 0.25)):
        x = a[0, k]
        assert abs(x.real.mean()) < 0.02 * s and abs(x.imag.mean()) < 0.02 * s
        assert abs(x.real.std() / s - 1) < 0.02 and abs(x.imag.std() / s - 1) < 0.02


def _ddgpe():
    d = ng.DDGPE(gamma=0.07 / H, power=1.0, window=64.0, g=1e-2 / H, omega=5.07 / H, T=2.0,
                 omega_exc=1484.44 / H, omega_cav=1482.76 / H, detuning=0.17 / H, k_z=27.0,
                 NX=32, NY=32)
    d.delta_z = 0.1 / 32
    d.noise_seed = 5
    return d


def _loop(monkeypatch, graph):
    monkeypatch.setenv("NLSE_DEVICE_CALLBACKS", "1" if graph else "0")
    d = _ddgpe()
    n = len(np.arange(0, 2.0, d.delta_z))
    Fr = np.exp(-(d.XX**2 + d.YY**2) / 10.0**2).astype(np.complex64)
    Ft = np.ones(n + 8, dtype=np.complex64)
    Pr = np.zeros_like(Fr)
    Pt = np.zeros_like(Ft)
    E = torch.zeros((2, 32, 32), dtype=torch.complex64, device="cuda")
    norms = np.zeros(n + 8)
    d.out_field(E, 2.0, d.laser_excitation, verbose=False,
                callback=[d.add_noise, ng.norm], callback_args=[[Fr, Ft, Pr, Pt], (0.1,), (1, norms)])
    return norms[:ng.count_steps(2.0, d.delta_z)]


def test_ddgpe_noise_in_the_loop_graph_equals_host_loop(monkeypatch):
    a = _loop(monkeypatch, True)
    b = _loop(monkeypatch, False)
    assert np.array_equal(a, b)
    assert a[-10:].min() > 0


def test_per_field_gamma_scales_the_shared_draws():
    """gamma of shape (B, 1, 1) (the reference broadcasts it against its one
    (NY, NX) draw): every field gets the same draws times its own scale."""
    d = _ddgpe()
    B = 3
    gam = np.array([0.5, 1.0, 2.0]).reshape(B, 1, 1) * d.gamma
    A = torch.zeros((B, 2, 32, 32), dtype=torch.complex128, device="cuda")
    d.gamma = gam
    d._add_noise(A, 4, 0.1)
    got = A.cpu().numpy()
    d.gamma = float(gam[1, 0, 0])
    A1 = torch.zeros((1, 2, 32, 32), dtype=torch.complex128, device="cuda")
    d._add_noise(A1, 4, 0.1)
    one = A1.cpu().numpy()[0]
    for b in range(B):
        scale = np.sqrt(gam[b, 0, 0] / gam[1, 0, 0])
        np.testing.assert_allclose(got[b, 0], scale * one[0], rtol=1e-12, atol=0)
        np.testing.assert_array_equal(got[b, 1], one[1])  # gamma2 is shared
