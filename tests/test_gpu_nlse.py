"""NLSE family on the GPU against the oracle and the reference's known answers."""

import numpy as np
import pytest
from scipy.constants import c, epsilon_0

from tests import cases

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402

C64_TOL = 1e-5   # rel-L2, complex64 field, "single" scheme
C128_TOL = 1e-12  # rel-L2, complex128 field, "double" scheme


def _run_pair(N, dtype, precision, z=cases.L, **kw):
    p, o, E = cases.oracle_pair(ng.NLSE, orc.OracleNLSE, N, dtype=dtype, **kw)
    got = p.out_field(E, z, precision=precision, verbose=False)
    ref, n = o.out_field(E, z, precision=precision)
    return got, ref, n, p


@pytest.mark.parametrize("N", [64, 256])
def test_nlse_c64_single_matches_oracle(N):
    got, ref, n, _ = _run_pair(N, np.complex64, "single")
    assert n == 201
    assert got.dtype == np.complex64 and got.shape == (N, N)
    err = cases.rel_l2(got, ref)
    assert err <= C64_TOL, err


@pytest.mark.parametrize("N", [64, 256])
def test_nlse_c128_double_matches_oracle(N):
    got, ref, n, _ = _run_pair(N, np.complex128, "double")
    err = cases.rel_l2(got, ref)
    assert err <= C128_TOL, err


def test_nlse_c64_double_and_c128_single():
    got, ref, _, _ = _run_pair(128, np.complex64, "double")
    assert cases.rel_l2(got, ref) <= C64_TOL
    got, ref, _, _ = _run_pair(128, np.complex128, "single")
    assert cases.rel_l2(got, ref) <= C128_TOL


def test_nlse_noisy_field_without_potential():
    got, ref, n, _ = _run_pair(128, np.complex64, "single", noise=0.01, with_v=False, dz=2e-5)
    assert n == 501
    assert cases.rel_l2(got, ref) <= C64_TOL


def test_split_step_identity_at_zero_dz():
    """tests/test_nlse.py:243-282 of the reference: dz = 0, E = 1, double scheme."""
    N = 256
    simu = ng.NLSE(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N, NY=N,
                   Isat=cases.ISAT)
    simu.delta_z = 0
    simu.propagator = simu._build_propagator()
    E = np.ones((N, N), dtype=np.complex64)
    A, A_sq = simu._prepare_output_array(E, normalize=False)
    simu.plans = simu._build_fft_plan(A)
    simu._send_arrays_to_gpu()
    simu.split_step(A, A_sq, simu.V, simu.propagator, simu.plans, precision="double")
    assert torch.allclose(A, torch.ones_like(A))


def test_out_field_conserves_power_without_loss():
    """tests/test_nlse.py:287-311 of the reference at N = 256."""
    N = 256
    E = np.ones((N, N), dtype=np.complex64)
    simu = ng.NLSE(0, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N, NY=N,
                   Isat=cases.ISAT)
    E = simu.out_field(E, cases.L, verbose=False, plot=False, precision="single")
    norm = np.sum(np.abs(E) ** 2 * simu.delta_X * simu.delta_Y) * c * epsilon_0 / 2
    assert E.shape == (N, N)
    assert np.allclose(norm, simu.power, rtol=1e-4)


def test_prepare_output_array_normalises():
    N = 128
    simu = ng.NLSE(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N, NY=N,
                   Isat=cases.ISAT)
    rng = np.random.default_rng(1)
    E = (rng.random((N, N)) + 1j * rng.random((N, N))).astype(np.complex64)
    A, A_sq = simu._prepare_output_array(E, normalize=True)
    assert A.is_contiguous() and A_sq.is_contiguous()
    a = A.cpu().numpy()
    integral = (np.abs(a) ** 2 * simu.delta_X * simu.delta_Y).sum() * c * epsilon_0 / 2
    assert np.allclose(integral, simu.power)
    assert np.allclose(a / np.abs(a).max(), E / np.abs(E).max(), atol=1e-6)


def test_callbacks_path_matches_fused_path():
    N = 128
    p1, E = cases.nlse_beam(ng.NLSE, N)
    p2, _ = cases.nlse_beam(ng.NLSE, N)
    norms = np.zeros(201)
    a = p1.out_field(E, cases.L, verbose=False)
    b = p2.out_field(E, cases.L, verbose=False, callback=ng.norm, callback_args=(1, norms))
    assert cases.rel_l2(a, b) < 1e-6
    assert np.all(np.diff(norms) < 0)  # lossy medium: the norm decreases every step


def test_broadcast_fields_with_per_field_parameters():
    """Batch of fields with n2 of shape (B, 1, 1) and power of shape (B,)."""
    N, B = 64, 3
    n2 = np.array([-1.6e-9, -1e-9, -4e-10]).reshape(B, 1, 1)
    power = np.array([1.05, 0.5, 2.0])
    p = ng.NLSE(cases.ALPHA, power, cases.WINDOW, n2, None, cases.L, NX=N, NY=N, Isat=cases.ISAT)
    o = orc.OracleNLSE(cases.ALPHA, power, cases.WINDOW, n2, None, cases.L, NX=N, NY=N,
                       Isat=cases.ISAT)
    for s in (p, o):
        s.delta_z = 5e-5
        s.V = cases.potential(s.XX, s.YY).astype(np.complex64)
    E = np.broadcast_to(cases.gaussian(p.XX, p.YY), (B, N, N)).astype(np.complex64)
    got = p.out_field(E, cases.L, verbose=False)
    ref, _ = o.out_field(E, cases.L)
    assert got.shape == (B, N, N)
    # the reference computes the nonlinear phase in FP64 when n2 is an FP64 array
    assert cases.rel_l2(got, ref) <= 1e-5


def test_torch_input_returns_torch():
    N = 64
    p, E = cases.nlse_beam(ng.NLSE, N)
    out = p.out_field(torch.from_numpy(E).cuda(), cases.L, verbose=False)
    assert isinstance(out, torch.Tensor) and out.is_cuda
