"""Imaginary-time / complex delta_z (NLSE/nlse.py:505-508, 568-569): the
propagator and the nonlinear factor take the complex step as the reference
does; checked against the oracle (complex128: rel-L2 <= 1e-12)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402
from tests import cases  # noqa: E402
from tests import golden_cases as gc  # noqa: E402


@pytest.mark.parametrize("N", [64, 256])
@pytest.mark.parametrize("dz,precision", [(-1j * 5e-5, "double"), ((1 - 0.3j) * 5e-5, "single")])
def test_nlse_complex_step_matches_oracle(N, dz, precision):
    p, o, E = cases.oracle_pair(ng.NLSE, orc.OracleNLSE, N, dtype=np.complex128)
    for s in (p, o):
        s.delta_z = dz
    z = 20 * 5e-5
    got = p.out_field(E, z, precision=precision, verbose=False)
    ref, n = o.out_field(E, z, precision=precision)
    assert n == 20
    assert cases.rel_l2(got, ref) <= 1e-12


def test_nlse_complex_step_complex64():
    p, o, E = cases.oracle_pair(ng.NLSE, orc.OracleNLSE, 128, dtype=np.complex64)
    for s in (p, o):
        s.delta_z = -1j * 5e-5
    got = p.out_field(E, 20 * 5e-5, precision="double", verbose=False)
    ref, _ = o.out_field(E, 20 * 5e-5, precision="double")
    assert cases.rel_l2(got, ref) <= 1e-5


def test_nlse_1d_and_cnlse_complex_step():
    kw = dict(NX=256, Isat=cases.ISAT)
    p = ng.NLSE_1d(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, **kw)
    o = orc.OracleNLSE_1d(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, **kw)
    E = np.exp(-(p.X**2) / cases.WAIST**2).astype(np.complex128)
    for s in (p, o):
        s.delta_z = -1j * 5e-5
    got = p.out_field(E, 20 * 5e-5, verbose=False)
    ref, _ = o.out_field(E, 20 * 5e-5)
    assert cases.rel_l2(got, ref) <= 1e-12
    kw = dict(NX=32, NY=32, Isat=cases.ISAT)
    p = ng.CNLSE(cases.ALPHA, 0.5, cases.WINDOW, cases.N2, -0.8e-9, None, 20e-3, **kw)
    o = orc.OracleCNLSE(cases.ALPHA, 0.5, cases.WINDOW, cases.N2, -0.8e-9, None, 20e-3, **kw)
    E = np.stack([cases.gaussian(p.XX, p.YY), 0.3 * cases.gaussian(p.XX, p.YY)]).astype(
        np.complex128)
    for s in (p, o):
        s.delta_z = (1 - 0.5j) * 5e-5
    got = p.out_field(E, 20 * 5e-5, verbose=False)
    ref, _ = o.out_field(E, 20 * 5e-5)
    assert cases.rel_l2(got, ref) <= 1e-12


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
def test_rabi_coupling_with_complex_step(dtype, tol):
    """The Rabi rotation with the complex cosine and sine of (omega/2) dz, as the
    reference's rabi_coupling on a complex step (kernels_gpu.py:155-156)."""
    kw = dict(NX=32, NY=32, Isat=cases.ISAT, omega=2e3)
    p = ng.CNLSE(cases.ALPHA, 0.5, cases.WINDOW, cases.N2, -0.8e-9, None, 20e-3, **kw)
    o = orc.OracleCNLSE(cases.ALPHA, 0.5, cases.WINDOW, cases.N2, -0.8e-9, None, 20e-3, **kw)
    E = np.stack([cases.gaussian(p.XX, p.YY), 0.3 * cases.gaussian(p.XX, p.YY)]).astype(dtype)
    for s in (p, o):
        s.delta_z = (1 - 0.4j) * 5e-5
    got = p.out_field(E, 20 * 5e-5, verbose=False)
    ref, _ = o.out_field(E, 20 * 5e-5)
    assert cases.rel_l2(got, ref) <= tol


def _ddgpe():
    H = 0.654
    return ng.DDGPE(gamma=0.07 / H, power=1.0, window=64.0, g=1e-2 / H, omega=5.07 / H, T=2.0,
                    omega_exc=1484.44 / H, omega_cav=1482.76 / H, detuning=0.17 / H, k_z=27.0,
                    NX=32, NY=32)


@pytest.mark.parametrize("fused", [True, False])
def test_ddgpe_complex_step_matches_the_reference(fused):
    """DDGPE (pump, probe, potential, Rabi coupling) with a complex step against
    the reference's own complex128 result (ddgpe_c128_single_V_cdz): the
    source term's complex product F dz i in the row pass (fused) or in the
    host callback."""
    f = gc.load("ddgpe_c128_single_V_cdz")
    d = _ddgpe()
    d.delta_z = complex(f["dz"][()])
    d.V = f["V"].copy()
    final = {}

    def grab(simu, A, z, i):
        final["A"] = A.clone()

    cb = d.laser_excitation if fused else (lambda *a: ng.DDGPE.laser_excitation(*a))
    d.out_field(f["E_in"].copy(), 2.0, cb, verbose=False, callback=[grab],
                callback_args=[[f["Fr"], f["Ft"], f["Pr"], f["Pt"]], []])
    assert cases.rel_l2(final["A"].cpu().numpy(), f["out"]) <= 1e-12


def test_ddgpe_noise_with_complex_step_raises_like_the_reference():
    """add_noise draws with scale = delta_z (ddgpe.py:114-119): a complex step
    is rejected there, as NumPy's and CuPy's normal reject a complex scale."""
    d = _ddgpe()
    d.delta_z = (1 - 0.3j) * 0.1 / 32
    A = torch.zeros((2, 32, 32), dtype=torch.complex64, device="cuda")
    with pytest.raises(TypeError):
        ng.DDGPE.add_noise(d, A, 0.0, 0, noise=1.0)
