"""Nonlocal response (oaconvolve(|A|^2, nl_profile, "same")) on the GPU."""

import numpy as np
import pytest
from scipy.constants import c, epsilon_0

from tests import cases

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402


def _gauss_kernel(sigma_px: float, half: int) -> np.ndarray:
    r = np.arange(-half, half + 1)
    xx, yy = np.meshgrid(r, r)
    k = np.exp(-(xx**2 + yy**2) / (2 * sigma_px**2))
    return k / k.sum()


def _pair_cnlse(N, dtype, nl_profile, precision):
    """CNLSE with a Gaussian nonlocal kernel (the 1024^2 coupled configuration's physics)."""
    out = []
    for cls in (ng.CNLSE, orc.OracleCNLSE):
        s = cls(20, 0.5, 4 * 1.5e-3, -1.6e-9, -0.8e-9, None, 20e-3, NX=N, NY=N, Isat=1e5,
                nl_length=100e-6)
        s.nl_profile = nl_profile
        s.delta_z = 5e-5
        s.power2 = 0.05
        s.n22 = -1.6e-9
        E = np.array([cases.gaussian(s.XX, s.YY, 1.5e-3), cases.gaussian(s.XX, s.YY, 0.5e-3)])
        out.append((s, E.astype(dtype)))
    (p, E), (o, _) = out
    z = 4e-3
    got = p.out_field(E, z, precision=precision, verbose=False)
    ref, _ = o.out_field(E, z, precision=precision)
    return got, ref, o, E


@pytest.mark.parametrize("precision", ["single", "double"])
def test_cnlse_gaussian_nonlocal_c128(precision):
    N = 128
    dx = 4 * 1.5e-3 / N
    k = _gauss_kernel(100e-6 / dx, 10)
    got, ref, _, _ = _pair_cnlse(N, np.complex128, k, precision)
    assert got.shape == (2, N, N)
    assert cases.rel_l2(got, ref) <= 1e-12


def test_cnlse_gaussian_nonlocal_c64():
    N = 128
    dx = 4 * 1.5e-3 / N
    k = _gauss_kernel(100e-6 / dx, 10)
    got, ref, o, E = _pair_cnlse(N, np.complex64, k, "single")
    o2 = orc.OracleCNLSE(20, 0.5, 4 * 1.5e-3, -1.6e-9, -0.8e-9, None, 20e-3, NX=N, NY=N,
                         Isat=1e5, nl_length=100e-6)
    o2.nl_profile = k
    o2.delta_z, o2.power2, o2.n22 = 5e-5, 0.05, -1.6e-9
    truth, _ = o2.out_field(E.astype(np.complex128), 4e-3)
    e_ref, e_got = cases.rel_l2(ref, truth), cases.rel_l2(got, truth)
    print(f"c64 nonlocal CNLSE error vs FP64: product {e_got:.3e}, reference arithmetic {e_ref:.3e}")
    assert e_got <= max(2 * e_ref, 1e-5)


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, None)])
def test_nlse_1d_and_cnlse_1d_nonlocal(dtype, tol):
    N = 512
    for pcls, ocls, two in ((ng.NLSE_1d, orc.OracleNLSE_1d, False),
                            (ng.CNLSE_1d, orc.OracleCNLSE_1d, True)):
        sims = []
        for cls in (pcls, ocls):
            args = (20, 1.05, 4 * 2.23e-3, -1.6e-9) + ((-1e-10,) if two else ()) + (None, 1e-2)
            s = cls(*args, NX=N, Isat=1e5, nl_length=200e-6)
            s.delta_z = 5e-5
            if two:
                s.power2 = 0.02
            sims.append(s)
        p, o = sims
        E = cases.gaussian(p.X, 0)
        # one field: the reference convolves a single 1-D line (scipy's oaconvolve
        # needs the kernel and the data to have the same number of axes)
        E = np.stack([E, cases.gaussian(p.X, 0, 0.5e-3)]) if two else E
        E = E.astype(dtype)
        got = p.out_field(E, 5e-3, verbose=False)
        ref, _ = o.out_field(E, 5e-3)
        err = cases.rel_l2(got, ref)
        if tol is not None:
            assert err <= tol, (pcls.__name__, err)
        else:
            assert err <= 1e-4, (pcls.__name__, err)


def test_batched_nonlocal_matches_per_field_runs():
    """The engine convolves each field of a batch independently (the reference
    handles one field at a time)."""
    N = 64
    s = ng.NLSE(20, 1.05, 4 * 2.23e-3, -1.6e-9, None, 1e-2, NX=N, NY=N, Isat=1e5, nl_length=300e-6)
    s.delta_z = 1e-4
    E1 = cases.gaussian(s.XX, s.YY).astype(np.complex128)
    E2 = cases.gaussian(s.XX, s.YY, 1.5e-3).astype(np.complex128)
    batch = s.out_field(np.stack([E1, E2]), 5e-3, verbose=False, normalize=False)
    one = s.out_field(E1, 5e-3, verbose=False, normalize=False)
    two = s.out_field(E2, 5e-3, verbose=False, normalize=False)
    assert cases.rel_l2(batch[0], one) < 1e-13 and cases.rel_l2(batch[1], two) < 1e-13


def test_nonlocality_conserves_power():
    """tests/test_nonlocality.py of the reference (alpha = 0, rtol 1e-3), at N = 256."""
    N = 256
    waist, L = 2.23e-3, 1e-3
    s2 = ng.NLSE(0, 1.05, 4 * waist, -1e-9, None, L, NX=N, NY=N, Isat=1e5, nl_length=60e-6 * 8)
    s2.delta_z = 1e-5
    E0 = np.exp(-(s2.XX**2 + s2.YY**2) / waist**2).astype(np.complex64)
    E = s2.out_field(E0, L, verbose=False)
    norm = (np.abs(E) ** 2).sum() * c * epsilon_0 / 2 * s2.delta_X * s2.delta_Y
    assert np.allclose(norm, s2.power, rtol=1e-3)
    g = ng.GPE(0, 1.05, 4 * waist, -1e-9, None, NX=N, NY=N, sat=1e5, nl_length=60e-6 * 8)
    g.delta_z = 1e-5
    E = g.out_field(E0, L, verbose=False)
    assert np.allclose((np.abs(E) ** 2).sum() * g.delta_X * g.delta_Y, g.N, rtol=1e-3)


@pytest.mark.parametrize("cls_name,N", [("CNLSE", 256), ("CNLSE", 512), ("NLSE", 512),
                                        ("CNLSE", 2048)])
def test_fused_nonlocal_passes_match_the_complex128_run(cls_name, N):
    """complex64 fields on padded grids of 512 to 4096 points per axis take the
    fused nonlocal passes (packing + forward rows, columns x kernel spectrum,
    inverse rows + nonlinear step); complex128 fields take the separate passes.
    A few steps from the same input agree to complex64 rounding."""
    waist = 1.5e-3
    dx = 4 * waist / N
    k = _gauss_kernel(100e-6 / dx, 10)  # 21 x 21: padded grid 2N
    outs = {}
    for dt in (np.complex64, np.complex128):
        if cls_name == "CNLSE":
            s = ng.CNLSE(20, 0.5, 4 * waist, -1.6e-9, -0.8e-9, None, 20e-3, NX=N, NY=N, Isat=1e5,
                         nl_length=100e-6)
            s.power2, s.n22 = 0.05, -1.6e-9
            E = np.array([cases.gaussian(s.XX, s.YY, waist), cases.gaussian(s.XX, s.YY, 0.5 * waist)])
        else:
            s = ng.NLSE(20, 1.05, 4 * waist, -1.6e-9, None, 20e-3, NX=N, NY=N, Isat=1e5,
                        nl_length=100e-6)
            E = cases.gaussian(s.XX, s.YY, waist)
        s.nl_profile = k
        s.delta_z = 5e-5
        outs[dt] = s.out_field(E.astype(dt), 4.5 * 5e-5, verbose=False)
    assert cases.rel_l2(outs[np.complex64], outs[np.complex128]) <= 1e-5
