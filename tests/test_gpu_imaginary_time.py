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


def test_complex_step_rejected_where_unsupported():
    cn = ng.CNLSE(cases.ALPHA, 0.5, cases.WINDOW, cases.N2, -0.8e-9, None, 20e-3, NX=32, NY=32,
                  omega=1e3)
    cn.delta_z = -1j * 5e-5
    E = np.stack([cases.gaussian(cn.XX, cn.YY)] * 2).astype(np.complex128)
    with pytest.raises(NotImplementedError):
        cn.out_field(E, 5e-4, verbose=False)
