"""Whole propagations across grid geometries against the oracle.

Every geometry path of the engine -- tiny grids, rectangular and strongly
non-square 2-D grids (TMA-fed persistent passes and one CTA per line or
tile, several lines per CTA for short rows), batches with per-field
parameters, 1-D lengths and 3-D boxes: complex128 within 1e-12 of the oracle
("single" and "double"); complex64 within 1e-5 of the oracle's FP64 run of
the same input over the same few steps.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402
from tests.cases import rel_l2  # noqa: E402
from tests.golden_cases import ALPHA, ISAT, L, N2, POWER, WAIST, WAIST2, WINDOW  # noqa: E402

DZ, STEPS = 5e-5, 6


def _beam(cls, NY, NX, batch, dtype, seed):
    window = WINDOW if NY == NX else [WINDOW, WINDOW * NY / NX]
    power = POWER if not batch else np.linspace(0.5, 2.0, batch)
    n2 = N2 if not batch else np.linspace(-1.6e-9, -4e-10, batch).reshape(batch, 1, 1)
    s = cls(ALPHA, power, window, n2, None, L, NX=NX, NY=NY, Isat=ISAT)
    s.delta_z = DZ
    rng = np.random.default_rng(seed)
    shape = (batch, NY, NX) if batch else (NY, NX)
    E = np.exp(-(s.XX**2 + s.YY**2) / WAIST**2) * (
        1 + 0.01 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    s.V = (-1e-4 * np.exp(-(s.XX**2 + s.YY**2) / WAIST2**2)).astype(np.complex64)
    return s, E.astype(dtype)


SHAPES_2D = [(2, 2, None), (4, 8, 2), (8, 4, None), (16, 16, 3), (32, 64, None), (64, 32, 2),
             (128, 512, None), (512, 128, None), (256, 1024, 2), (64, 4096, None),
             (4096, 64, None), (2048, 2048, None)]


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("NY,NX,batch", SHAPES_2D)
def test_2d_geometry_c128(NY, NX, batch, precision):
    p, E = _beam(ng.NLSE, NY, NX, batch, np.complex128, NY + NX)
    o, _ = _beam(orc.OracleNLSE, NY, NX, batch, np.complex128, NY + NX)
    z = STEPS * DZ
    got = p.out_field(E, z, precision=precision, verbose=False)
    ref, _ = o.out_field(E, z, precision=precision)
    assert got.shape == ref.shape
    assert rel_l2(got, ref) <= 1e-12


@pytest.mark.parametrize("NY,NX,batch", SHAPES_2D)
def test_2d_geometry_c64(NY, NX, batch):
    p, E = _beam(ng.NLSE, NY, NX, batch, np.complex64, NY + NX + 1)
    o, _ = _beam(orc.OracleNLSE, NY, NX, batch, np.complex128, NY + NX + 1)
    z = STEPS * DZ
    got = p.out_field(E, z, verbose=False)
    ref, _ = o.out_field(E.astype(np.complex128), z)
    assert got.dtype == np.complex64
    assert rel_l2(got, ref) <= 1e-5


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("NX,batch", [(2, None), (8, 3), (64, None), (512, 2), (4096, None)])
def test_1d_lengths_c128(NX, batch, precision):
    out = []
    for cls in (ng.NLSE_1d, orc.OracleNLSE_1d):
        s = cls(ALPHA, POWER if not batch else np.linspace(0.5, 2.0, batch), WINDOW, N2, None, L,
                NX=NX, Isat=ISAT)
        s.delta_z = DZ
        s.V = (-1e-4 * np.exp(-s.X**2 / WAIST2**2)).astype(np.complex64)
        E = np.exp(-s.X**2 / WAIST**2).astype(np.complex128)
        if batch:
            E = np.broadcast_to(E, (batch, NX)).copy()
        out.append((s, E))
    (p, E), (o, _) = out
    got = p.out_field(E, STEPS * DZ, precision=precision, verbose=False)
    ref, _ = o.out_field(E, STEPS * DZ, precision=precision)
    assert rel_l2(got, ref) <= 1e-12


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("NY,NX,NZ", [(4, 4, 4), (8, 16, 4), (16, 8, 32), (32, 32, 16)])
def test_3d_boxes_c128(NY, NX, NZ, precision):
    out = []
    for cls in (ng.NLSE_3d, orc.OracleNLSE_3d):
        s = cls(alpha=ALPHA, energy=1.05 * 2e-6, window=np.array([WINDOW, 16e-6]), n2=N2,
                D0=1e-16, vg=3e7, V=None, L=L, NX=NX, NY=NY, NZ=NZ, Isat=ISAT)
        s.delta_z = 2.5e-4
        E = (np.exp(-(s.XX**2 + s.YY**2) / WAIST**2) * np.exp(-s.TT**2 / (4e-6) ** 2))
        out.append((s, E.astype(np.complex128)))
    (p, E), (o, _) = out
    got = p.out_field(E, 3 * 2.5e-4, precision=precision, verbose=False)
    ref, _ = o.out_field(E, 3 * 2.5e-4, precision=precision)
    assert got.shape == (NY, NX, NZ)
    assert rel_l2(got, ref) <= 1e-12


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("omega", [None, 2e3])
@pytest.mark.parametrize("NY,NX", [(8, 8), (16, 64), (64, 16), (256, 256), (128, 1024),
                                   (1024, 1024)])
def test_cnlse_geometry_c128(NY, NX, omega, precision):
    out = []
    for cls in (ng.CNLSE, orc.OracleCNLSE):
        window = WINDOW if NY == NX else [WINDOW, WINDOW * NY / NX]
        s = cls(ALPHA, 0.5, window, N2, -0.8e-9, None, 20e-3, NX=NX, NY=NY, Isat=ISAT,
                omega=omega)
        s.delta_z = DZ
        s.power2 = 0.05
        s.n22 = -1.2e-9
        s.k2 = 2 * np.pi / 795e-9
        s.V = (-1e-4 * np.exp(-(s.XX**2 + s.YY**2) / WAIST2**2)).astype(np.complex64)
        E = np.array([np.exp(-(s.XX**2 + s.YY**2) / w**2) for w in (1.5e-3, 0.5e-3)])
        out.append((s, E.astype(np.complex128)))
    (p, E), (o, _) = out
    got = p.out_field(E, STEPS * DZ, precision=precision, verbose=False)
    ref, _ = o.out_field(E, STEPS * DZ, precision=precision)
    assert got.shape == (2, NY, NX)
    assert rel_l2(got, ref) <= 1e-12


@pytest.mark.parametrize("NX", [4, 64, 2048])
def test_cnlse_1d_lengths_c128(NX):
    out = []
    for cls in (ng.CNLSE_1d, orc.OracleCNLSE_1d):
        s = cls(ALPHA, POWER, WINDOW, N2, -1e-10, None, L, NX=NX, Isat=ISAT)
        s.delta_z = DZ
        s.power2 = 10e-3
        E = np.array([np.exp(-s.X**2 / w**2) for w in (WAIST, WAIST / 2)])
        out.append((s, E.astype(np.complex128)))
    (p, E), (o, _) = out
    got = p.out_field(E, STEPS * DZ, verbose=False)
    ref, _ = o.out_field(E, STEPS * DZ)
    assert rel_l2(got, ref) <= 1e-12
