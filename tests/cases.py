"""Matching product / oracle set-ups for the parity tests.

Physics of the workloads the reference is benchmarked on (the NLSE 2-D
beam with a Gaussian potential well, its noisy large-grid variant, the
coupled two-component case), at sizes the oracle finishes in seconds.
"""

from __future__ import annotations

import numpy as np

from oracle import nlse_oracle as orc

WAIST = 2.23e-3
WAIST2 = 70e-6
WINDOW = 4 * WAIST
POWER = 1.05
N2 = -1.6e-9
ISAT = 1e5
ALPHA = 20
L = 10e-3


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def gaussian(XX, YY, w=WAIST):
    return np.exp(-(XX**2 + YY**2) / w**2)


def potential(XX, YY):
    return -1e-4 * np.exp(-(XX**2 + YY**2) / WAIST2**2)


def nlse_beam(cls, N, dtype=np.complex64, noise=0.0, seed=0, with_v=True, dz=5e-5, batch=None,
              **kw):
    """NLSE 2-D beam (Gaussian, power 1.05 W, n2 = -1.6e-9, Isat = 1e5, alpha = 20)."""
    sim = cls(ALPHA, POWER, WINDOW, N2, None, L, NX=N, NY=N, Isat=ISAT, **kw)
    sim.delta_z = dz
    E = gaussian(sim.XX, sim.YY).astype(np.complex128)
    if noise:
        rng = np.random.default_rng(seed)
        shape = (batch, N, N) if batch else (N, N)
        E = E * (1 + noise * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    elif batch:
        E = np.broadcast_to(E, (batch, N, N)).copy()
    if with_v:
        sim.V = potential(sim.XX, sim.YY).astype(np.complex64)
    return sim, E.astype(dtype)


def oracle_pair(product_cls, oracle_cls, N, **kw):
    p, E = nlse_beam(product_cls, N, **kw)
    o, _ = nlse_beam(oracle_cls, N, **kw)
    return p, o, E


ORACLES = {
    "NLSE": orc.OracleNLSE,
    "NLSE_1d": orc.OracleNLSE_1d,
    "NLSE_3d": orc.OracleNLSE_3d,
    "CNLSE": orc.OracleCNLSE,
    "CNLSE_1d": orc.OracleCNLSE_1d,
    "GPE": orc.OracleGPE,
    "DDGPE": orc.OracleDDGPE,
}
