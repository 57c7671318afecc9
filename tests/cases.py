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


_LN2_HI = 6.93147180369123816490e-01  # ln 2 split for Cody-Waite reduction
_LN2_LO = 1.90821492927058770002e-10


def portable_exp(x):
    """exp of a float array, evaluated in float64 with IEEE +, -, *, / and
    ldexp only, so the same bits on every machine.  Library exp differs in
    its last bit between x86 and Arm NumPy builds, and the full-size
    workloads (2048^2, 501 steps) carry such input differences through to
    ~1e-7 in their outputs; fixtures made on one machine are replayed on the
    other.  Cody-Waite reduction x = k ln2 + r, |r| <= ln2 / 2, and the
    degree-13 Taylor polynomial of exp(r) (truncation below 1e-17)."""
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x * 1.4426950408889634)  # x / ln 2
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.ones_like(r)
    for n in range(13, 0, -1):
        p = 1.0 + p * r / n
    out = np.ldexp(p, np.clip(k, -1100, 1100).astype(np.int64))
    return np.where(x < -745.0, 0.0, out)


def gaussian(XX, YY, w=WAIST):
    XX, YY = np.asarray(XX, np.float64), np.asarray(YY, np.float64)
    return portable_exp(-(XX**2 + YY**2) / w**2)


def potential(XX, YY):
    XX, YY = np.asarray(XX, np.float64), np.asarray(YY, np.float64)
    return -1e-4 * portable_exp(-(XX**2 + YY**2) / WAIST2**2)


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


def mixed_batch(groups, seed=0, dtype=np.complex64, cls=None, dz=5e-5):
    """Seeded mixed batch: for each (count, N) a group of `count` fields on an N x N grid.

    Per field (the 164-field configuration's distributions): power ~ U[0.1, 2] W,
    n2 = -10^U[-10, -8.4] m^2/W, waist ~ U[0.8, 2.5] mm, potential = sum of 1-8
    Gaussian wells (depth U[0.5, 2]e-4, width U[30, 150] um, centres uniform in the
    inner half of the window); Isat = 1e5, alpha = 20, L = 10 mm, dz = 5e-5 m.
    Returns [(simulation, E_0)], one simulation per group with per-field
    parameter arrays, as the reference expresses such a batch.
    """
    import nlse_gb300 as ng

    cls = cls or ng.NLSE
    rng = np.random.default_rng(seed)
    jobs = []
    for count, N in groups:
        power = rng.uniform(0.1, 2.0, count)
        n2 = -(10.0 ** rng.uniform(-10, -8.4, count)).reshape(count, 1, 1)
        waist = rng.uniform(0.8e-3, 2.5e-3, count)
        sim = cls(ALPHA, power, WINDOW, n2, None, L, NX=N, NY=N, Isat=ISAT)
        sim.delta_z = dz
        V = np.zeros((count, N, N))
        for b in range(count):
            for _ in range(rng.integers(1, 9)):
                depth = rng.uniform(0.5e-4, 2e-4)
                width = rng.uniform(30e-6, 150e-6)
                x0, y0 = rng.uniform(-WINDOW / 4, WINDOW / 4, 2)
                dx = np.asarray(sim.XX, np.float64) - x0
                dy = np.asarray(sim.YY, np.float64) - y0
                V[b] -= depth * portable_exp(-(dx**2 + dy**2) / width**2)
        sim.V = V.astype(np.float32)
        r2 = np.asarray(sim.XX, np.float64) ** 2 + np.asarray(sim.YY, np.float64) ** 2
        E = portable_exp(-r2[None] / waist[:, None, None] ** 2)
        jobs.append((sim, E.astype(dtype)))
    return jobs


# ---------------------------------------------------------------------------
# the benchmark configurations at their stated sizes (fixtures under
# tests/golden/fullsize/, made by tests/golden/make_parity.py with the
# reference's own classes; the same builders serve the product's tests)
# ---------------------------------------------------------------------------
def nlse2048_inputs(cls, dtype, N=2048, seed=0):
    """The 2048^2 configuration: Gaussian beam times (1 + 0.01 (a + ib)), a, b
    standard normal from default_rng(seed), potential well, dz = 2e-5 m."""
    sim = cls(ALPHA, POWER, WINDOW, N2, None, L, NX=N, NY=N, Isat=ISAT)
    sim.delta_z = 2e-5
    rng = np.random.default_rng(seed)
    E = gaussian(sim.XX, sim.YY)
    E = E * (1 + 0.01 * (rng.standard_normal(E.shape) + 1j * rng.standard_normal(E.shape)))
    sim.V = potential(sim.XX, sim.YY).astype(np.complex64)
    return sim, E.astype(dtype)


def cnlse1024_inputs(cls, dtype, N=1024):
    """The coupled 1024^2 configuration: waists 1.5 / 0.5 mm, powers 0.5 / 0.05 W,
    n2 = n22 = -1.6e-9, n12 = -0.8e-9, Gaussian nonlocal kernel (sigma 100 um on a
    67^2 support, normalised, set through nl_profile), L = 20 mm, dz = 5e-5."""
    sim = cls(ALPHA, 0.5, WINDOW, N2, -0.8e-9, None, 20e-3, NX=N, NY=N, Isat=ISAT,
              nl_length=100e-6)
    sim.delta_z = 5e-5
    sim.power2 = 0.05
    sim.n22 = N2
    r = np.arange(-33, 34) * sim.delta_X
    kern = portable_exp(-(r[:, None] ** 2 + r[None, :] ** 2) / (2 * (100e-6) ** 2))
    sim.nl_profile = kern / kern.sum()
    E = np.array([gaussian(sim.XX, sim.YY, w) for w in (1.5e-3, 0.5e-3)])
    return sim, E.astype(dtype)


MIXED_GROUPS = [(96, 256), (48, 512), (16, 1024), (4, 2048)]
MIXED_SEED = 11


def mixed_field0(cls, dtype, group: int):
    """Field 0 of group `group` of the 164-field batch (mixed_batch, seed 11) as a
    one-field simulation with its per-field arrays: power (1,), n2 (1, 1, 1)
    float64, V (1, N, N)."""
    jobs = mixed_batch(MIXED_GROUPS, seed=MIXED_SEED, dtype=dtype, cls=cls)
    sim_b, E_b = jobs[group]
    N = E_b.shape[-1]
    sim = cls(ALPHA, np.asarray(sim_b.power)[:1], WINDOW, np.asarray(sim_b.n2)[:1], None, L,
              NX=N, NY=N, Isat=ISAT)
    sim.delta_z = sim_b.delta_z
    sim.V = np.asarray(sim_b.V)[:1].copy()
    return sim, E_b[:1].copy()


SAMPLES = 128  # full-size outputs are compared on a SAMPLES x SAMPLES grid


def subsample(E):
    s = E.shape[-1] // SAMPLES
    return np.ascontiguousarray(np.asarray(E)[..., ::s, ::s])


def power_fp64(E):
    e = np.asarray(E).astype(np.complex128)
    return (e.real ** 2 + e.imag ** 2).sum(axis=(-2, -1))
