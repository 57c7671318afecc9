"""The benchmark configurations at their stated sizes against the reference.

Fixtures (tests/golden/fullsize/, tests/golden/make_parity.py) hold the
reference's own outputs on a 128 x 128 subsample grid and the FP64 power of
the whole field:
  nlse2048   2048^2 noisy beam, dz = 2e-5, 501 steps, "single";
  cnlse1024  CNLSE 1024^2, Gaussian nonlocal kernel, 400 steps, "single";
  mixed<N>   field 0 of each grid size of the 164-field batch, 201 steps,
             run here inside the whole batch through out_fields; its n2 and
             power are per-field float64 arrays, so the reference evaluates
             the complex64 nonlinear step in FP64 while the product keeps
             FP32.
Both dtypes are held to the reference's own FFT spread: the fixtures hold the
reference run three times, with scipy's, NumPy's and torch's FFT, and the
product must agree with the scipy run within 2 x the larger of the other two
runs' distances from it (floors: 1e-12 for complex128, 1e-5 for complex64).
The noisy 2048^2 beam is modulationally unstable, so FP64 rounding grows over
its 501 steps (the reference's complex128 runs differ by ~1e-8 from FFT
rounding alone); a fixed 1e-12 would test the FFT library, not the path.
complex64 also keeps its error against the complex128 run within 2x the
reference's own (or 1e-5).
"""

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from tests import cases  # noqa: E402

FULL = Path(__file__).resolve().parent / "golden" / "fullsize"
C128_TOL = 1e-12
SPREAD_SLACK = 2.0
C64_SLACK = 2.0


def _fixture(name):
    p = FULL / f"{name}.npz"
    if not p.exists():
        pytest.skip(f"fixture {p.name} not generated")
    with np.load(p) as z:
        return {k: z[k] for k in z.files}


def _spread(f):
    """How far the reference moves when only its FFT changes (field, power)."""
    ref, pref = f["sub_scipy"], f["power_scipy"]
    if "sub_numpy" not in f:
        return 0.0, 0.0
    field = max(cases.rel_l2(f["sub_numpy"], ref), cases.rel_l2(f["sub_torch"], ref))
    power = max(float(np.max(np.abs(f[k] / pref - 1))) for k in ("power_numpy", "power_torch"))
    return field, power


def _check_c128(tag, got, f):
    sub = cases.subsample(got)
    err = cases.rel_l2(sub, f["sub_scipy"])
    perr = float(np.max(np.abs(cases.power_fp64(got) / f["power_scipy"] - 1)))
    spread, pspread = _spread(f)
    print(f"{tag} complex128: rel-L2 vs reference {err:.2e} (reference FFT spread "
          f"{spread:.2e}), power {perr:.2e} (spread {pspread:.2e})")
    assert err <= max(SPREAD_SLACK * spread, C128_TOL), (err, spread)
    assert perr <= max(SPREAD_SLACK * pspread, C128_TOL), (perr, pspread)


def _check_c64(tag, got, f, f128):
    sub = cases.subsample(got)
    ref = f["sub_scipy"]
    err = cases.rel_l2(sub, ref)
    spread = _spread(f)[0]
    truth = f128["sub_scipy"]
    e64, e64_ref = cases.rel_l2(sub, truth), cases.rel_l2(ref, truth)
    print(f"{tag} complex64: vs reference {err:.2e} (reference FFT spread {spread:.2e}); vs "
          f"complex128 run: product {e64:.2e}, reference {e64_ref:.2e}")
    assert err <= max(SPREAD_SLACK * spread, 1e-5), (err, spread)
    assert e64 <= max(C64_SLACK * e64_ref, 1e-5), (e64, e64_ref)


def _out(sim, E, z):
    return sim.out_field(E, z, precision="single", verbose=False)


def test_nlse_2048_noisy_501_steps():
    f128, f64 = _fixture("nlse2048_c128_single"), _fixture("nlse2048_c64_single")
    sim, E = cases.nlse2048_inputs(ng.NLSE, np.complex128)
    assert ng.count_steps(10e-3, sim.delta_z) == 501
    _check_c128("nlse2048", _out(sim, E, 10e-3), f128)
    sim, E = cases.nlse2048_inputs(ng.NLSE, np.complex64)
    _check_c64("nlse2048", _out(sim, E, 10e-3), f64, f128)


def test_cnlse_1024_gaussian_nonlocal_400_steps():
    f128, f64 = _fixture("cnlse1024_c128_single"), _fixture("cnlse1024_c64_single")
    sim, E = cases.cnlse1024_inputs(ng.CNLSE, np.complex128)
    assert ng.count_steps(20e-3, sim.delta_z) == 400
    _check_c128("cnlse1024", _out(sim, E, 20e-3), f128)
    sim, E = cases.cnlse1024_inputs(ng.CNLSE, np.complex64)
    _check_c64("cnlse1024", _out(sim, E, 20e-3), f64, f128)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_mixed_batch_164_fields_one_field_per_size(dtype):
    """The whole 164-field batch through out_fields; field 0 of each grid size
    against the reference run of that field alone."""
    jobs = cases.mixed_batch(cases.MIXED_GROUPS, seed=cases.MIXED_SEED, dtype=dtype)
    outs = ng.out_fields(jobs, 10e-3)
    for g, (_, N) in enumerate(cases.MIXED_GROUPS):
        got = outs[g][:1]
        f128 = _fixture(f"mixed{N}_c128_single")
        if dtype == np.complex128:
            _check_c128(f"mixed {N}^2", got, f128)
        else:
            _check_c64(f"mixed {N}^2", got, _fixture(f"mixed{N}_c64_single"), f128)
