"""The pair passes (two complex64 lines per thread, packed FP32) against the
scalar TMA passes and the oracle, over the cases their code distinguishes:
a potential shared by an even batch (prefetched once per pair), an odd batch
(pairs spanning two rows), per-field and complex potentials, no potential,
rectangular grids, complex (imaginary-time) steps and both schemes.  Short
horizons (6 steps), where complex64 implementations agree to ~1e-6: rel-L2
<= 1e-5 against both."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import _lib, engine  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402
from tests import cases  # noqa: E402

STEPS = 6


def _setup(cls, NY, NX, B, vmode, dz):
    sim = cls(cases.ALPHA, cases.POWER, cases.WINDOW if NX == NY else [cases.WINDOW, cases.WINDOW * NY / NX],
              cases.N2, None, cases.L, NX=NX, NY=NY, Isat=cases.ISAT)
    sim.delta_z = dz
    rng = np.random.default_rng(NX + NY + B)
    E = cases.gaussian(sim.XX, sim.YY)
    shape = (B, NY, NX) if B > 1 else (NY, NX)
    E = (E * (1 + 0.02 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
         ).astype(np.complex64)
    V0 = cases.potential(sim.XX, sim.YY)
    if vmode == "shared":
        sim.V = V0.astype(np.float32)
    elif vmode == "per_field":
        sim.V = (V0[None] * rng.uniform(0.5, 1.5, (B, 1, 1))).astype(np.float32)
    elif vmode == "complex":
        sim.V = (V0 * (1 - 0.2j)).astype(np.complex64)
    else:
        sim.V = None
    return sim, E


CASES = [
    # (NY, NX, fields, potential, dz, scheme)
    (256, 256, 4, "shared", 5e-5, "single"),
    (256, 256, 3, "per_field", 5e-5, "double"),
    (128, 512, 1, "complex", 5e-5, "single"),
    (64, 64, 2, "none", (1 - 0.3j) * 5e-5, "single"),
    (64, 4096, 2, "shared", 5e-5, "double"),
    (2048, 2048, 2, "shared", 2e-5, "single"),
]


@pytest.mark.parametrize("NY,NX,B,vmode,dz,scheme", CASES)
def test_pair_passes_match_scalar_passes_and_oracle(NY, NX, B, vmode, dz, scheme, monkeypatch):
    monkeypatch.setenv("NLSE_AUTOTUNE", "0")
    p, E = _setup(ng.NLSE, NY, NX, B, vmode, dz)
    o, _ = _setup(orc.OracleNLSE, NY, NX, B, vmode, dz)
    z = (STEPS - 0.5) * abs(dz)
    plan = engine.Plan.get(2, (NY, NX), B, 1, _lib.NLSE_C64, torch.device("cuda", 0))
    avail = plan.get_variant()
    assert {_lib.ROWS_PAIR, _lib.ROWS_PAIR8, _lib.ROWS_DEEP} <= set(avail["rows_avail"])
    assert {_lib.COLS_PAIR, _lib.COLS_PAIR8, _lib.COLS_DEEP} <= set(avail["cols_avail"])
    outs = {}
    for v in ((_lib.ROWS_PAIR, _lib.COLS_PAIR), (_lib.ROWS_TMA, _lib.COLS_TMA),
              (_lib.ROWS_PAIR, _lib.COLS_TMA), (_lib.ROWS_TMA, _lib.COLS_PAIR),
              (_lib.ROWS_PAIR8, _lib.COLS_PAIR8), (_lib.ROWS_PAIR8, _lib.COLS_PAIR),
              (_lib.ROWS_DEEP, _lib.COLS_DEEP)):
        plan.set_variant(*v)
        outs[v] = p.out_field(E, z, precision=scheme, verbose=False)
        plan.status()
    plan.set_variant(_lib.ROWS_PAIR, _lib.COLS_PAIR)
    ref, n = o.out_field(E, z, precision=scheme)
    assert n == STEPS
    pair = outs[(_lib.ROWS_PAIR, _lib.COLS_PAIR)]
    e_ref = cases.rel_l2(pair, ref)
    e_scalar = cases.rel_l2(pair, outs[(_lib.ROWS_TMA, _lib.COLS_TMA)])
    print(f"{NY}x{NX} B={B} V={vmode} dz={dz} {scheme}: pair vs oracle {e_ref:.2e}, "
          f"vs scalar passes {e_scalar:.2e}")
    # the deep-prefetch forms run the same arithmetic with another copy schedule
    assert cases.rel_l2(outs[(_lib.ROWS_DEEP, _lib.COLS_DEEP)], pair) <= 1e-6
    assert e_ref <= 1e-5 and e_scalar <= 1e-5
    for v, out in outs.items():
        assert cases.rel_l2(out, ref) <= 1e-5, v
