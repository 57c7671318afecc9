"""Kernel-variant autotuner: every variant of a plan gives the same field up to
complex64 rounding (the kernels contract multiply-adds differently, so not bit
for bit; rel-L2 <= 1e-5 after 7 steps), the tuner picks one of them, caches
it, and reuses the cache."""

import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import _lib, autotune, engine  # noqa: E402
from tests import cases  # noqa: E402


@pytest.mark.parametrize("N,B", [(256, 6), (1024, 2)])
def test_variants_agree_and_tuner_caches(N, B, tmp_path, monkeypatch):
    monkeypatch.setenv("NLSE_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    sim = ng.NLSE(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N, NY=N,
                  Isat=cases.ISAT)
    sim.delta_z = 5e-5
    V = cases.potential(sim.XX, sim.YY).astype(np.float32)
    rng = np.random.default_rng(4)
    E = (cases.gaussian(sim.XX, sim.YY) * (1 + 0.01 * rng.standard_normal((B, N, N)))).astype(
        np.complex64)
    A0 = torch.from_numpy(E).cuda()
    sim.propagator = sim._build_propagator()
    plan = sim._build_fft_plan(A0)[0]
    op = sim._operator(A0, torch.from_numpy(V).cuda(), sim.propagator, "single")
    outs = {}
    for v in autotune.variants(plan):
        plan.set_variant(*v)
        A = A0.clone()
        engine.propagate(plan, A, op, 7, 0, graph=True)
        plan.status()
        outs[v] = A.cpu().numpy()
    # line/tile, TMA, pair, 8-position pair and deep-prefetch pair variants of both passes
    assert len(outs) == 25, sorted(outs)
    base = outs[(_lib.ROWS_TMA, _lib.COLS_TMA)]
    for v, o in outs.items():
        assert cases.rel_l2(o, base) <= 1e-5, v
    rec = autotune.tune(plan, A0, op)
    best = rec["variant"]
    assert (best["rows"], best["cols"]) in set(autotune.variants(plan))
    assert len(rec["ms_per_step"]) >= 25
    data = json.loads((tmp_path / "tune.json").read_text())
    assert data[autotune.plan_key(plan)]["variant"] == best
    plan.set_variant(_lib.ROWS_LINE, _lib.COLS_TILE)
    again = autotune.tune(plan, A0, op)  # from the cache
    assert again == rec
    got = plan.get_variant()
    assert (got["rows"], got["cols"], got["rows_cap"], got["cols_cap"]) == (
        best["rows"], best["cols"], best["rows_cap"], best["cols_cap"])


def test_set_variant_rejects_what_the_plan_lacks():
    dev = torch.device("cuda", 0)
    # complex128 plans have no pair variants
    plan = engine.Plan(2, (256, 256), 2, 1, _lib.NLSE_C128, dev)
    v = plan.get_variant()
    assert _lib.ROWS_PAIR not in v["rows_avail"] and _lib.COLS_PAIR not in v["cols_avail"]
    with pytest.raises(NotImplementedError):
        plan.set_variant(_lib.ROWS_PAIR, _lib.COLS_TMA)
    with pytest.raises(ValueError):
        plan.set_variant(_lib.ROWS_TMA, _lib.COLS_TMA, 40, 0)
