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
from nlse_gb300 import autotune, engine  # noqa: E402
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
    outs = []
    for v in autotune.variants(plan):
        plan.set_kernels(*v)
        A = A0.clone()
        engine.propagate(plan, A, op, 7, 0, graph=True)
        outs.append(A)
    assert len(outs) >= 2
    for o in outs[1:]:
        assert cases.rel_l2(o.cpu().numpy(), outs[0].cpu().numpy()) <= 1e-5
    rec = autotune.tune(plan, A0, op)
    assert tuple(rec["variant"]) in set(autotune.variants(plan))
    data = json.loads((tmp_path / "tune.json").read_text())
    assert data[autotune.plan_key(plan)]["variant"] == rec["variant"]
    plan.set_kernels(False, False)
    again = autotune.tune(plan, A0, op)  # from the cache
    assert again == rec and plan.get_kernels()[:2] == tuple(rec["variant"])
