"""The bench workload at full size (8 fields of 2048 x 2048), through properties
that do not need an oracle run of the whole batch: fields of a batch do not
interact (each equals its own single-field run bit for bit), the replayed CUDA
graph equals the same passes launched one by one, power is conserved without
loss (the reference's KAT, rtol 1e-4), and a few complex128 steps match the
oracle to 1e-12."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import _lib, engine  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402
from tests import cases  # noqa: E402

N, B, DZ = 2048, 8, 2e-5


def _setup(nfields, dtype=np.complex64, alpha=cases.ALPHA, seed=1000):
    sim = ng.NLSE(alpha, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N, NY=N,
                  Isat=cases.ISAT)
    sim.delta_z = DZ
    V = cases.potential(sim.XX, sim.YY).astype(np.float32)
    sim.V = V
    rng = np.random.default_rng(seed)
    E = cases.gaussian(sim.XX, sim.YY)
    a = rng.standard_normal((nfields, N, N))
    b = rng.standard_normal((nfields, N, N))
    E = (E * (1 + 0.01 * (a + 1j * b))).astype(dtype)
    return sim, E, V


def _engine(sim, A, V):
    sim.propagator = sim._build_propagator()
    plan = sim._build_fft_plan(A)[0]
    op = sim._operator(A, torch.from_numpy(V).cuda(), sim.propagator, "single")
    return plan, op


def test_batch_fields_equal_their_single_field_runs(monkeypatch):
    # one kernel variant for both plans: the autotuner may pick different ones for
    # 8 fields and for 1, and variants agree only to rounding
    monkeypatch.setenv("NLSE_AUTOTUNE", "0")
    sim, E, V = _setup(B)
    z = 19.5 * DZ
    out = sim.out_field(torch.from_numpy(E).cuda(), z, verbose=False)
    for k in (0, B - 1):
        s1, _, _ = _setup(1)
        one = s1.out_field(torch.from_numpy(E[k:k + 1]).cuda(), z, verbose=False)
        assert torch.equal(out[k:k + 1], one)


def test_graph_replay_equals_pass_by_pass_launches():
    sim, E, V = _setup(B)
    A0 = torch.from_numpy(E).cuda()
    plan, op = _engine(sim, A0, V)
    n = 12
    A1 = A0.clone()
    engine.propagate(plan, A1, op, n, 0, graph=True)
    A2 = A0.clone()
    engine.run_pass(plan, A2, op, _lib.PASS_FORWARD, 0)
    for s in range(n):
        engine.run_pass(plan, A2, op, _lib.PASS_LINEAR, s)
        engine.run_pass(plan, A2, op, _lib.PASS_INV_NL_FWD if s < n - 1 else _lib.PASS_INV_NL, s)
    torch.cuda.synchronize()
    plan.status()  # raises if a bounded wait gave up
    assert torch.equal(A1, A2)


def test_power_conserved_without_loss_at_full_size():
    sim, E, V = _setup(2, alpha=0)
    out = sim.out_field(torch.from_numpy(E).cuda(), 99.5 * DZ, verbose=False)
    p = engine.power(out.contiguous(), 2).cpu().numpy()
    p0 = engine.power(torch.from_numpy(E).cuda(), 2).cpu().numpy()
    # out_field normalises E to the set power first: compare against that
    target = cases.POWER / sim._norm_coef()
    np.testing.assert_allclose(p, target, rtol=1e-4)
    assert np.all(p0 > 0)


def test_complex128_steps_match_oracle_at_full_size():
    sim, E, V = _setup(1, dtype=np.complex128)
    o = orc.OracleNLSE(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N, NY=N,
                       Isat=cases.ISAT)
    o.delta_z = DZ
    o.V = V
    z = 2.5 * DZ
    got = sim.out_field(E, z, verbose=False)
    ref, n = o.out_field(E, z)
    assert n == 3
    assert cases.rel_l2(got, ref) <= 1e-12
