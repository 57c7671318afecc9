"""A mixed batch as two launches per step (one column pass and one row pass
over every grid size) against the per-instance branches and the oracle.

The 164-field configuration's distributions (tests/cases.py mixed_batch) at
reduced counts, complex64, 20 steps: the fused path must be taken, agree
with the branch path to complex64 rounding (rel-L2 <= 1e-5: different kernels
contract multiply-adds differently) and, field 0 of every grid size, with
the oracle to 1e-5 (short horizon)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import batch  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402
from tests import cases  # noqa: E402

GROUPS = [(6, 256), (3, 512), (2, 1024), (1, 2048)]
Z = 19.5 * 5e-5  # 20 steps


def _jobs():
    return cases.mixed_batch(GROUPS, seed=5)


def test_fused_batch_matches_branches_and_oracle(monkeypatch):
    monkeypatch.setenv("NLSE_AUTOTUNE", "0")
    jobs = _jobs()
    fused = ng.out_fields(jobs, Z)
    assert batch.last_fused
    monkeypatch.setenv("NLSE_GROUP_FUSED", "0")
    jobs2 = _jobs()
    branches = ng.out_fields(jobs2, Z)
    assert not batch.last_fused
    for (sim, E), f, b in zip(jobs, fused, branches):
        assert f.shape == E.shape and f.dtype == np.complex64
        err = cases.rel_l2(f, b)
        # field 0 against the oracle, built with that field's parameters
        N = E.shape[-1]
        o = orc.OracleNLSE(cases.ALPHA, np.asarray(sim.power)[:1], cases.WINDOW,
                           np.asarray(sim.n2)[:1], None, cases.L, NX=N, NY=N, Isat=cases.ISAT)
        o.delta_z = sim.delta_z
        o.V = np.asarray(sim.V)[:1].copy()
        ref, n = o.out_field(E[:1].copy(), Z)
        assert n == 20
        e_ref = cases.rel_l2(f[:1], ref)
        print(f"{E.shape}: fused vs branches {err:.2e}, fused vs oracle {e_ref:.2e}")
        assert err <= 1e-5 and e_ref <= 1e-5


def test_fused_batch_replays_identically():
    jobs = _jobs()
    a = ng.out_fields(jobs, Z)
    b = ng.out_fields(jobs, Z)
    assert batch.last_fused
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
