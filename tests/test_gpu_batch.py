"""Mixed batches (different grid sizes and per-field parameters) in one graph launch."""

import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402

GROUPS = [(6, 64), (4, 128), (2, 256), (1, 512)]


def test_out_fields_equals_separate_out_field_calls():
    jobs = cases.mixed_batch(GROUPS, seed=3)
    together = ng.out_fields(jobs, 2e-3)
    for (sim, E), got in zip(cases.mixed_batch(GROUPS, seed=3), together):
        alone = sim.out_field(E, 2e-3, verbose=False)
        assert got.shape == E.shape
        assert np.array_equal(got, alone)


def test_out_fields_replays_and_matches_oracle_c128():
    jobs = cases.mixed_batch([(3, 64), (2, 128)], seed=5, dtype=np.complex128)
    first = ng.out_fields(jobs, 2e-3)
    again = ng.out_fields(jobs, 2e-3)  # the captured graph is replayed
    for a, b in zip(first, again):
        assert np.array_equal(a, b)
    for (sim, E), got in zip(jobs, first):
        o = orc.OracleNLSE(cases.ALPHA, sim.power, cases.WINDOW, sim.n2, None, cases.L,
                           NX=sim.NX, NY=sim.NY, Isat=cases.ISAT)
        o.delta_z = sim.delta_z
        o.V = sim.V
        ref, _ = o.out_field(E, 2e-3)
        assert cases.rel_l2(got, ref) <= 1e-12
