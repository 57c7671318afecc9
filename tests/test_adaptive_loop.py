"""The z-loop with adapt_delta_z (callbacks.run_adaptive) against the
reference's loop semantics, on the CPU with a fake engine.

The reference loop (NLSE/nlse.py:570-586) runs split_step, then the
callbacks, then z_prop += delta_z, while abs(z_prop) < z; adapt_delta_z
(NLSE/callbacks.py:85-112) appends delta_z every step and, every
update_every steps, sets delta_z = |1 / (k * peak)| / 12 from the field the
step left.  run_adaptive runs the steps between updates as device segments
and reads the peak once per update; with the engine faked (known peaks per
step) its recorded steps, step count, parameter refreshes and other
callbacks' record steps must equal the restated loop's exactly.
"""

import numpy as np
import pytest
import torch

from nlse_gb300 import callbacks as cb


class _Simu:
    def __init__(self, dz, k):
        self.delta_z, self.k = dz, k


class _Op:
    pump = None


def _peak(i):
    return np.float64(1e-4 * (1.0 + 0.3 * np.sin(0.7 * i)))


def _reference(z, dz0, u, k, every=None):
    dzs, recs, delta_z, z_prop, i = [], [], dz0, 0, 0
    while abs(z_prop) < z:
        if every and i % every == 0:
            recs.append(i)
        dzs.append(delta_z)
        if i % u == 0:
            delta_z = np.abs(float(1 / (k * _peak(i)))) / 12
        z_prop += delta_z
        i += 1
    return dzs, i, recs


@pytest.mark.parametrize("z,dz0,u,every", [(2e-3, 5e-5, 4, None), (3e-3, 2e-5, 1, 3),
                                           (1e-3, 1e-4, 7, 2), (5e-4, 6e-4, 3, None),
                                           (4e-3, 3e-5, 10, 5)])
def test_adaptive_loop_follows_the_reference(monkeypatch, z, dz0, u, every):
    k = 2 * np.pi / 780e-9
    state = {"steps": 0, "refresh": 0, "recs": []}

    def fake_propagate(plan, A, op, n, step0=0, graph=False):
        assert n > 0
        state["steps"] += n

    def fake_max(A, pix, n2a, isat, c, eps0, flags, out):
        out.fill_(float(_peak(state["steps"] - 1)))  # the field of the last step taken

    def fake_record(kind, A, st):
        state["recs"].append(state["steps"] - 1)
        return torch.zeros(())

    monkeypatch.setattr(cb.engine, "propagate", fake_propagate)
    monkeypatch.setattr(cb.engine, "delta_n_max", fake_max)
    monkeypatch.setattr(cb, "_record", fake_record)
    monkeypatch.setattr(cb, "index_change_setup",
                        lambda simu, A, adapt: (4, None, None, 1, torch.float64))

    def refresh():
        state["refresh"] += 1

    simu = _Simu(dz0, k)
    dzs = []
    recs = [("adapt", u, dzs)]
    sink = {}
    if every:
        recs.insert(0, ("norm", every, sink))
    A = torch.zeros(4, dtype=torch.complex64)
    assert cb.run_adaptive(simu, None, A, _Op(), z, recs, refresh)
    ref_dzs, ref_n, ref_recs = _reference(z, dz0, u, k, every)
    assert state["steps"] == ref_n
    assert dzs == ref_dzs  # the same values in the same order
    assert state["refresh"] == len(range(0, ref_n, u))
    assert state["recs"] == ref_recs
    assert sorted(sink) == [r // every for r in ref_recs] if every else not sink
