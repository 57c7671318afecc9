"""Which callback lists run on the device (callbacks.device_plan), on the CPU:
the reference's norm / sample / evaluate_delta_n / adapt_delta_z become
device work, anything else keeps the per-step host loop, and so do lists the
device forms cannot express (two adaptive steps, an adaptive step with DDGPE
noise, malformed arguments) or NLSE_DEVICE_CALLBACKS=0."""

import numpy as np
import pytest

import nlse_gb300 as ng
from nlse_gb300 import callbacks as cb


class _Simu:
    pass


class _Noisy:
    def add_noise(self, simu, A, z, i, amp=0.0):
        pass

    def _add_noise(self, A, step, amp):
        pass

    def _noise_sigmas(self, amp):
        return (amp, amp)


def test_reference_callbacks_map_to_device_kinds(monkeypatch):
    monkeypatch.delenv("NLSE_DEVICE_CALLBACKS", raising=False)
    norms, samples, dn, dzs = np.zeros(4), np.zeros((4, 2, 2)), np.zeros((4, 2, 2)), []
    plan = cb.device_plan(_Simu(), [ng.norm, ng.sample, ng.evaluate_delta_n, ng.adapt_delta_z],
                          [(2, norms), (3, samples), (4, dn), (5, dzs)])
    assert [(k, e) for k, e, _ in plan] == [("norm", 2), ("sample", 3), ("delta_n", 4),
                                            ("adapt", 5)]
    assert plan[0][2] is norms and plan[3][2] is dzs
    single = cb.device_plan(_Simu(), ng.norm, (1, norms))
    assert single == [("norm", 1, norms)]


@pytest.mark.parametrize("callbacks,args", [
    ([lambda s, A, z, i: None], [()]),                         # a user callback
    ([ng.norm], [(0, np.zeros(2))]),                           # every = 0
    ([ng.sample], [(2,)]),                                     # missing destination
    ([ng.adapt_delta_z], [(2, np.zeros(3))]),                  # the step list must append
    ([ng.adapt_delta_z, ng.adapt_delta_z], [(2, []), (3, [])]),  # one step size per loop
])
def test_lists_the_device_cannot_express_stay_on_the_host(callbacks, args, monkeypatch):
    monkeypatch.delenv("NLSE_DEVICE_CALLBACKS", raising=False)
    assert cb.device_plan(_Simu(), callbacks, args) is None


def test_adaptive_step_with_noise_stays_on_the_host(monkeypatch):
    monkeypatch.delenv("NLSE_DEVICE_CALLBACKS", raising=False)
    s = _Noisy()
    assert cb.device_plan(s, [s.add_noise], [(0.1,)])[0][0] == "noise"
    assert cb.device_plan(s, [s.add_noise, ng.adapt_delta_z], [(0.1,), (2, [])]) is None


def test_switch_turns_device_callbacks_off(monkeypatch):
    monkeypatch.setenv("NLSE_DEVICE_CALLBACKS", "0")
    assert cb.device_plan(_Simu(), [ng.norm], [(1, np.zeros(2))]) is None
