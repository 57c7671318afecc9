"""norm / sample callbacks run as nodes of one CUDA graph over the z-loop and
record what the per-step host loop records (NLSE_DEVICE_CALLBACKS=0)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from tests import cases  # noqa: E402


def _run(monkeypatch, device_cb, every_norm, every_sample, torch_dst=False):
    monkeypatch.setenv("NLSE_DEVICE_CALLBACKS", "1" if device_cb else "0")
    p, E = cases.nlse_beam(ng.NLSE, 128)
    n = 201
    ns = len(range(0, n, every_sample))
    if torch_dst:
        norms = torch.zeros(len(range(0, n, every_norm)), dtype=torch.float64, device="cuda")
        samples = torch.zeros((ns, 128, 128), dtype=torch.complex64, device="cuda")
    else:
        norms = np.zeros(len(range(0, n, every_norm)))
        samples = np.zeros((ns, 128, 128), np.complex64)
    out = p.out_field(E, cases.L, verbose=False, callback=[ng.norm, ng.sample],
                      callback_args=[(every_norm, norms), (every_sample, samples)])
    if torch_dst:
        norms, samples = norms.cpu().numpy(), samples.cpu().numpy()
    return out, norms, samples


def test_graph_callbacks_equal_host_loop_step_by_step(monkeypatch):
    a = _run(monkeypatch, True, 1, 5)
    b = _run(monkeypatch, False, 1, 5)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)  # same kernels step by step
    assert np.all(np.diff(a[1]) < 0)


def test_graph_callbacks_with_fused_segments(monkeypatch):
    a = _run(monkeypatch, True, 10, 25, torch_dst=True)
    b = _run(monkeypatch, False, 10, 25)
    assert cases.rel_l2(a[0], b[0]) <= 1e-5
    np.testing.assert_allclose(a[1], b[1], rtol=1e-5)
    assert cases.rel_l2(a[2], b[2]) <= 1e-5
