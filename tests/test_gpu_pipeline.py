"""out_field on a page-locked host batch: the pipelined path (uploads,
propagations and downloads of field chunks overlapped) against the same call
on device input.  Fields are independent and every chunk runs the kernel
variant of the first, so the results are bit-identical."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from tests import cases  # noqa: E402


def _sim(N, B, per_field, seed):
    rng = np.random.default_rng(seed)
    if per_field:
        power = rng.uniform(0.5, 1.5, B)
        n2 = -(10.0 ** rng.uniform(-9.5, -8.6, B)).reshape(B, 1, 1)
    else:
        power, n2 = cases.POWER, cases.N2
    sim = ng.NLSE(cases.ALPHA, power, cases.WINDOW, n2, None, cases.L, NX=N, NY=N,
                  Isat=cases.ISAT)
    sim.delta_z = 5e-5
    V0 = cases.potential(sim.XX, sim.YY)
    sim.V = (V0[None] * rng.uniform(0.5, 1.5, (B, 1, 1))).astype(np.float32) if per_field \
        else V0.astype(np.float32)
    E = cases.gaussian(sim.XX, sim.YY) * (1 + 0.01 * rng.standard_normal((B, N, N)))
    return sim, E.astype(np.complex64)


@pytest.mark.parametrize("N,B,per_field,chunks", [(1024, 8, True, 4), (2048, 3, False, 2),
                                                   (1024, 9, False, 4)])
def test_pipelined_host_batch_equals_device_call(N, B, per_field, chunks, monkeypatch):
    monkeypatch.setenv("NLSE_AUTOTUNE", "0")
    z = 11.5 * 5e-5
    sim, E = _sim(N, B, per_field, N + B)
    Eh = torch.from_numpy(E).pin_memory()
    assert sim._pipeline_chunks(Eh) == chunks
    got = sim.out_field(Eh, z, verbose=False)
    assert isinstance(got, torch.Tensor) and not got.is_cuda and got.shape == Eh.shape
    sim2, _ = _sim(N, B, per_field, N + B)
    ref = sim2.out_field(torch.from_numpy(E).cuda(), z, verbose=False).cpu()
    assert torch.equal(got, ref)
    # a pageable NumPy batch takes the unsplit path and agrees as well
    assert sim._pipeline_chunks(E) == 1
    np.testing.assert_array_equal(sim.out_field(E, z, verbose=False), ref.numpy())
