"""out_field on a page-locked host batch: the pipelined path (uploads,
propagations and downloads of field chunks overlapped) against the same call
on device input.  Fields are independent, so with the same kernel variant
the results are bit-identical; the chunks' plans are other geometries than
the whole batch's, and left to their own (tuned) variants they agree to
complex64 rounding."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import _lib, engine  # noqa: E402
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


@pytest.mark.parametrize("N,B,per_field,bounds", [(1024, 8, True, [0, 1, 7, 8]),
                                                   (2048, 3, False, [0, 1, 3]),
                                                   (1024, 9, False, [0, 1, 8, 9])])
def test_pipelined_host_batch_equals_device_call(N, B, per_field, bounds, monkeypatch):
    monkeypatch.setenv("NLSE_AUTOTUNE", "0")
    z = 11.5 * 5e-5
    sim, E = _sim(N, B, per_field, N + B)
    Eh = torch.from_numpy(E).pin_memory()
    assert sim._pipeline_bounds(Eh, ng.count_steps(z, sim.delta_z)) == bounds
    # loops longer than PIPELINE_MAX_STEPS run unsplit (whole-batch kernels)
    assert sim._pipeline_bounds(Eh, sim.PIPELINE_MAX_STEPS + 1) is None
    # every plan involved on one variant: the pipelined fields are the unsplit call's
    dev = torch.device("cuda", 0)
    plans = [engine.Plan.get(2, (N, N), b1 - b0, 1, _lib.NLSE_C64, dev, slot=i)
             for i, (b0, b1) in enumerate(zip(bounds, bounds[1:]))]
    plans.append(engine.Plan.get(2, (N, N), B, 1, _lib.NLSE_C64, dev))
    for p in plans:
        p.set_variant(_lib.ROWS_DEEP, _lib.COLS_PAIR)
    got = sim.out_field(Eh, z, verbose=False)
    assert isinstance(got, torch.Tensor) and not got.is_cuda and got.shape == Eh.shape
    sim2, _ = _sim(N, B, per_field, N + B)
    ref = sim2.out_field(torch.from_numpy(E).cuda(), z, verbose=False).cpu()
    assert torch.equal(got, ref)
    # the chunks on another variant than the whole batch: complex64 rounding apart
    for p in plans[:-1]:
        p.set_variant(_lib.ROWS_TMA, _lib.COLS_TILE)
    other = sim.out_field(Eh, z, verbose=False)
    assert cases.rel_l2(other.numpy(), ref.numpy()) <= 1e-5
    # a pageable NumPy batch takes the unsplit path and agrees as well
    assert sim._pipeline_bounds(E, 12) is None
    np.testing.assert_array_equal(sim.out_field(E, z, verbose=False), ref.numpy())
