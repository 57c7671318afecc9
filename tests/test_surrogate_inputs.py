"""The surrogate's input sets (surrogate.sample_inputs) on the CPU: seeded and
reproducible, drawn from the 164-field batch's distributions restricted to
256^2 -- power U[0.1, 2] W, n2 = -10^U[-10, -8.4], unit-peak Gaussian beams,
potentials that are sums of 1-8 Gaussian wells of depth U[0.5, 2]e-4 --, and
the potential equal to the direct sum of its wells."""

import numpy as np
import torch

from nlse_gb300 import surrogate as sg


def test_inputs_are_seeded_and_reproducible():
    a = sg.sample_inputs(5, seed=3, device="cpu")
    b = sg.sample_inputs(5, seed=3, device="cpu")
    c = sg.sample_inputs(5, seed=4, device="cpu")
    for k in a:
        same = torch.equal(a[k], b[k]) if isinstance(a[k], torch.Tensor) else np.array_equal(a[k], b[k])
        assert same, k
    assert not torch.equal(a["V"], c["V"])
    assert a["E0"].shape == (5, sg.N, sg.N) and a["E0"].dtype == torch.complex64
    assert a["V"].shape == (5, sg.N, sg.N) and a["V"].dtype == torch.float32


def test_inputs_follow_the_batch_distributions():
    inp = sg.sample_inputs(400, seed=1, device="cpu")
    p, n2 = inp["power"], inp["n2"]
    assert p.min() >= 0.1 and p.max() <= 2.0
    assert np.all(n2 < 0) and (-n2).min() >= 1e-10 and (-n2).max() <= 10 ** -8.4
    peak = inp["E0"].abs().amax(dim=(-2, -1))
    assert torch.allclose(peak, torch.ones_like(peak), atol=1e-3)  # unit-peak beams
    V = inp["V"]
    assert float(V.max()) <= 0.0
    assert float(V.min()) >= -sg.MAX_WELLS * 2e-4 * (1 + 1e-6)
    assert float(V.amin(dim=(-2, -1)).max()) < -0.4e-4  # every field has at least one well


def test_potential_is_the_sum_of_its_wells():
    # the same draws in the same order as sample_inputs, summed well by well
    n, seed = 3, 7
    rng = np.random.default_rng(seed)
    rng.uniform(0.1, 2.0, n)
    rng.uniform(-10, -8.4, n)
    rng.uniform(0.8e-3, 2.5e-3, n)
    count = rng.integers(1, sg.MAX_WELLS + 1, n)
    depth = rng.uniform(0.5e-4, 2e-4, (n, sg.MAX_WELLS)) * (np.arange(sg.MAX_WELLS) < count[:, None])
    width = rng.uniform(30e-6, 150e-6, (n, sg.MAX_WELLS))
    centre = rng.uniform(-sg.WINDOW / 4, sg.WINDOW / 4, (n, sg.MAX_WELLS, 2))
    X, Y, _, _ = sg._grid()
    XX, YY = np.meshgrid(X, Y)
    ref = np.zeros((n, sg.N, sg.N))
    for f in range(n):
        for k in range(sg.MAX_WELLS):
            ref[f] -= depth[f, k] * np.exp(-((XX - centre[f, k, 0]) ** 2 + (YY - centre[f, k, 1]) ** 2)
                                           / width[f, k] ** 2)
    got = sg.sample_inputs(n, seed=seed, device="cpu")["V"].numpy()
    assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(np.abs(ref))
