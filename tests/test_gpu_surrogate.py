"""The surrogate on the GPU: trained on solver pairs, the network must improve
on the coarse solve it corrects (the same method without the network), and
the judge must hand back the solver's field wherever a sampled prediction is
off by more than the tolerance."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_sampled_inputs_match_the_batch_generator_distributions():
    from nlse_gb300 import surrogate as sg

    inp = sg.sample_inputs(64, seed=3)
    V = inp["V"].cpu().numpy()
    assert V.shape == (64, 256, 256) and V.max() <= 0 and V.min() >= -8 * 2e-4
    E0 = inp["E0"].cpu().numpy()
    assert np.allclose(np.abs(E0).max(axis=(1, 2)), 1.0, atol=1e-3)
    assert inp["power"].min() >= 0.1 and inp["power"].max() <= 2.0
    assert (-inp["n2"]).min() >= 1e-10 and (-inp["n2"]).max() <= 10 ** -8.4


def test_network_improves_on_the_coarse_solve_and_the_judge_enforces_tolerance():
    from nlse_gb300 import surrogate as sg

    train = sg.sample_inputs(1024, seed=1)
    s = sg.Surrogate(coarse=5, seed=0)
    s.fit(train, sg.solve(train), epochs=4, batch=32, lr=2e-3)
    s.net.check_status()
    test = sg.sample_inputs(128, seed=2)
    ref = sg.solve(test)
    P, Ec = s.predict(test, with_coarse=True)
    e_coarse = sg.rel_l2(Ec, ref).cpu().numpy()
    e_net = sg.rel_l2(P, ref).cpu().numpy()
    assert np.median(e_net) < 0.8 * np.median(e_coarse), (np.median(e_net), np.median(e_coarse))
    out, rep = s.judge(test, P, every=4, seed=5)
    assert rep["sampled"] == 32 and rep["resolved"] >= 32
    e_out = sg.rel_l2(out, ref).cpu().numpy()
    rng = np.random.default_rng(5)
    sample = np.sort(rng.choice(128, size=32, replace=False))
    assert e_out[sample].max() <= 1e-2
    assert np.all(e_out <= np.maximum(e_net, 1e-6) + 1e-7)  # the judge never makes a field worse
