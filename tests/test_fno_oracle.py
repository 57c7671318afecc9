"""CPU checks of the surrogate's oracle (oracle/fno_oracle.py): bf16 rounding,
transform adjoints and the analytic gradient against finite differences."""

import numpy as np
import torch

from oracle import fno_oracle as fo


def test_bf16_rounding_matches_torch():
    x = np.random.default_rng(0).normal(0, 3, 10000).astype(np.float32)
    x[:4] = [0.0, -0.0, 1.0 + 2**-8, 1.0 + 3 * 2**-8]  # ties to even
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(fo.bf16(x), ref)


def test_synthesis_is_adjoint_of_analysis():
    rng = np.random.default_rng(1)
    h = rng.normal(size=(1, fo.N, fo.N, 2))
    S = rng.normal(size=(1, fo.NM, 2)) + 1j * rng.normal(size=(1, fo.NM, 2))
    # <Re F^-1_R S, h> * N^2 = Re <S, F_R h>
    lhs = np.sum(fo.synthesis(S) * h) * fo.N**2
    rhs = np.sum(np.real(S * np.conj(fo.analysis(h))))
    assert abs(lhs - rhs) <= 1e-9 * abs(rhs)


def test_rounded_synthesis_is_the_synthesis_to_bf16_accuracy():
    rng = np.random.default_rng(4)
    S = rng.normal(size=(1, fo.NM, 3)) + 1j * rng.normal(size=(1, fo.NM, 3))
    exact, rounded = fo.synthesis(S), fo.synthesis_rounded(S)
    rel = np.linalg.norm(rounded - exact) / np.linalg.norm(exact)
    assert 1e-5 < rel < 1e-2, rel
    cb, sb = fo._basis()
    assert cb[0, 5] == 1.0 and sb[0, 5] == 0.0 and cb[8, 8] == fo.bf16(np.cos(np.pi / 2))


def test_rounded_analysis_is_the_analysis_to_bf16_accuracy():
    rng = np.random.default_rng(5)
    h = fo.bf16(rng.normal(size=(1, fo.N, fo.N, 3)))
    exact, rounded = fo.analysis(h), fo.analysis_rounded(h)
    rel = np.linalg.norm(rounded - exact) / np.linalg.norm(exact)
    assert 1e-5 < rel < 1e-2, rel
    # a pure row harmonic lands on its own mode up to the basis rounding
    x = np.arange(fo.N)
    g = np.zeros((1, fo.N, fo.N, 1))
    g[0, :, :, 0] = np.cos(2 * np.pi * 5 * x / fo.N)[None, :]
    H = fo.analysis_rounded(g)[0, :, 0]
    assert abs(H[5] - fo.N * fo.N / 2) < 1e-2 * fo.N * fo.N and np.abs(np.delete(H, 5)).max() < 2e-2 * fo.N**2


def _problem(seed=2, B=1):
    """Seeded parameters, smooth beam-like inputs and a random target."""
    rng = np.random.default_rng(seed)
    flat = np.zeros(fo.Params.size())
    v = fo.Params.views(flat)
    for name, s in fo.Params.SHAPES:
        v[name][...] = rng.normal(0, 0.3 if name.startswith("W") and len(s) == 4 else 0.2, s)
    y, x = np.mgrid[0:fo.N, 0:fo.N] / fo.N - 0.5
    beam = np.exp(-(x**2 + y**2) / 0.05)
    xin = np.stack([beam, 0.1 * beam * x, -np.exp(-((x - 0.1) ** 2 + y**2) / 0.01)], -1)
    xin = np.repeat(xin[None], B, 0) * (1 + 0.1 * rng.normal(size=(B, 1, 1, 1)))
    xs = rng.normal(size=(B, 2))
    tgt = rng.normal(size=(B, fo.N, fo.N)) + 1j * rng.normal(size=(B, fo.N, fo.N))
    return flat, xin, xs, tgt


def test_oracle_gradient_matches_finite_differences():
    flat, xin, xs, tgt = _problem()

    def L(f):
        out, _ = fo.forward(f, xin, xs, exact=True)
        return fo.loss(out, tgt)[0]

    out, cache = fo.forward(flat, xin, xs, exact=True)
    _, dout = fo.loss(out, tgt)
    g = fo.backward(flat, cache, dout, exact=True)
    rng = np.random.default_rng(3)
    o = 0
    for name, s in fo.Params.SHAPES:
        n = int(np.prod(s))
        d = np.zeros_like(flat)
        d[o:o + n] = rng.normal(size=n)
        eps = 1e-4 / np.sqrt(n)
        fd = (L(flat + eps * d) - L(flat - eps * d)) / (2 * eps)
        an = float(g @ d)
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-8) + 1e-10, (name, fd, an)
        o += n
