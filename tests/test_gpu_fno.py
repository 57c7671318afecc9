"""Surrogate kernels on the GPU against the oracle (oracle/fno_oracle.py).

Tolerances: the forward pass differs from the oracle by FP32 transform and
accumulation rounding (and rare BF16 rounding flips of stored activations):
rel-L2 <= 5e-3.  The backward pass also rounds dz and the spectral gradient
to BF16 as tensor-core operands and evaluates GELU' at the BF16 z:
rel-L2 <= 3e-2 per parameter tensor.
"""

import ctypes as ct

import numpy as np
import pytest
import torch

from oracle import fno_oracle as fo
from tests.test_fno_oracle import _problem

pytestmark = pytest.mark.gpu


def _bf16(a):
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16)


@pytest.mark.parametrize("n,k", [(32, 32), (64, 64), (32, 64), (64, 32)])
def test_tensor_core_gemm_selftest(n, k):
    from nlse_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(n + k)
    A = _bf16(rng.normal(size=(128, k)))
    B = _bf16(rng.normal(size=(n, k)))
    ref = A.double().numpy() @ B.double().numpy().T
    dA, dB = A.cuda(), B.cuda()
    C = torch.empty((128, n), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(lib.nlse_fno_gemm_selftest(dA.data_ptr(), dB.data_ptr(), C.data_ptr(), n, k,
                                          st.data_ptr(),
                                          ct.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "selftest")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    np.testing.assert_allclose(C.cpu().numpy(), ref, rtol=1e-5, atol=1e-4)


def _canonical(t):
    """(..., R, K) -> the tensor-core operand layout (8 x 8 core matrices, K-adjacent
    ones packed): element (r, k) at (r/8)*8K + (k/8)*64 + (r%8)*8 + k%8."""
    *lead, R, K = t.shape
    t = t.reshape(*lead, R // 8, 8, K // 8, 8)
    return t.transpose(-3, -2).reshape(*lead, R * K)


def test_mode_mixing_over_partial_tiles_matches_numpy():
    """nlse_fno_mix on 130 fields (two 128-row tiles, the second holding 2):
    every mode's product against NumPy; rows past the batch are NaN in the
    operand and must not reach the stored rows."""
    from nlse_gb300 import _lib

    lib = _lib.load()
    nb, NM, XK = 130, fo.NM, 2 * fo.C
    nmt = (nb + 127) // 128
    rng = np.random.default_rng(21)
    A = torch.full((NM, nmt * 128, XK), float("nan"), dtype=torch.bfloat16)
    A[:, :nb] = _bf16(rng.normal(size=(NM, nb, XK)))
    B = _bf16(rng.normal(size=(NM, XK, XK)))
    X = _canonical(A.reshape(NM, nmt, 128, XK)).contiguous().cuda()
    Wb = _canonical(B).contiguous().cuda()
    Y = torch.zeros((NM, nb, fo.C), dtype=torch.complex64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(lib.nlse_fno_mix(nb, X.data_ptr(), Wb.data_ptr(), Y.data_ptr(), st.data_ptr(),
                                ct.c_void_p(torch.cuda.current_stream().cuda_stream)), "mix")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    D = np.einsum("mbk,mnk->mbn", A[:, :nb].double().numpy(), B.double().numpy())
    ref = D[..., :fo.C] + 1j * D[..., fo.C:]
    got = Y.cpu().numpy()
    assert np.isfinite(got).all()
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-4)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _net(flat):
    from nlse_gb300.fno import FNO

    net = FNO("cuda")
    net.set_flat(flat.astype(np.float32))
    return net


@pytest.mark.parametrize("B", [1, 3])
def test_forward_matches_oracle(B):
    # B = 1: fewer image rows (256) than resident row-kernel CTAs; B = 3: each
    # persistent CTA walks several rows
    flat, xin, xs, _ = _problem(seed=5, B=B)
    flat = flat.astype(np.float32).astype(np.float64)
    xin, xs = xin.astype(np.float32), xs.astype(np.float32)
    net = _net(flat)
    out = net.predict(xin, xs).cpu().numpy()
    net.check_status()
    ref, _ = fo.forward(flat, xin, xs)
    assert _rel(out, ref) <= 5e-3


def test_gradient_matches_oracle():
    flat, xin, xs, tgt = _problem(seed=6, B=2)
    flat = flat.astype(np.float32).astype(np.float64)
    xin, xs = xin.astype(np.float32), xs.astype(np.float32)
    net = _net(flat)
    loss, g = net.gradient(xin, xs, tgt.astype(np.complex64))
    net.check_status()
    g = g.cpu().numpy().astype(np.float64)
    out, cache = fo.forward(flat, xin, xs)
    ref_loss, dout = fo.loss(out, tgt)
    ref = fo.backward(flat, cache, dout)
    assert abs(loss - ref_loss) <= 1e-2 * ref_loss
    gv, rv = fo.Params.views(g), fo.Params.views(ref)
    errs = {name: _rel(gv[name], rv[name]) for name, _ in fo.Params.SHAPES}
    assert max(errs.values()) <= 3e-2, errs


def test_training_lowers_the_loss():
    _, xin, xs, _ = _problem(seed=7, B=8)
    from nlse_gb300.fno import FNO

    net = FNO("cuda", seed=1)
    tgt = (xin[..., 0] * np.exp(1j * xin[..., 2])).astype(np.complex64)  # a smooth map to learn
    first = net.train_step(xin, xs, tgt, 3e-3)
    for _ in range(40):
        last = net.train_step(xin, xs, tgt, 3e-3)
    net.check_status()
    assert last < 0.5 * first
