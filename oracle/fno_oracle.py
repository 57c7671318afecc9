"""CPU oracle of the Fourier-neural-operator surrogate (test infrastructure).

NumPy float64 restatement of the model the CUDA kernels implement
(nlse_gb300/csrc/fno.cu, include/nlse_fno.h), forward and backward, used only
by the tests to check the GPU forward pass and gradients.  The surrogate has
no reference counterpart (it is new to this project), so this file is the
specification it is checked against: grid N = 256, C = 32 channels, retained
modes kx in [0, 32), ky in [0, 32) u [224, 256) (mode index iy*32 + kx).

    h0      = bf16(lift(x))
    H_l     = F_R h_l                      (unnormalised DFT on the kept modes; the
                                            row stage with BF16 cos/sin over quarter
                                            rows, FP32 sums: analysis_rounded)
    S_l     = bf16(H_l) . bf16(W_l)         per mode, complex 32 x 32
    s_l     = Re(ifft2(zero-filled S_l))    ((1/N^2) Re sum_k S(k) e^{+ik.x}; the row
                                            stage with BF16 cos/sin and BF16 row
                                            spectra U/N^2, FP32 sums: synthesis_rounded)
    z_l     = h_l . bf16(Wc_l) + s_l + b_l
    h_{l+1} = bf16(GELU(z_l)) (l < 3),  h_4 = bf16(z_3)   (tanh-form GELU)
    out     = h_4 . Wp + bp                 (Re, Im)

Gradients pass through the bf16() roundings unchanged.  With exact=True no
rounding is applied (for finite-difference checks of the gradients).
"""

from __future__ import annotations

import numpy as np

N, C, KX, KY, NL = 256, 32, 32, 64, 4
NM = KX * KY
KY_ROWS = np.r_[np.arange(KY // 2), np.arange(N - KY // 2, N)]


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even) via float32, back to float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16c(z: np.ndarray) -> np.ndarray:
    return bf16(z.real) + 1j * bf16(z.imag)


GA, GB = np.sqrt(2.0 / np.pi), 0.044715


def gelu(z):
    """GELU in its tanh form (the kernels' activation)."""
    return 0.5 * z * (1.0 + np.tanh(GA * (z + GB * z**3)))


def gelu_grad(z):
    t = np.tanh(GA * (z + GB * z**3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GA * (1.0 + 3.0 * GB * z * z)


def analysis(h: np.ndarray) -> np.ndarray:
    """(B, N, N, C) real -> (B, NM, C) complex: kept modes of the unnormalised DFT."""
    F = np.fft.fft2(h, axes=(1, 2))
    return F[:, KY_ROWS, :KX, :].reshape(h.shape[0], NM, h.shape[-1])


def synthesis(S: np.ndarray) -> np.ndarray:
    """(B, NM, C) complex -> (B, N, N, C): Re(ifft2) of the zero-filled spectrum."""
    B = S.shape[0]
    F = np.zeros((B, N, N, S.shape[-1]), np.complex128)
    F[:, KY_ROWS, :KX, :] = S.reshape(B, KY, KX, -1)
    return np.fft.ifft2(F, axes=(1, 2)).real


def _basis():
    """The BF16 row-synthesis basis: cos and sin of 2 pi kx x / N, (KX, N)."""
    j = (np.arange(KX)[:, None] * np.arange(N)[None, :]) % N
    ang = 2.0 * np.pi * j / N
    return bf16(np.cos(ang)), bf16(np.sin(ang))


def synthesis_rounded(S: np.ndarray) -> np.ndarray:
    """synthesis() as the kernels evaluate it: the column stage exact, then
    s(x) = sum_kx bf16(Re U(kx)/N^2) bf16(cos) - bf16(Im U(kx)/N^2) bf16(sin)
    for each image row, U the row's half spectrum (kx < KX)."""
    B = S.shape[0]
    F = np.zeros((B, N, KX, S.shape[-1]), np.complex128)
    F[:, KY_ROWS, :, :] = S.reshape(B, KY, KX, -1)
    U = np.fft.ifft(F, axis=1) * N                      # (B, y, kx, c), unnormalised
    ur, ui = bf16(U.real / N**2), bf16(U.imag / N**2)
    cb, sb = _basis()
    return np.einsum("bykc,kx->byxc", ur, cb) - np.einsum("bykc,kx->byxc", ui, sb)


def _analysis_basis():
    """BF16 cos and sin of 2 pi kx x' / N over a quarter row, x' < N/4: (KX, N/4)."""
    j = (np.arange(KX)[:, None] * np.arange(N // 4)[None, :]) % N
    ang = 2.0 * np.pi * j / N
    return bf16(np.cos(ang)), bf16(np.sin(ang))


def analysis_rounded(h: np.ndarray) -> np.ndarray:
    """analysis() as the kernels evaluate it: the row stage over quarter rows
    (x = 64 q + x') with BF16 cos/sin of 2 pi kx x' / N, the exact factor
    (-i)^(kx q) of each quarter and FP32 sums of the BF16 activations; the
    column stage exact."""
    B = h.shape[0]
    cb, sb = _analysis_basis()
    hq = h.reshape(B, N, 4, N // 4, h.shape[-1])                 # b, y, q, x', c
    Dq = np.einsum("byqxc,kx->byqkc", hq, cb) - 1j * np.einsum("byqxc,kx->byqkc", hq, sb)
    rot = (-1j) ** ((np.arange(KX)[None, :] * np.arange(4)[:, None]) % 4)  # (q, kx)
    Hrow = np.einsum("byqkc,qk->bykc", Dq, rot)                  # (B, y, kx, c)
    F = np.fft.fft(Hrow, axis=1)
    return F[:, KY_ROWS, :, :].reshape(B, NM, h.shape[-1])


class Params:
    """Flat parameter vector with named views (layout of the CUDA host code)."""

    SHAPES = ([("wl", (5, C)), ("bl", (C,))]
              + [(f"{n}{l}", s) for l in range(NL)
                 for n, s in (("W", (NM, C, C, 2)), ("Wc", (C, C)), ("b", (C,)))]
              + [("wp", (C, 2)), ("bp", (2,))])

    @classmethod
    def size(cls) -> int:
        return sum(int(np.prod(s)) for _, s in cls.SHAPES)

    @classmethod
    def views(cls, flat: np.ndarray) -> dict:
        out, o = {}, 0
        for name, s in cls.SHAPES:
            n = int(np.prod(s))
            out[name] = flat[o:o + n].reshape(s)
            o += n
        return out


def _cw(W, exact):
    w = W[..., 0] + 1j * W[..., 1]
    return w if exact else bf16c(w)


def forward(flat: np.ndarray, xin: np.ndarray, xs: np.ndarray, exact: bool = False):
    """xin (B, N, N, 3), xs (B, 2) -> out (B, N, N) complex, cache."""
    P = Params.views(np.asarray(flat, np.float64))
    r = (lambda a: a) if exact else bf16
    lift = (np.einsum("bpqi,io->bpqo", xin, P["wl"][:3])
            + np.einsum("bi,io->bo", xs, P["wl"][3:])[:, None, None, :] + P["bl"])
    h = [r(lift)]
    zs, Xs = [], []
    for l in range(NL):
        X = analysis(h[l]) if exact else bf16c(analysis_rounded(h[l]))
        S = np.einsum("bmc,mco->bmo", X, _cw(P[f"W{l}"], exact))
        z = h[l] @ r(P[f"Wc{l}"]) + (synthesis(S) if exact else synthesis_rounded(S)) + P[f"b{l}"]
        zs.append(z)
        Xs.append(X)
        h.append(r(gelu(z)) if l < NL - 1 else r(z))
    o = h[-1] @ P["wp"] + P["bp"]
    return o[..., 0] + 1j * o[..., 1], {"h": h, "z": zs, "X": Xs, "xin": xin, "xs": xs}


def loss(out: np.ndarray, tgt: np.ndarray):
    """mean_b ||out_b - tgt_b||^2 / ||tgt_b||^2 and its gradient (complex)."""
    B = out.shape[0]
    d = out - tgt
    nt = np.sum(np.abs(tgt) ** 2, axis=(1, 2))
    L = float(np.mean(np.sum(np.abs(d) ** 2, axis=(1, 2)) / nt))
    return L, 2.0 * d / (B * nt[:, None, None])


def backward(flat: np.ndarray, cache: dict, dout: np.ndarray, exact: bool = False) -> np.ndarray:
    """Gradient of sum(Re(conj(dout) * out)) w.r.t. the flat parameters."""
    P = Params.views(np.asarray(flat, np.float64))
    G = np.zeros(Params.size())
    gv = Params.views(G)
    r = (lambda a: a) if exact else bf16
    h, zs, Xs = cache["h"], cache["z"], cache["X"]
    d2 = np.stack([dout.real, dout.imag], axis=-1)
    gv["wp"][:] = np.einsum("bpqo,bpqj->oj", h[-1], d2)
    gv["bp"][:] = d2.sum(axis=(0, 1, 2))
    dh = d2 @ P["wp"].T
    for l in reversed(range(NL)):
        dz = dh * gelu_grad(zs[l]) if l < NL - 1 else dh
        gv[f"b{l}"][:] = dz.sum(axis=(0, 1, 2))
        gv[f"Wc{l}"][:] = np.einsum("bpqc,bpqo->co", h[l], dz)
        gS = analysis(dz) / (N * N)
        gW = np.einsum("bmc,bmo->mco", np.conj(Xs[l]), gS)
        gv[f"W{l}"][:] = np.stack([gW.real, gW.imag], axis=-1)
        gX = np.einsum("bmo,mco->bmc", gS, np.conj(_cw(P[f"W{l}"], exact)))
        dh = dz @ r(P[f"Wc{l}"]).T + synthesis(gX) * (N * N)
    xin, xs = cache["xin"], cache["xs"]
    gv["wl"][:3] = np.einsum("bpqi,bpqo->io", xin, dh)
    gv["wl"][3:] = np.einsum("bi,bo->io", xs, dh.sum(axis=(1, 2)))
    gv["bl"][:] = dh.sum(axis=(0, 1, 2))
    return G
