"""Fourier-neural-operator surrogate of the 256^2 split step: host side.

The network (4 spectral layers, 32 channels, 2048 retained modes, BF16
tensor-core contractions with FP32 accumulation) is defined and computed by
the kernels of csrc/fno.cu through the C ABI of include/nlse_fno.h; this
module owns the parameters (one flat FP32 vector, Adam moments), the BF16
tensor-core copies of the weights, the activation workspaces, and the order of
the kernel calls for inference, training (forward, loss, backward, Adam) and
gradient evaluation.  PyTorch only provides device memory and the stream.
"""

from __future__ import annotations

import ctypes as ct
import math

import numpy as np
import torch

from . import _lib
from .engine import stream_handle

N, C, NM, NL, KX = 256, 32, 2048, 4, 32
PART_LAYER, PART_PROJ, PART_LIFT = 1056, 66, 192
TILE_M = 128

# flat parameter layout (also the oracle's)
SHAPES = ([("wl", (5, C)), ("bl", (C,))]
          + [(f"{n}{l}", s) for l in range(NL)
             for n, s in (("W", (NM, C, C, 2)), ("Wc", (C, C)), ("b", (C,)))]
          + [("wp", (C, 2)), ("bp", (2,))])


def _ptr(t: torch.Tensor | None):
    return None if t is None else ct.c_void_p(t.data_ptr())


def param_size() -> int:
    return sum(math.prod(s) for _, s in SHAPES)


def _views(flat: torch.Tensor) -> dict:
    out, o = {}, 0
    for name, s in SHAPES:
        n = math.prod(s)
        out[name] = flat[o:o + n].view(s)
        o += n
    return out


class _Workspace:
    """Device buffers of one batch size (training keeps every activation)."""

    def __init__(self, nb: int, train: bool, dev: torch.device):
        bf, f32, c64 = torch.bfloat16, torch.float32, torch.complex64
        nmt = (nb + TILE_M - 1) // TILE_M
        nh = NL + 1 if train else 2
        self.nb, self.train = nb, train
        self.h = [torch.empty((nb, N, N, C), dtype=bf, device=dev) for _ in range(nh)]
        self.z = ([torch.empty((nb, N, N, C), dtype=bf, device=dev) for _ in range(NL - 1)]
                  if train else None)
        self.T = torch.empty((nb, N, KX, C), dtype=c64, device=dev)
        self.U = torch.empty((nb, N, KX, C), dtype=c64, device=dev)
        self.X = torch.empty((NM * nmt * TILE_M * 2 * C,), dtype=bf, device=dev)
        self.Y = torch.empty((NM, nb, C), dtype=c64, device=dev)
        self.Hs = ([torch.empty((NM, nb, C), dtype=c64, device=dev) for _ in range(NL)]
                   if train else None)
        self.out = torch.empty((nb, N, N), dtype=c64, device=dev)
        if train:
            self.Gs = torch.empty((NM, nb, C), dtype=c64, device=dev)
            self.dout = torch.empty((nb, N, N), dtype=c64, device=dev)
            self.dh = [torch.empty((nb, N, N, C), dtype=f32, device=dev) for _ in range(2)]
            self.part = torch.empty((nb * N * PART_LAYER,), dtype=f32, device=dev)
            self.stats = torch.empty((nb, 2), dtype=f32, device=dev)


class FNO:
    """The surrogate network on one GPU (the CUDA kernels are its only compute path)."""

    def __init__(self, device="cuda", seed: int = 0):
        self.lib = _lib.load()
        self.dev = torch.device(device)
        if self.dev.type != "cuda":
            raise ValueError("the surrogate runs on a CUDA device only")
        self.size = param_size()
        self.flat = torch.zeros(self.size, dtype=torch.float32, device=self.dev)
        self.grad = torch.zeros_like(self.flat)
        self.m = torch.zeros_like(self.flat)
        self.v = torch.zeros_like(self.flat)
        self.P = _views(self.flat)
        self.G = _views(self.grad)
        self.steps = 0
        bf = torch.bfloat16
        self.wf = [torch.empty(NM * 4 * C * C, dtype=bf, device=self.dev) for _ in range(NL)]
        self.wb = [torch.empty(NM * 4 * C * C, dtype=bf, device=self.dev) for _ in range(NL)]
        self.cf = [torch.empty(C * C, dtype=bf, device=self.dev) for _ in range(NL)]
        self.cb = [torch.empty(C * C, dtype=bf, device=self.dev) for _ in range(NL)]
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._ws: dict = {}
        self.init(seed)

    # ---- parameters -----------------------------------------------------------
    def init(self, seed: int = 0, out_scale: float = 1.0) -> None:
        """Seeded initial weights; out_scale scales the projection (a small value
        starts a residual predictor near zero)."""
        g = np.random.default_rng(seed)
        flat = np.zeros(self.size, np.float32)
        o = 0
        for name, s in SHAPES:
            n = math.prod(s)
            if name == "wl":
                flat[o:o + n] = g.normal(0, 1 / math.sqrt(5), n)
            elif name.startswith("Wc"):
                flat[o:o + n] = g.normal(0, 1 / math.sqrt(C), n)
            elif name == "wp":
                flat[o:o + n] = g.normal(0, out_scale / math.sqrt(C), n)
            elif name.startswith("W"):
                flat[o:o + n] = g.normal(0, 1 / math.sqrt(2 * C), n)
            o += n
        self.set_flat(flat)

    def set_flat(self, flat) -> None:
        self.flat.copy_(torch.as_tensor(np.asarray(flat, np.float32)).to(self.dev))
        self.m.zero_()
        self.v.zero_()
        self.steps = 0
        self.pack()

    def get_flat(self) -> np.ndarray:
        return self.flat.cpu().numpy()

    def pack(self) -> None:
        """Refresh the BF16 tensor-core operands from the FP32 parameters."""
        s = stream_handle(self.dev)
        for l in range(NL):
            _lib.check(self.lib.nlse_fno_pack_spectral(_ptr(self.P[f"W{l}"]), _ptr(self.wf[l]),
                                                       _ptr(self.wb[l]), s), "fno pack")
            _lib.check(self.lib.nlse_fno_pack_conv(_ptr(self.P[f"Wc{l}"]), _ptr(self.cf[l]),
                                                   _ptr(self.cb[l]), s), "fno pack")

    def _workspace(self, nb: int, train: bool) -> _Workspace:
        key = (nb, train)
        ws = self._ws.get(key)
        if ws is None:
            if len(self._ws) > 4:
                self._ws.clear()
            ws = self._ws[key] = _Workspace(nb, train, self.dev)
        return ws

    def check_status(self) -> None:
        if int(self.status.item()) != 0:
            self.status.zero_()
            raise RuntimeError("a surrogate kernel gave up waiting for its tensor-core work")

    # ---- forward ----------------------------------------------------------------
    def _forward(self, ws: _Workspace, xin: torch.Tensor, xs: torch.Tensor) -> torch.Tensor:
        L, P, s, nb = self.lib, self.P, stream_handle(self.dev), ws.nb
        ck = _lib.check
        ck(L.nlse_fno_lift_rows(nb, _ptr(xin), _ptr(xs), _ptr(P["wl"]), _ptr(P["bl"]),
                                _ptr(ws.h[0]), _ptr(ws.T), _ptr(self.status), s), "fno lift")
        for l in range(NL):
            last = l == NL - 1
            hin = ws.h[l] if ws.train else ws.h[l % 2]
            hout = ws.h[l + 1] if ws.train else (None if last else ws.h[(l + 1) % 2])
            ck(L.nlse_fno_cols_analysis(nb, _ptr(ws.T), 1.0, 1, _ptr(ws.X),
                                        _ptr(ws.Hs[l]) if ws.train else None, s), "fno analysis")
            ck(L.nlse_fno_mix(nb, _ptr(ws.X), _ptr(self.wf[l]), _ptr(ws.Y), _ptr(self.status), s),
               "fno mix")
            ck(L.nlse_fno_cols_synthesis(nb, _ptr(ws.Y), _ptr(ws.U), s), "fno synthesis")
            ck(L.nlse_fno_layer_rows(
                nb, _ptr(ws.U), _ptr(hin), _ptr(self.cf[l]), _ptr(P[f"b{l}"]), 0 if last else 1,
                _ptr(ws.z[l]) if (ws.train and not last) else None, _ptr(hout),
                None if last else _ptr(ws.T),
                _ptr(P["wp"]) if last else None, _ptr(P["bp"]) if last else None,
                _ptr(ws.out) if last else None, _ptr(self.status), s), "fno layer")
        return ws.out

    @staticmethod
    def _inputs(xin, xs, dev):
        xin = torch.as_tensor(xin).to(dev, torch.float32).contiguous()
        xs = torch.as_tensor(xs).to(dev, torch.float32).contiguous()
        if xin.ndim != 4 or tuple(xin.shape[1:]) != (N, N, 3) or tuple(xs.shape) != (xin.shape[0], 2):
            raise ValueError("inputs: xin (B, 256, 256, 3) and xs (B, 2)")
        return xin, xs

    def predict(self, xin, xs, chunk: int = 512) -> torch.Tensor:
        """Network output (B, 256, 256) complex64 on the device."""
        xin, xs = self._inputs(xin, xs, self.dev)
        B = xin.shape[0]
        out = torch.empty((B, N, N), dtype=torch.complex64, device=self.dev)
        for b0 in range(0, B, chunk):
            nb = min(chunk, B - b0)
            ws = self._workspace(nb, False)
            out[b0:b0 + nb].copy_(self._forward(ws, xin[b0:b0 + nb], xs[b0:b0 + nb]))
        return out

    # ---- backward -----------------------------------------------------------------
    def _backward(self, ws: _Workspace, xin: torch.Tensor, xs: torch.Tensor) -> None:
        L, P, G, s, nb = self.lib, self.P, self.G, stream_handle(self.dev), ws.nb
        ck = _lib.check
        rows = nb * N
        ck(L.nlse_fno_proj_bwd(nb, _ptr(ws.dout), _ptr(P["wp"]), _ptr(ws.h[NL]), _ptr(ws.dh[0]),
                               _ptr(ws.part), s), "fno proj bwd")
        ck(L.nlse_fno_reduce(_ptr(ws.part), rows, PART_PROJ, _ptr(G["wp"]), s), "fno reduce")
        dhc_in, Uin, k = ws.dh[0], None, 0
        for l in reversed(range(NL)):
            act = l < NL - 1
            dhc_out = ws.dh[1 - k]
            ck(L.nlse_fno_layer_rows_bwd(nb, _ptr(dhc_in), _ptr(Uin),
                                         _ptr(ws.z[l]) if act else None, 1 if act else 0,
                                         _ptr(ws.h[l]), _ptr(self.cb[l]), _ptr(dhc_out),
                                         _ptr(ws.T), _ptr(ws.part), _ptr(self.status), s),
               "fno layer bwd")
            ck(L.nlse_fno_reduce(_ptr(ws.part), rows, PART_LAYER, _ptr(G[f"Wc{l}"]), s),
               "fno reduce")
            ck(L.nlse_fno_cols_analysis(nb, _ptr(ws.T), 1.0 / (N * N), 0, _ptr(ws.X), _ptr(ws.Gs),
                                        s), "fno analysis")
            ck(L.nlse_fno_mix_wgrad(nb, _ptr(ws.Hs[l]), _ptr(ws.Gs), _ptr(G[f"W{l}"]), s),
               "fno wgrad")
            ck(L.nlse_fno_mix(nb, _ptr(ws.X), _ptr(self.wb[l]), _ptr(ws.Y), _ptr(self.status), s),
               "fno mix")
            ck(L.nlse_fno_cols_synthesis(nb, _ptr(ws.Y), _ptr(ws.U), s), "fno synthesis")
            dhc_in, Uin, k = dhc_out, ws.U, 1 - k
        ck(L.nlse_fno_lift_bwd(nb, _ptr(dhc_in), _ptr(Uin), _ptr(xin), _ptr(xs), _ptr(ws.part), s),
           "fno lift bwd")
        ck(L.nlse_fno_reduce(_ptr(ws.part), rows, PART_LIFT, _ptr(G["wl"]), s), "fno reduce")

    def gradient(self, xin, xs, tgt, ref=None) -> tuple[float, torch.Tensor]:
        """Loss mean_b ||out_b - tgt_b||^2 / ||ref_b||^2 (ref defaults to tgt) and its
        gradient (flat, FP32)."""
        xin, xs = self._inputs(xin, xs, self.dev)
        tgt = torch.as_tensor(tgt).to(self.dev, torch.complex64).contiguous()
        if ref is not None:
            ref = torch.as_tensor(ref).to(self.dev, torch.complex64).contiguous()
        ws = self._workspace(xin.shape[0], True)
        out = self._forward(ws, xin, xs)
        _lib.check(self.lib.nlse_fno_loss(ws.nb, _ptr(out), _ptr(tgt), _ptr(ref), _ptr(ws.stats),
                                          _ptr(ws.dout), stream_handle(self.dev)), "fno loss")
        self._backward(ws, xin, xs)
        st = ws.stats
        loss = (st[:, 0] / st[:, 1].clamp_min(1e-30)).mean()
        return float(loss.item()), self.grad

    def train_step(self, xin, xs, tgt, lr: float, wd: float = 0.0, ref=None) -> float:
        loss, _ = self.gradient(xin, xs, tgt, ref)
        self.steps += 1
        _lib.check(self.lib.nlse_fno_adam(_ptr(self.flat), _ptr(self.grad), _ptr(self.m),
                                          _ptr(self.v), self.size, lr, 0.9, 0.999, 1e-8,
                                          self.steps, wd, stream_handle(self.dev)), "fno adam")
        self.pack()
        return loss
