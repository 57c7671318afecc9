"""Callbacks with the reference's signature cb(simu, A, z, i, *args).

Mirrors NLSE/callbacks.py:1-112 for device (torch) fields.  Reductions are
accumulated in FP64 on the device (libnlse_sm103 nlse_power); a result is
copied to the host only when the destination array is a NumPy array.
"""

from __future__ import annotations

import numpy as np
import torch
from scipy.constants import c, epsilon_0

from . import engine


def _store(dst, idx, value) -> None:
    if isinstance(dst, np.ndarray):
        if isinstance(value, torch.Tensor):
            value = value.detach().cpu().numpy()
        dst[idx] = value
    else:
        dst[idx] = value


def sample(simu, A, z: float, i: int, save_every: int, E_samples) -> None:
    """Save A every save_every steps into E_samples (callbacks.py:7-29)."""
    if i % save_every == 0:
        _store(E_samples, i // save_every, A.clone() if isinstance(A, torch.Tensor) else A.copy())


def norm(simu, A, z: float, i: int, save_every: int, norms) -> None:
    """Sum of |A|^2 every save_every steps, FP64 on the device (callbacks.py:32-54)."""
    if i % save_every == 0:
        if isinstance(A, torch.Tensor) and A.is_cuda and A.is_contiguous():
            s = engine.power(A, 1)[0]
        else:
            s = (A.real * A.real + A.imag * A.imag).sum()
        _store(norms, i // save_every, s)


def evaluate_delta_n(simu, A, z: float, i: int, save_every: int, delta_n) -> None:
    """Nonlinear index change every save_every steps (callbacks.py:57-82)."""
    if i % save_every == 0:
        A_sq = A.real * A.real + A.imag * A.imag
        _store(delta_n, i // save_every,
               c * epsilon_0 / 2 * simu.n2 * A_sq / (1 + A_sq / simu.I_sat))


def adapt_delta_z(simu, A, z: float, i: int, update_every: int, delta_z: list) -> None:
    """Adaptive step from the peak index change (callbacks.py:85-112).

    Keeps the reference's expression, in which c eps0 / 2 multiplies only the
    imaginary part (callbacks.py:109).
    """
    delta_z.append(simu.delta_z)
    if i % update_every == 0:
        A_sq = A.real * A.real + A.imag * A.imag * c * epsilon_0 / 2
        n2 = simu.n2
        if isinstance(n2, torch.Tensor):
            n2 = n2.abs()
        else:
            n2 = np.abs(n2)
        delta_n = n2 * A_sq / (1 + A_sq / simu.I_sat)
        z_nl = float(1 / (simu.k * float(delta_n.max())))
        simu.delta_z = np.abs(z_nl) / 12


# ---- callbacks as graph nodes ------------------------------------------------
# norm and sample read only the live field, so when every callback of a loop
# is one of them the whole z-loop becomes one CUDA graph: segments of steps up
# to each recording step, then the recording nodes (an FP64 power sum or a
# device copy into a preallocated slot).  Results reach the caller's arrays
# once, after the loop.  No per-step host synchronisation.

def device_plan(simu, callback, callback_args):
    """[(kind, every, payload)] if every callback can run as graph nodes, else
    None (NLSE_DEVICE_CALLBACKS=0 turns this off).  Kinds: "norm" and
    "sample" (payload: the destination array) and, for DDGPE, "noise"
    (payload: a function (A, step) adding that step's noise)."""
    import os

    if os.environ.get("NLSE_DEVICE_CALLBACKS", "") == "0":
        return None
    if callable(callback):
        pairs = [(callback, callback_args)]
    elif isinstance(callback, list) and callback and all(callable(cb) for cb in callback):
        pairs = list(zip(callback, callback_args))
    else:
        return None
    noise_fn = getattr(type(simu), "add_noise", None)
    out = []
    for cb, args in pairs:
        fn = getattr(cb, "__func__", cb)
        if fn is norm or fn is sample:
            if len(args) != 2 or int(args[0]) <= 0:
                return None
            out.append(("norm" if fn is norm else "sample", int(args[0]), args[1]))
        elif noise_fn is not None and fn is noise_fn and hasattr(simu, "_add_noise"):
            amp = float(args[0]) if len(args) else 0.0
            simu._noise_sigmas(amp)  # raises here, not inside a capture, if unsupported
            out.append(("noise", 1, lambda A, step, amp=amp: simu._add_noise(A, step, amp)))
        else:
            return None
    return out


def run_in_graph(plan, A: torch.Tensor, op, n: int, recs) -> bool:
    """Advance A by n steps with the callbacks of recs as graph nodes; False
    (nothing done) if the recording buffers would not fit comfortably."""
    store = [(k, s, d) for k, s, d in recs if k != "noise"]
    counts = [len(range(0, n, s)) for _, s, _ in store]
    need = sum(c * (A.numel() * A.element_size() if k == "sample" else 8)
               for (k, _, _), c in zip(store, counts))
    free, _ = torch.cuda.mem_get_info(A.device)
    if need > free // 4:
        return False
    bufs = [torch.empty((c,) + (tuple(A.shape) if k == "sample" else ()),
                        dtype=A.dtype if k == "sample" else torch.float64, device=A.device)
            for (k, _, _), c in zip(store, counts)]
    points = sorted({i for _, s, _ in recs for i in range(0, n, s)})
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        i0 = 0
        for p in points:
            engine.propagate(plan, A, op, p + 1 - i0, i0, graph=False)
            i0 = p + 1
            j = 0
            for kind, s, payload in recs:  # in the callbacks' order
                if kind == "noise":
                    payload(A, p)
                    continue
                buf = bufs[j]
                j += 1
                if p % s == 0:
                    if kind == "norm":
                        buf[p // s].copy_(engine.power(A, 1)[0])
                    else:
                        buf[p // s].copy_(A)
        if i0 < n:
            engine.propagate(plan, A, op, n - i0, i0, graph=False)
    g.replay()
    for (kind, _, dst), buf in zip(store, bufs):
        for j in range(buf.shape[0]):
            _store(dst, j, buf[j])
    return True
