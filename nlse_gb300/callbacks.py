"""Callbacks with the reference's signature cb(simu, A, z, i, *args).

Mirrors NLSE/callbacks.py:1-112 for device (torch) fields.  Reductions are
accumulated in FP64 on the device (libnlse_sm103 nlse_power); a result is
copied to the host only when the destination array is a NumPy array.
"""

from __future__ import annotations

import numpy as np
import torch
from scipy.constants import c, epsilon_0

from . import _lib, engine


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


def _host(x):
    """A parameter as NumPy sees it: device tensors become NumPy arrays (a
    0-d array stays an array), Python and NumPy scalars are kept."""
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return x


def index_change_params(n2, isat, shape: tuple, na: int, complex64: bool, adapt: bool):
    """Host part of index_change_setup: (pix, coef, isat, flags, out dtype)
    with coef and isat FP64 NumPy arrays of one value per segment, or None.

    The precisions follow NumPy's rules for the callbacks' expressions
    (callbacks.py:80-82 and 108-110): |A|^2 in the field precision; a
    parameter that NumPy treats as a weak scalar (a Python float) is rounded
    to it, a float64 array or NumPy scalar widens the product or quotient it
    enters -- np.abs(n2) of adapt_delta_z is a float64 NumPy scalar."""
    if len(shape) < na or int(np.prod(shape)) == 0:
        return None
    pix = int(np.prod(shape[len(shape) - na:]))
    lead = tuple(shape[:len(shape) - na])
    asq = np.dtype(np.float32 if complex64 else np.float64)
    cf = np.abs(n2) if adapt else c * epsilon_0 / 2 * n2
    try:
        tc, td = np.result_type(asq, cf), np.result_type(asq, isat)
    except TypeError:
        return None
    real = (np.dtype(np.float32), np.dtype(np.float64))
    if tc not in real or td not in real:
        return None
    flags = 0
    if asq == np.float32:
        flags = ((_lib.DN_COEF_F64 if tc == np.float64 else 0)
                 | (_lib.DN_ISAT_F64 if td == np.float64 else 0))
    segs = []
    for v in (cf, isat):
        x = np.asarray(v, dtype=np.float64)
        if x.ndim > len(shape):
            return None
        k = max(0, x.ndim - na)
        if any(d != 1 for d in x.shape[k:]):
            return None  # varies across the grid
        try:
            if tuple(np.broadcast_shapes(tuple(shape), x.shape)) != tuple(shape):
                return None
            xb = np.broadcast_to(x.reshape(x.shape[:k]), lead)
        except ValueError:
            return None
        segs.append(np.ascontiguousarray(xb, dtype=np.float64).reshape(-1))
    out = np.dtype(np.float64 if (flags or asq == np.float64) else np.float32)
    return pix, segs[0], segs[1], flags, out


def index_change_setup(simu, A, adapt: bool):
    """Per-segment parameters of the callbacks' index change on the device:
    (pix, coef, isat, flags, out dtype), coef and isat FP64 device arrays
    with one value per segment (field, component) of pix points; None where
    the field is not a contiguous CUDA tensor or a parameter does not map
    onto whole segments (the callback then evaluates its expression as is)."""
    if not (isinstance(A, torch.Tensor) and A.is_cuda and A.is_contiguous()
            and A.dtype in (torch.complex64, torch.complex128)):
        return None
    na = len(getattr(simu, "_last_axes", (-2, -1)))
    r = index_change_params(_host(simu.n2), _host(simu.I_sat), tuple(A.shape), na,
                            A.dtype == torch.complex64, adapt)
    if r is None:
        return None
    pix, cf, isat, flags, out = r
    odt = torch.float64 if out == np.float64 else torch.float32
    return (pix, torch.from_numpy(cf).to(A.device), torch.from_numpy(isat).to(A.device), flags,
            odt)


def _delta_n_device(A, setup) -> torch.Tensor:
    pix, cf, isat, flags, odt = setup
    out = torch.empty(A.shape, dtype=odt, device=A.device)
    engine.delta_n(A, pix, cf, isat, flags, out)
    return out


def _peak_to_delta_z(simu, peak):
    """callbacks.py:111-112 on the peak (a NumPy scalar of the peak's precision)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        z_nl = float(1 / (simu.k * peak))
    return np.abs(z_nl) / 12


def evaluate_delta_n(simu, A, z: float, i: int, save_every: int, delta_n) -> None:
    """Nonlinear index change every save_every steps (callbacks.py:57-82);
    on a CUDA field by nlse_delta_n."""
    if i % save_every == 0:
        setup = index_change_setup(simu, A, adapt=False)
        if setup is not None:
            _store(delta_n, i // save_every, _delta_n_device(A, setup))
            return
        A_sq = A.real * A.real + A.imag * A.imag
        _store(delta_n, i // save_every,
               c * epsilon_0 / 2 * simu.n2 * A_sq / (1 + A_sq / simu.I_sat))


def adapt_delta_z(simu, A, z: float, i: int, update_every: int, delta_z: list) -> None:
    """Adaptive step from the peak index change (callbacks.py:85-112); on a
    CUDA field the peak comes from nlse_delta_n_max (one value read back).

    Keeps the reference's expression, in which c eps0 / 2 multiplies only the
    imaginary part (callbacks.py:109).
    """
    delta_z.append(simu.delta_z)
    if i % update_every == 0:
        setup = index_change_setup(simu, A, adapt=True)
        if setup is not None:
            pix, n2a, isat, flags, odt = setup
            buf = torch.empty(1, dtype=torch.float64, device=A.device)
            engine.delta_n_max(A, pix, n2a, isat, c, epsilon_0, flags, buf)
            peak = (np.float64 if odt == torch.float64 else np.float32)(buf.item())
            simu.delta_z = _peak_to_delta_z(simu, peak)
            return
        A_sq = A.real * A.real + A.imag * A.imag * c * epsilon_0 / 2
        n2 = simu.n2
        if isinstance(n2, torch.Tensor):
            n2 = n2.abs()
        else:
            n2 = np.abs(n2)
        delta_n = n2 * A_sq / (1 + A_sq / simu.I_sat)
        peak = delta_n.max()
        if isinstance(peak, torch.Tensor):
            peak = (np.float64 if peak.dtype == torch.float64 else np.float32)(peak.item())
        simu.delta_z = _peak_to_delta_z(simu, peak)


# ---- callbacks as graph nodes ------------------------------------------------
# norm, sample and evaluate_delta_n read only the live field, so when every
# callback of a loop is one of them the whole z-loop becomes one CUDA graph:
# segments of steps up to each recording step, then the recording nodes (an
# FP64 power sum, a device copy or the index-change kernel writing into a
# preallocated slot).  Results reach the caller's arrays once, after the
# loop.  No per-step host synchronisation.  adapt_delta_z changes the step
# count as it goes: its loop synchronises once per update (run_adaptive).

def device_plan(simu, callback, callback_args):
    """[(kind, every, payload)] if every callback can run on the device without
    a per-step host step, else None (NLSE_DEVICE_CALLBACKS=0 turns this off).
    Kinds: "norm", "sample" and "delta_n" (payload: the destination array),
    "adapt" (adapt_delta_z; payload: the caller's step list) and, for DDGPE,
    "noise" (payload: a function (A, step) adding that step's noise)."""
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
        kind = {norm: "norm", sample: "sample", evaluate_delta_n: "delta_n",
                adapt_delta_z: "adapt"}.get(fn)
        if kind is not None:
            if len(args) != 2 or int(args[0]) <= 0:
                return None
            if kind == "adapt" and not hasattr(args[1], "append"):
                return None
            out.append((kind, int(args[0]), args[1]))
        elif noise_fn is not None and fn is noise_fn and hasattr(simu, "_add_noise"):
            amp = float(args[0]) if len(args) else 0.0
            simu._noise_sigmas(amp)  # raises here, not inside a capture, if unsupported
            out.append(("noise", 1, lambda A, step, amp=amp: simu._add_noise(A, step, amp)))
        else:
            return None
    kinds = [k for k, _, _ in out]
    if "adapt" in kinds and (kinds.count("adapt") > 1 or "noise" in kinds):
        return None  # one step size per loop; the noise amplitude follows it
    return out


def _setups(simu, A, recs):
    """index_change_setup of every delta_n record (None if one has none)."""
    out = []
    for kind, _, _ in recs:
        if kind == "delta_n":
            st = index_change_setup(simu, A, adapt=False)
            if st is None:
                return None
            out.append(st)
        else:
            out.append(None)
    return out


def _record(kind, A, setup):
    if kind == "norm":
        return engine.power(A, 1)[0]
    if kind == "sample":
        return A.clone()
    return _delta_n_device(A, setup)


def run_in_graph(simu, plan, A: torch.Tensor, op, n: int, recs) -> bool:
    """Advance A by n steps with the callbacks of recs as graph nodes; False
    (nothing done) if the recording buffers would not fit comfortably or a
    delta_n record has no device form."""
    setups = _setups(simu, A, recs)
    if setups is None:
        return False
    store = [(k, s, d, st) for (k, s, d), st in zip(recs, setups) if k != "noise"]
    counts = [len(range(0, n, s)) for _, s, _, _ in store]

    def rec_bytes(k, st):
        if k == "norm":
            return 8
        if k == "sample":
            return A.numel() * A.element_size()
        return A.numel() * (8 if st[4] == torch.float64 else 4)

    need = sum(c * rec_bytes(k, st) for (k, _, _, st), c in zip(store, counts))
    free, _ = torch.cuda.mem_get_info(A.device)
    if need > free // 4:
        return False

    def buffer(k, st, c):
        if k == "norm":
            return torch.empty((c,), dtype=torch.float64, device=A.device)
        dt = A.dtype if k == "sample" else st[4]
        return torch.empty((c,) + tuple(A.shape), dtype=dt, device=A.device)

    bufs = [buffer(k, st, c) for (k, _, _, st), c in zip(store, counts)]
    points = sorted({i for _, s, _ in recs for i in range(0, n, s)})
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        i0 = 0
        for p in points:
            engine.propagate(plan, A, op, p + 1 - i0, i0, graph=False)
            i0 = p + 1
            j = 0
            for (kind, s, payload), st in zip(recs, setups):  # in the callbacks' order
                if kind == "noise":
                    payload(A, p)
                    continue
                buf = bufs[j]
                j += 1
                if p % s == 0:
                    if kind == "norm":
                        buf[p // s].copy_(engine.power(A, 1)[0])
                    elif kind == "sample":
                        buf[p // s].copy_(A)
                    else:
                        pix, cf, isat, flags, _ = st
                        engine.delta_n(A, pix, cf, isat, flags, buf[p // s])
        if i0 < n:
            engine.propagate(plan, A, op, n - i0, i0, graph=False)
    g.replay()
    for (kind, _, dst, _), buf in zip(store, bufs):
        for j in range(buf.shape[0]):
            _store(dst, j, buf[j])
    return True


def run_adaptive(simu, plan, A: torch.Tensor, op, z: float, recs, refresh,
                 plen: int | None = None) -> bool:
    """The z-loop of out_field (nlse.py:570-586) with adapt_delta_z among
    device callbacks.  Between two updates the step is constant, so the steps
    up to the next update run as graph replays with the other records as
    device work; at an update step nlse_delta_n_max leaves the peak on the
    device and one 8-byte read gives the new step (callbacks.py:108-112,
    evaluated on the host as the reference does), which refresh() writes into
    the operator's parameter block in place (the captured step graphs read it
    there).  As in the reference, the propagator keeps the initial step; the
    nonlinear step and the distance count take the new one (z_prop advances
    by the step in force after each step's callbacks).  Records reach the
    caller's arrays after the loop.  False (nothing done) if a record has no
    device form."""
    setups = _setups(simu, A, recs)
    ad = index_change_setup(simu, A, adapt=True)
    if setups is None or ad is None:
        return False
    (u, dzs), = [(s, d) for k, s, d in recs if k == "adapt"]
    others = [(k, s, d, st) for (k, s, d), st in zip(recs, setups) if k != "adapt"]
    peak_buf = torch.empty(1, dtype=torch.float64, device=A.device)
    peak_type = np.float64 if ad[4] == torch.float64 else np.float32
    pending = []
    timed = op.pump is not None  # the step index matters only for time profiles

    def advance(i0, n):
        if n > 0:
            engine.propagate(plan, A, op, n, i0 if timed else 0, graph=n > 4)

    z_prop, i = 0, 0
    while abs(z_prop) < z:
        dz = simu.delta_z
        # steps i..j share dz: up to the next update step, or the last step
        j, zp, upd = i, z_prop, False
        while True:
            if j % u == 0:
                upd = True
                break
            zp += dz
            if not abs(zp) < z:
                break
            j += 1
        if plen is not None and j >= plen:
            raise IndexError(f"pump time profile index {j} out of range ({plen})")
        i0 = i
        for p in range(i, j + 1):
            hits = [(k, s, d, st) for k, s, d, st in others if p % s == 0]
            if hits or p == j:
                advance(i0, p + 1 - i0)
                i0 = p + 1
            for k, s, d, st in hits:
                pending.append((d, p // s, _record(k, A, st)))
        dzs.extend([dz] * (j + 1 - i))
        if upd:
            pix, n2a, isat, flags, _ = ad
            engine.delta_n_max(A, pix, n2a, isat, c, epsilon_0, flags, peak_buf)
            simu.delta_z = _peak_to_delta_z(simu, peak_type(peak_buf.item()))
            refresh()
            zp += simu.delta_z
        z_prop, i = zp, j + 1
    for d, idx, v in pending:
        _store(d, idx, v)
    return True
