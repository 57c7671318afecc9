"""Learned surrogate of the 256^2 NLSE propagation, with the solver as data
source, fallback and judge.

Workload: the 164-field configuration's distributions restricted to 256 x 256
(power ~ U[0.1, 2] W, n2 = -10^U[-10, -8.4] m^2/W, Gaussian beam of waist
~ U[0.8, 2.5] mm, potential = sum of 1-8 Gaussian wells of depth
U[0.5, 2]e-4 and width U[30, 150] um centred in the inner half-window;
Isat = 1e5 W/m^2, alpha = 20 /m, L = 10 mm, dz = 5e-5 m, window 4 x 2.23 mm).

The network (fno.FNO) maps (Re E0, Im E0, V) on the grid plus (power, n2)
to E(L) / a, where a is the factor out_field's normalisation applies to E0;
the prediction is a times the network output.

Judge (the solver decides):
  * power check: the predicted field's power must lie within tol of
    [P0 exp(-alpha L), P0].  Under the GPU path's saturated loss the power
    decays more slowly than P0 exp(-alpha L), so that is a lower bound, and
    the loss term cannot create power, so P0 is an upper bound;
  * a seeded 1-in-`every` sample is re-solved; a sampled field whose
    prediction is off by more than tol (relative L2) takes the solver's
    field, and if more than `max_fail` of the sample fails, the whole batch
    is re-solved;
  * fields failing the power check are re-solved.
"""

from __future__ import annotations

import math
import time

import numpy as np
import torch
from scipy.constants import c, epsilon_0

from . import engine
from .fno import FNO
from .nlse import NLSE

N = 256
WINDOW, ALPHA, L, ISAT, DZ = 4 * 2.23e-3, 20.0, 10e-3, 1e5, 5e-5
P_MID, P_HALF = 1.05, 0.95
LOGN2_MID, LOGN2_HALF = -9.2, 0.8
V_SCALE = 1e-4


def _grid():
    sim = NLSE(ALPHA, 1.0, WINDOW, -1e-9, None, L, NX=N, NY=N, Isat=ISAT)
    return sim.XX, sim.YY, sim.delta_X, sim.delta_Y


def sample_inputs(n: int, seed: int = 0) -> dict:
    """n seeded input sets: E0 (n, N, N) complex64 unit-peak beams, V (n, N, N)
    float32, power (n,), n2 (n,)."""
    rng = np.random.default_rng(seed)
    XX, YY, _, _ = _grid()
    power = rng.uniform(0.1, 2.0, n)
    n2 = -(10.0 ** rng.uniform(-10, -8.4, n))
    waist = rng.uniform(0.8e-3, 2.5e-3, n)
    V = np.zeros((n, N, N), np.float32)
    E0 = np.empty((n, N, N), np.complex64)
    r2 = XX**2 + YY**2
    for b in range(n):
        v = np.zeros((N, N))
        for _ in range(rng.integers(1, 9)):
            depth = rng.uniform(0.5e-4, 2e-4)
            width = rng.uniform(30e-6, 150e-6)
            x0, y0 = rng.uniform(-WINDOW / 4, WINDOW / 4, 2)
            v -= depth * np.exp(-((XX - x0) ** 2 + (YY - y0) ** 2) / width**2)
        V[b] = v
        E0[b] = np.exp(-r2 / waist[b] ** 2)
    return {"E0": E0, "V": V, "power": power, "n2": n2}


def subset(inp: dict, idx) -> dict:
    return {k: v[idx] for k, v in inp.items()}


def scale(inp: dict) -> np.ndarray:
    """a per field: the factor out_field's power normalisation applies to E0."""
    _, _, dx, dy = _grid()
    s = np.sum(np.abs(inp["E0"].astype(np.complex128)) ** 2, axis=(1, 2)) * dx * dy * c * epsilon_0 / 2
    return np.sqrt(inp["power"] / s)


def features(inp: dict) -> tuple[np.ndarray, np.ndarray]:
    """Network inputs: xin (n, N, N, 3) = (Re E0, Im E0, V / 1e-4), xs (n, 2)."""
    E0 = inp["E0"]
    xin = np.stack([E0.real, E0.imag, inp["V"] / V_SCALE], axis=-1).astype(np.float32)
    xs = np.stack([(inp["power"] - P_MID) / P_HALF,
                   (np.log10(-inp["n2"]) - LOGN2_MID) / LOGN2_HALF], axis=-1).astype(np.float32)
    return xin, xs


def solve(inp: dict, device="cuda", chunk: int = 2048) -> torch.Tensor:
    """E(L) of every input set by the split-step solver, (n, N, N) complex64 on the device."""
    n = len(inp["power"])
    out = torch.empty((n, N, N), dtype=torch.complex64, device=device)
    for b0 in range(0, n, chunk):
        sl = slice(b0, min(n, b0 + chunk))
        B = sl.stop - sl.start
        sim = NLSE(ALPHA, inp["power"][sl], WINDOW, inp["n2"][sl].reshape(B, 1, 1), None, L,
                   NX=N, NY=N, Isat=ISAT)
        sim.delta_z = DZ
        sim.V = inp["V"][sl]
        E0 = torch.from_numpy(np.ascontiguousarray(inp["E0"][sl])).to(device)
        out[sl] = sim.out_field(E0, L, verbose=False)
    return out


def rel_l2(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Per-field relative L2 distance ||a - b|| / ||b|| (FP64 sums)."""
    d = (a - b).to(torch.complex128).abs().pow(2).sum(dim=(-2, -1))
    n = b.to(torch.complex128).abs().pow(2).sum(dim=(-2, -1))
    return (d / n).sqrt()


def power(E: torch.Tensor) -> torch.Tensor:
    """Per-field power (W) of fields on the grid (FP64 reduction on the device)."""
    _, _, dx, dy = _grid()
    E = E.contiguous()
    return engine.power(E, E.shape[0]) * (dx * dy * c * epsilon_0 / 2)


class Surrogate:
    def __init__(self, device="cuda", seed: int = 0):
        self.dev = torch.device(device)
        self.net = FNO(self.dev, seed)
        self.history: list = []

    def _prepare(self, inp: dict):
        xin, xs = features(inp)
        a = torch.as_tensor(scale(inp), dtype=torch.float32, device=self.dev)
        return (torch.from_numpy(xin).to(self.dev), torch.from_numpy(xs).to(self.dev), a)

    def fit(self, inp: dict, E_L: torch.Tensor, epochs: int = 10, batch: int = 32,
            lr: float = 2e-3, time_budget: float | None = None, seed: int = 0) -> list:
        """Adam on mean relative squared error of E(L)/a; cosine learning-rate decay."""
        xin, xs, a = self._prepare(inp)
        tgt = (E_L.to(self.dev) / a[:, None, None]).to(torch.complex64)
        n = xin.shape[0]
        order = torch.from_numpy(np.random.default_rng(seed).permutation(n)).to(self.dev)
        xin, xs, tgt = xin[order].contiguous(), xs[order].contiguous(), tgt[order].contiguous()
        steps_per_epoch = max(1, n // batch)
        total = epochs * steps_per_epoch
        t0 = time.perf_counter()
        step = 0
        for ep in range(epochs):
            shift = (ep * batch // 3) % max(1, n - batch + 1)
            for i in range(steps_per_epoch):
                b0 = (shift + i * batch) % max(1, n - batch + 1)
                lr_t = lr * 0.5 * (1 + math.cos(math.pi * step / total))
                loss = self.net.train_step(xin[b0:b0 + batch], xs[b0:b0 + batch],
                                           tgt[b0:b0 + batch], lr_t)
                self.history.append(loss)
                step += 1
                if time_budget is not None and time.perf_counter() - t0 > time_budget:
                    return self.history
        return self.history

    def predict(self, inp: dict) -> torch.Tensor:
        xin, xs, a = self._prepare(inp)
        return self.net.predict(xin, xs) * a[:, None, None]

    def judge(self, inp: dict, E_pred: torch.Tensor, every: int = 16, seed: int = 0,
              tol: float = 1e-2, max_fail: float = 0.25):
        """Checked output fields and a report (see the module docstring)."""
        n = E_pred.shape[0]
        out = E_pred.clone()
        P0 = torch.as_tensor(inp["power"], dtype=torch.float64, device=self.dev)
        Pp = power(out)
        lo = P0 * math.exp(-ALPHA * L) * (1 - tol)
        bad_power = ((Pp < lo) | (Pp > P0 * (1 + tol))).cpu().numpy()
        rng = np.random.default_rng(seed)
        k = max(1, math.ceil(n / every))
        sample = np.sort(rng.choice(n, size=k, replace=False))
        E_s = solve(subset(inp, sample), self.dev)
        err = rel_l2(out[sample], E_s).cpu().numpy()
        fail = err > tol
        if fail.any():
            out[torch.as_tensor(sample[fail], device=self.dev)] = \
                E_s[torch.as_tensor(np.nonzero(fail)[0], device=self.dev)]
        whole = bool(fail.mean() > max_fail)
        redo = (np.setdiff1d(np.arange(n), sample) if whole
                else np.setdiff1d(np.nonzero(bad_power)[0], sample))
        if redo.size:
            out[torch.as_tensor(redo, device=self.dev)] = solve(subset(inp, redo), self.dev)
        report = {"fields": n, "sampled": int(k), "sample_rel_l2_median": float(np.median(err)),
                  "sample_rel_l2_max": float(err.max()), "sample_failed": int(fail.sum()),
                  "power_check_failed": int(bad_power.sum()), "batch_resolved": whole,
                  "resolved": int(k + redo.size), "surrogate_kept": int(n - k - redo.size)}
        return out, report
