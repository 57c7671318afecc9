"""Learned surrogate of the 256^2 NLSE propagation, with the split-step solver
as data source, fallback and judge.

Workload: the 164-field configuration's distributions restricted to 256 x 256
(power ~ U[0.1, 2] W, n2 = -10^U[-10, -8.4] m^2/W, Gaussian beam of waist
~ U[0.8, 2.5] mm, potential = sum of 1-8 Gaussian wells of depth
U[0.5, 2]e-4 and width U[30, 150] um centred in the inner half-window;
Isat = 1e5 W/m^2, alpha = 20 /m, L = 10 mm, dz = 5e-5 m, window 4 x 2.23 mm).
The solver's output ("fine") is out_field(E0, L) with those parameters:
count_steps(L, dz) = 201 Lie steps, i.e. a propagation length of 201 dz.

Prediction (residual form): a coarse solve over the same length, `coarse`
Strang steps, gives E_c; the network (fno.FNO) maps (Re E_c/a, Im E_c/a,
V/1e-4) on the grid and the scalars (power, log10 |n2|) to the correction
(E_fine - E_c) / (a * RES), where a is the factor out_field's power
normalisation applies to E0.  Prediction: E_c + a * RES * net(...).  The
nonlinear and potential phases of this workload reach tens of radians over L,
which a 32-mode network does not map to 1e-2 from E0 alone; the correction to
a coarse solve is small and smooth.  "Without the network" means E_c alone.

Judge (the solver decides):
  * power check: the predicted field's power must lie within tol of
    [P0 exp(-alpha L'), P0] (L' the propagation length).  Under the GPU path's
    saturated loss the power decays more slowly than P0 exp(-alpha L'), so
    that is a lower bound, and the loss term cannot create power;
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
from .nlse import NLSE, count_steps

N = 256
WINDOW, ALPHA, L, ISAT, DZ = 4 * 2.23e-3, 20.0, 10e-3, 1e5, 5e-5
P_MID, P_HALF = 1.05, 0.95
LOGN2_MID, LOGN2_HALF = -9.2, 0.8
V_SCALE = 1e-4
RES = 0.05  # scale of the learned correction relative to the field
MAX_WELLS = 8


def _grid():
    sim = NLSE(ALPHA, 1.0, WINDOW, -1e-9, None, L, NX=N, NY=N, Isat=ISAT)
    return sim.X, sim.Y, sim.delta_X, sim.delta_Y


def fine_length() -> float:
    """Propagation length of the solver's out_field(E0, L) loop (201 steps of dz)."""
    return count_steps(L, DZ) * DZ


def sample_inputs(n: int, seed: int = 0, device="cuda") -> dict:
    """n seeded input sets: E0 (n, N, N) complex64 unit-peak beams and V (n, N, N)
    float32 on the device; power (n,), n2 (n,) as host arrays."""
    rng = np.random.default_rng(seed)
    power = rng.uniform(0.1, 2.0, n)
    n2 = -(10.0 ** rng.uniform(-10, -8.4, n))
    waist = rng.uniform(0.8e-3, 2.5e-3, n)
    count = rng.integers(1, MAX_WELLS + 1, n)
    depth = rng.uniform(0.5e-4, 2e-4, (n, MAX_WELLS)) * (np.arange(MAX_WELLS) < count[:, None])
    width = rng.uniform(30e-6, 150e-6, (n, MAX_WELLS))
    centre = rng.uniform(-WINDOW / 4, WINDOW / 4, (n, MAX_WELLS, 2))
    X, Y, _, _ = _grid()
    f64 = dict(dtype=torch.float64, device=device)
    Xd, Yd = torch.as_tensor(X, **f64), torch.as_tensor(Y, **f64)
    w = torch.as_tensor(width, **f64)[..., None]
    gx = torch.exp(-(Xd - torch.as_tensor(centre[..., 0], **f64)[..., None]) ** 2 / w**2)
    gy = torch.exp(-(Yd - torch.as_tensor(centre[..., 1], **f64)[..., None]) ** 2 / w**2)
    # V[y][x] = -sum_k depth_k gy_k(y) gx_k(x): one batched product of (N x wells) (wells x N)
    V = -torch.bmm((gy * torch.as_tensor(depth, **f64)[..., None]).transpose(1, 2), gx)
    wb = torch.as_tensor(waist, **f64)[:, None]
    E0 = torch.exp(-Yd**2 / wb**2)[:, :, None] * torch.exp(-Xd**2 / wb**2)[:, None, :]
    return {"E0": E0.to(torch.complex64).contiguous(), "V": V.to(torch.float32).contiguous(),
            "power": power, "n2": n2}


def subset(inp: dict, idx) -> dict:
    """Input sets idx (a slice or an index array)."""
    out = {}
    for k, v in inp.items():
        if isinstance(v, torch.Tensor) and not isinstance(idx, slice):
            out[k] = v[torch.as_tensor(np.asarray(idx), device=v.device)]
        else:
            out[k] = v[idx]
    return out


def scale(inp: dict) -> torch.Tensor:
    """a per field (device, float64): the factor out_field's power normalisation applies to E0."""
    _, _, dx, dy = _grid()
    E0 = inp["E0"]
    s = engine.power(E0.contiguous(), E0.shape[0]) * (dx * dy * c * epsilon_0 / 2)
    return torch.sqrt(torch.as_tensor(inp["power"], dtype=torch.float64, device=E0.device) / s)


def solve(inp: dict, steps: int | None = None, chunk: int = 2048) -> torch.Tensor:
    """E at the solver's propagation length for every input set, (n, N, N)
    complex64 on the device.  steps=None: the solver itself (out_field(E0, L),
    Lie scheme, dz = 5e-5); otherwise `steps` Strang steps over the same length."""
    E0all = inp["E0"]
    n = E0all.shape[0]
    out = torch.empty((n, N, N), dtype=torch.complex64, device=E0all.device)
    for b0 in range(0, n, chunk):
        sl = slice(b0, min(n, b0 + chunk))
        B = sl.stop - sl.start
        sim = NLSE(ALPHA, inp["power"][sl], WINDOW, inp["n2"][sl].reshape(B, 1, 1), None, L,
                   NX=N, NY=N, Isat=ISAT)
        sim.V = inp["V"][sl]
        if steps is None:
            sim.delta_z = DZ
            out[sl] = sim.out_field(E0all[sl], L, verbose=False)
        else:
            dz = fine_length() / steps
            sim.delta_z = dz
            out[sl] = sim.out_field(E0all[sl], (steps - 0.5) * dz, precision="double",
                                    verbose=False)
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
    """Coarse Strang solve plus a learned correction, judged by the solver."""

    def __init__(self, device="cuda", seed: int = 0, coarse: int = 4):
        self.dev = torch.device(device)
        self.coarse = coarse
        self.net = FNO(self.dev, seed)
        self.net.init(seed, out_scale=1e-2)
        self.history: list = []

    def features(self, inp: dict, Ec: torch.Tensor):
        a = scale(inp).to(torch.float32)
        e = Ec / a[:, None, None]
        xin = torch.stack([e.real, e.imag, inp["V"] / V_SCALE], dim=-1).contiguous()
        xs = torch.as_tensor(np.stack([(inp["power"] - P_MID) / P_HALF,
                                       (np.log10(-inp["n2"]) - LOGN2_MID) / LOGN2_HALF], -1),
                             dtype=torch.float32, device=self.dev)
        return xin, xs, a

    def fit(self, inp: dict, E_f: torch.Tensor, epochs: int = 10, batch: int = 32,
            lr: float = 2e-3, time_budget: float | None = None, seed: int = 0,
            E_c: torch.Tensor | None = None) -> list:
        """Adam on mean_b ||pred_b - E_f,b||^2 / ||E_f,b||^2 (cosine learning-rate decay)."""
        Ec = solve(inp, self.coarse) if E_c is None else E_c
        xin, xs, a = self.features(inp, Ec)
        sa = (a * RES)[:, None, None]
        tgt = ((E_f - Ec) / sa).to(torch.complex64)
        ref = (E_f / sa).to(torch.complex64)
        n = xin.shape[0]
        order = torch.from_numpy(np.random.default_rng(seed).permutation(n)).to(self.dev)
        xin, xs = xin[order].contiguous(), xs[order].contiguous()
        tgt, ref = tgt[order].contiguous(), ref[order].contiguous()
        steps_per_epoch = max(1, n // batch)
        total = epochs * steps_per_epoch
        t0 = time.perf_counter()
        step = 0
        for ep in range(epochs):
            shift = (ep * batch // 3) % max(1, n - batch + 1)
            for i in range(steps_per_epoch):
                b0 = (shift + i * batch) % max(1, n - batch + 1)
                sl = slice(b0, b0 + batch)
                lr_t = lr * 0.5 * (1 + math.cos(math.pi * step / total))
                self.history.append(self.net.train_step(xin[sl], xs[sl], tgt[sl], lr_t, ref=ref[sl]))
                step += 1
                if time_budget is not None and time.perf_counter() - t0 > time_budget:
                    return self.history
        return self.history

    def predict(self, inp: dict, E_c: torch.Tensor | None = None,
                with_coarse: bool = False):
        """Predicted E at the solver's propagation length (and optionally E_c)."""
        Ec = solve(inp, self.coarse) if E_c is None else E_c
        xin, xs, a = self.features(inp, Ec)
        P = Ec + self.net.predict(xin, xs) * (a * RES)[:, None, None]
        return (P, Ec) if with_coarse else P

    def judge(self, inp: dict, E_pred: torch.Tensor, every: int = 16, seed: int = 0,
              tol: float = 1e-2, max_fail: float = 0.25):
        """Checked output fields and a report (see the module docstring)."""
        n = E_pred.shape[0]
        out = E_pred.clone()
        P0 = torch.as_tensor(inp["power"], dtype=torch.float64, device=self.dev)
        Pp = power(out)
        lo = P0 * math.exp(-ALPHA * fine_length()) * (1 - tol)
        bad_power = ((Pp < lo) | (Pp > P0 * (1 + tol))).cpu().numpy()
        rng = np.random.default_rng(seed)
        k = max(1, math.ceil(n / every))
        sample = np.sort(rng.choice(n, size=k, replace=False))
        E_s = solve(subset(inp, sample))
        err = rel_l2(out[torch.as_tensor(sample, device=self.dev)], E_s).cpu().numpy()
        fail = err > tol
        if fail.any():
            out[torch.as_tensor(sample[fail], device=self.dev)] = \
                E_s[torch.as_tensor(np.nonzero(fail)[0], device=self.dev)]
        whole = bool(fail.mean() > max_fail)
        redo = (np.setdiff1d(np.arange(n), sample) if whole
                else np.setdiff1d(np.nonzero(bad_power)[0], sample))
        if redo.size:
            out[torch.as_tensor(redo, device=self.dev)] = solve(subset(inp, redo))
        report = {"fields": n, "sampled": int(k), "sample_rel_l2_median": float(np.median(err)),
                  "sample_rel_l2_max": float(err.max()), "sample_failed": int(fail.sum()),
                  "power_check_failed": int(bad_power.sum()), "batch_resolved": whole,
                  "resolved": int(k + redo.size), "surrogate_kept": int(n - k - redo.size)}
        return out, report
