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
