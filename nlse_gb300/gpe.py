"""GPE: drop-in for the reference's GPE (NLSE/gpe.py:15-176).

Re-parameterises NLSE (k := m, n2 := g, Isat := sat * eps0 c / 2) and uses
the NLSE split step unchanged.
"""

from __future__ import annotations

from typing import Union

import numpy as np
from scipy.constants import atomic_mass, c, epsilon_0, hbar

from . import engine
from .nlse import NLSE, __BACKEND__


class GPE(NLSE):
    """A class to solve GPE."""

    def __init__(
        self,
        gamma: float,
        N: float,
        window: float,
        g: float,
        V: Union[np.ndarray, None],
        m: float = 87 * atomic_mass,
        NX: int = 1024,
        NY: int = 1024,
        sat: float = np.inf,
        nl_length: float = 0,
        backend: str = __BACKEND__,
    ) -> None:
        """Same arguments as the reference (gpe.py:18-79)."""
        super().__init__(alpha=gamma, power=N, window=window, n2=g, V=V, L=0, NX=NX, NY=NY,
                         Isat=sat, nl_length=nl_length, wvl=2 * np.pi / m, backend=backend)
        self.g = g
        self.V = V
        self.gamma = self.alpha
        self.N = self.power
        self.m = self.k
        self.sat = sat
        self.delta_t = self.delta_z
        self.I_sat *= epsilon_0 * c / 2

    def _build_propagator(self) -> np.ndarray:
        """exp(-i hbar K^2/(2m) delta_t), complex64 (gpe.py:81-90); uses delta_t."""
        return np.exp(
            -1j * 0.5 * hbar * (self.Kxx**2 + self.Kyy**2) / self.m * self.delta_t
        ).astype(np.complex64)

    def _norm_coef(self) -> float:
        """Atom number: no c eps0 / 2 factor (gpe.py:106-116)."""
        return self.delta_X * self.delta_Y

    def _norm_target(self, lead: tuple) -> np.ndarray:
        return engine.per_field(self.N, lead, 0, "N")
