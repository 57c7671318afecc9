"""CNLSE_1d: drop-in for the reference's CNLSE_1d (NLSE/cnlse_1d.py:13-167)."""

from __future__ import annotations

from typing import Union

import numpy as np
from scipy.constants import c, epsilon_0

from .cnlse import CNLSE
from .nlse import __BACKEND__


class CNLSE_1d(CNLSE):
    """A class to solve the coupled NLSE in 1d"""

    def __init__(
        self,
        alpha: float,
        power: float,
        window: float,
        n2: float,
        n12: float,
        V: Union[np.ndarray, None],
        L: float,
        NX: int = 1024,
        Isat: float = np.inf,
        nl_length: float = 0,
        wvl: float = 780e-9,
        omega: float = None,
        backend: str = __BACKEND__,
    ) -> None:
        """Same arguments as the reference (cnlse_1d.py:16-81)."""
        super().__init__(alpha=alpha, power=power, window=window, n2=n2, n12=n12, V=V, L=L,
                         NX=NX, Isat=Isat, nl_length=nl_length, wvl=wvl, omega=omega,
                         backend=backend)
        self._last_axes = (-1,)
        self.nl_profile = self.nl_profile[0]
        self.nl_profile /= self.nl_profile.sum()

    def _norm_coef(self) -> float:
        """delta_X**2 as in the reference (cnlse_1d.py:95-101)."""
        return self.delta_X**2 * (c * epsilon_0 / 2)

    def _take_components(self, A) -> tuple:
        return A[..., 0, :], A[..., 1, :]

    def _build_propagator(self) -> np.ndarray:
        """Not cast to complex64 (cnlse_1d.py:119-131)."""
        propagator1 = np.exp(-1j * 0.5 * (self.Kx**2) / self.k * self.delta_z)
        propagator2 = np.exp(-1j * 0.5 * (self.Kx**2) / self.k2 * self.delta_z)
        return np.array([propagator1, propagator2])
