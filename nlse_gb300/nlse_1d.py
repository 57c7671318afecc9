"""NLSE_1d: drop-in for the reference's NLSE_1d (NLSE/nlse_1d.py:15-132).

The whole z-loop of a 1-D field runs inside one kernel launch: each line is
held on chip across all steps (forward FFT, propagator, inverse FFT and the
nonlinear step per iteration) and written back once.
"""

from __future__ import annotations

from typing import Union

import numpy as np
from scipy.constants import c, epsilon_0

from .nlse import NLSE, __BACKEND__


class NLSE_1d(NLSE):
    """A class to solve NLSE in 1d"""

    def __init__(
        self,
        alpha: float,
        power: float,
        window: float,
        n2: float,
        V: Union[np.ndarray, None],
        L: float,
        NX: int = 1024,
        Isat: float = np.inf,
        nl_length: float = 0,
        wvl: float = 780e-9,
        backend: str = __BACKEND__,
    ) -> None:
        """Same arguments as the reference (nlse_1d.py:18-66)."""
        super().__init__(alpha=alpha, power=power, window=window, n2=n2, V=V, L=L, NX=NX,
                         Isat=Isat, nl_length=nl_length, wvl=wvl, backend=backend)
        self._last_axes = (-1,)
        # first row of the 2-D profile, renormalised (nlse_1d.py:65-66)
        self.nl_profile = self.nl_profile[0]
        self.nl_profile /= self.nl_profile.sum()

    def _norm_coef(self) -> float:
        """The reference integrates with delta_X**2 (nlse_1d.py:86-91)."""
        return self.delta_X**2 * (c * epsilon_0 / 2)

    def _build_propagator(self) -> np.ndarray:
        """Not cast to complex64 (nlse_1d.py:98-105)."""
        return np.exp(-1j * 0.5 * (self.Kx**2) / self.k * self.delta_z)
