"""NLSE_3d: drop-in for the reference's NLSE_3d (NLSE/nlse_3d.py:15-218).

Fields are (..., NY, NX, NT); the transform runs over all three axes: a row
pass along t, column passes along x and y (the y pass fused with the
propagator and GVD multiply), and the inverse row pass fused with the
nonlinear step.
"""

from __future__ import annotations

from typing import Union

import numpy as np
from scipy.constants import c, epsilon_0

from . import engine
from .nlse import NLSE, __BACKEND__, nonlinear_length


class NLSE_3d(NLSE):
    """A class to solve the 3D NLSE i.e propagation of pulses of light in nonlinear media."""

    def __init__(
        self,
        alpha: float,
        energy: float,
        window: Union[list, tuple],
        n2: float,
        D0: float,
        vg: float,
        V: Union[np.ndarray, None],
        L: float,
        NX: int = 1024,
        NY: int = 1024,
        NZ: int = 1024,
        Isat: float = np.inf,
        nl_length: float = 0,
        wvl: float = 780e-9,
        backend: str = __BACKEND__,
    ) -> None:
        """Same arguments as the reference (nlse_3d.py:20-103)."""
        if len(window) == 2:
            window = [window[0], window[0], window[-1]]
        super().__init__(alpha=alpha, power=energy, window=window[0:2], n2=n2, V=V, L=L, NX=NX,
                         NY=NY, Isat=Isat, nl_length=nl_length, wvl=wvl, backend=backend)
        self.energy = self.power
        self.NZ = NZ
        self.window_t = window[-1]
        self.power = self.energy / self.window_t
        z_nl = nonlinear_length(self.k, self.n2, self.power, min(self.window[0:2]) ** 2)
        self.delta_z = 0.5e-2 * z_nl
        self.T, self.delta_T = np.linspace(-self.window_t / 2, self.window_t / 2, self.NZ,
                                           retstep=True)
        self.omega = 2 * np.pi * np.fft.fftfreq(self.NZ, self.delta_T)
        self.D0 = D0
        self.vg = vg
        self.XX, self.YY, self.TT = np.meshgrid(self.X, self.Y, self.T)
        self.Kxx, self.Kyy, self.Omega = np.meshgrid(self.Kx, self.Ky, self.omega)
        self._last_axes = (-3, -2, -1)

    def _build_propagator(self) -> np.ndarray:
        """2-D propagator (complex64) times exp(-i D0/2 Omega^2), no dz (nlse_3d.py:105-114)."""
        prop_2d = super()._build_propagator()
        prop_t = np.exp(-1j * self.D0 / 2 * self.Omega**2)
        return prop_2d * prop_t

    def _norm_coef(self) -> float:
        return self.delta_X * self.delta_Y * self.delta_T * (c * epsilon_0 / 2)

    def _norm_target(self, lead: tuple) -> np.ndarray:
        """Normalised to the energy (nlse_3d.py:116-150)."""
        return engine.per_field(self.energy, lead, 0, "energy")

    _DEVICE_ATTRS = ("power", "n2", "alpha", "I_sat", "energy")
