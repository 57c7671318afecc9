"""CNLSE: drop-in for the reference's CNLSE (NLSE/cnlse.py:19-423).

Two components stacked at axis -3, (..., 2, NY, NX).  The inverse row pass
holds both components' rows of the same y in one CTA, so the cross-phase,
joint saturation and Rabi rotation read both |A|^2 without another sweep.
"""

from __future__ import annotations

from typing import Union

import numpy as np
import torch
from scipy.constants import c, epsilon_0

from . import _lib, engine
from .nlse import NLSE, __BACKEND__, _host


class CNLSE(NLSE):
    """A class to solve the coupled NLSE"""

    _comps = 2

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
        NY: int = 1024,
        Isat: float = np.inf,
        nl_length: float = 0,
        wvl: float = 780e-9,
        omega: float = None,
        backend: str = __BACKEND__,
    ) -> None:
        """Same arguments as the reference (cnlse.py:22-97)."""
        super().__init__(alpha=alpha, power=power, window=window, n2=n2, V=V, L=L, NX=NX, NY=NY,
                         Isat=Isat, nl_length=nl_length, wvl=wvl, backend=backend)
        self.I_sat2 = self.I_sat
        self.n12 = n12
        self.n22 = self.n2
        self.omega = omega
        self.alpha2 = self.alpha
        self.k2 = self.k
        self.power2 = self.power
        self.propagator1 = None
        self.propagator2 = None

    _DEVICE_ATTRS = ("power", "n2", "alpha", "I_sat", "n22", "n12")
    _OP_ATTRS = ("delta_z", "n2", "alpha", "I_sat", "k", "n22", "n12", "alpha2", "k2",
                 "I_sat2", "omega")

    def _norm_target(self, lead: tuple) -> np.ndarray:
        """[power, power2] per field (cnlse.py:111,137-141)."""
        p1 = engine.per_field(self.power, lead, 0, "power")
        p2 = engine.per_field(self.power2, lead, 0, "power2")
        return np.stack([p1, p2], axis=-1)

    def _build_propagator(self) -> np.ndarray:
        """Both components' propagators, complex64 (cnlse.py:179-190)."""
        propagator1 = super()._build_propagator()
        propagator2 = np.exp(
            -1j * 0.5 * (self.Kxx**2 + self.Kyy**2) / self.k2 * self.delta_z
        ).astype(np.complex64)
        return np.array([propagator1, propagator2])

    def _prop_layout(self, prop: torch.Tensor) -> int:
        na = len(self._last_axes)
        if prop.dim() > na and prop.shape[-na - 1] == 2:
            return int(np.prod(prop.shape[-na:]))
        return 0

    def _take_components(self, A) -> tuple:
        """cnlse.py:192-202."""
        return A[..., 0, :, :], A[..., 1, :, :]

    def _rabi_enabled(self, precision: str) -> bool:
        return precision == "single" and self.omega is not None

    def _nl_block(self, lead: tuple, precision: str, has_v: bool) -> np.ndarray:
        """Per-field, per-component parameters of nl_prop_c (cnlse.py:288-423)."""
        nf = int(np.prod(lead)) if lead else 1
        na = len(self._last_axes)
        P = np.zeros((nf, _lib.NLSE_PARAM_STRIDE), dtype=np.float64)
        pf = lambda x, name: engine.per_field(x, lead, na, name)  # noqa: E731
        k, k2 = self.k, self.k2
        g11 = pf(k / 2 * _host(self.n2) * c * epsilon_0, "n2")
        g12 = pf(k / 2 * _host(self.n12) * c * epsilon_0, "n12")
        g22 = pf(k2 / 2 * _host(self.n22) * c * epsilon_0, "n22")
        g21 = pf(k2 / 2 * _host(self.n12) * c * epsilon_0, "n12")
        is1 = pf(2 * _host(self.I_sat) / (epsilon_0 * c), "Isat")
        is2 = pf(2 * _host(self.I_sat2) / (epsilon_0 * c), "Isat2")
        a1 = pf(_host(self.alpha) / 2, "alpha")
        a2 = pf(_host(self.alpha2) / 2, "alpha2")
        dz = self.delta_z
        for s, dzs in ((0, dz / 2 if precision == "double" else dz), (1, dz / 2)):
            o = s * 16
            P[:, o + 0:o + 7] = np.stack(
                [np.full(nf, np.real(dzs)), a1, g11, g12, is1, is2, np.full(nf, k / 2)], axis=1)
            P[:, o + 7:o + 14] = np.stack(
                [np.full(nf, np.real(dzs)), a2, g22, g21, is2, is1, np.full(nf, k2 / 2)], axis=1)
            P[:, 32 + s] = np.imag(dzs)
        if self.omega is not None:
            w = pf(_host(self.omega) / 2, "omega")
            if np.iscomplexobj(dz):
                # the reference's cp.cos / cp.sin of a complex step (kernels_gpu.py:155-156)
                cw, sw = np.cos(w * dz), np.sin(w * dz)
                P[:, 14], P[:, 15] = cw.real, sw.real
                P[:, 34], P[:, 35] = cw.imag, sw.imag
            else:
                P[:, 14] = np.cos(w * dz)
                P[:, 15] = np.sin(w * dz)
        return P
