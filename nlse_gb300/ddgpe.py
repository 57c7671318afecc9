"""DDGPE: drop-in for the reference's DDGPE (NLSE/ddgpe.py:14-565).

Exciton-polariton driven-dissipative model: two components (exciton,
cavity).  When the pump callback is the class's own laser_excitation, its
term (ddgpe.py:155-156) is applied inside the inverse row pass of each step
instead of as a separate host callback; other callbacks run on the host
after each step as in the reference loop.
"""

from __future__ import annotations

from typing import Union

import numpy as np
import torch

from . import _lib, engine
from .cnlse import CNLSE
from .nlse import __BACKEND__, _host


class DDGPE(CNLSE):
    """A class to solve the 2D driven dissipative Gross-Pitaevskii equation"""

    def __init__(
        self,
        gamma: float,
        power: float,
        window: float,
        g: float,
        omega: float,
        T: float,
        omega_exc: float,
        omega_cav: float,
        detuning: float,
        k_z: float,
        V: np.ndarray = None,
        g12: float = 0,
        NX: int = 1024,
        NY: int = 1024,
        Isat: float = np.inf,
        nl_length: float = 0,
        backend: str = __BACKEND__,
    ) -> None:
        """Same arguments as the reference (ddgpe.py:17-94)."""
        super().__init__(alpha=gamma, power=power, window=window, n2=-g, n12=g12, V=V, L=T,
                         NX=NX, NY=NY, Isat=Isat, nl_length=nl_length, wvl=1e-30, omega=omega,
                         backend=backend)
        self.g = self.n2
        self.g12 = self.n12
        self.g2 = 0
        self.k_z = k_z
        self.gamma = gamma
        self.gamma2 = self.gamma
        self.omega_exc = omega_exc
        self.omega_cav = omega_cav
        self.detuning = detuning
        omega_lp = (omega_exc + omega_cav) / 2 - 0.5 * np.sqrt(
            (omega_exc - omega_cav) ** 2 + (omega) ** 2)
        self.omega_pump = omega_lp + detuning
        self._random = self._device_normal
        # add_noise draws from the library's counter-based generator keyed by
        # this seed and the step index: the same seed gives the same noise
        self.noise_seed = 0

    _DEVICE_ATTRS = ("power", "n2", "alpha", "I_sat", "n22", "n12", "gamma", "g", "omega",
                     "k_z", "omega_exc", "omega_cav", "detuning", "omega_pump")
    _OP_ATTRS = ("delta_z", "alpha", "gamma", "gamma2", "g", "g2", "g12", "I_sat", "I_sat2",
                 "k", "omega")

    def _device_normal(self, loc=0.0, scale=1.0, size=None):
        return torch.randn(size, dtype=torch.float64, device=self._device) * scale + loc

    @staticmethod
    def add_noise(simu, A, t, i, noise: float = 0) -> None:
        """Noise callback (ddgpe.py:96-125) on the device field.

        Adds complex Gaussian noise of standard deviation delta_z per
        quadrature, scaled by noise * sqrt(gamma_k / (4 dX dY)) on component k,
        as the reference; the draws come from nlse_add_noise (Philox4x32-10
        keyed by simu.noise_seed, counter = pixel and step i), so they are
        reproducible and the same for every field of a batch, like the
        reference's (NY, NX) draw broadcast over the batch.
        """
        simu._add_noise(A, i, noise)

    def _noise_sigmas(self, noise: float, nf: int | None = None) -> tuple:
        """Standard deviation of each component's noise: one value, or one per
        field when gamma / gamma2 are per-field arrays (the reference
        broadcasts gamma of shape (B, 1, 1) against its (NY, NX) draw)."""
        out = []
        for gam in (self.gamma, self.gamma2):
            g = np.asarray(_host(gam), dtype=np.float64).reshape(-1)
            if nf is not None and g.size not in (1, nf):
                raise ValueError(f"gamma with {g.size} values for {nf} fields")
            if np.iscomplexobj(self.delta_z):
                # the reference draws with scale=delta_z, which a complex step
                # makes fail (ddgpe.py:114-119)
                raise TypeError("add_noise: the noise scale delta_z must be real")
            out.append(noise * np.sqrt(g / (4 * (self.delta_X * self.delta_Y))) * self.delta_z)
        return tuple(out)

    def _add_noise(self, A, i: int, noise: float) -> None:
        engine.require_cuda(A)
        lead = self._lead_shape(tuple(A.shape))
        nf = int(np.prod(lead)) if lead else 1
        s0, s1 = self._noise_sigmas(noise, nf)
        lib = _lib.load()
        pix = self.NY * self.NX
        seed = int(self.noise_seed) & (2**64 - 1)
        with torch.cuda.device(A.device):
            st = engine.stream_handle(A.device)
            if s0.size == 1 and s1.size == 1:
                _lib.check(lib.nlse_add_noise(A.data_ptr(), engine.dtype_code(A), nf, pix,
                                              float(s0[0]), float(s1[0]), seed, int(i), st),
                           "add_noise")
                return
            # per-field scales: the same draws (counter = pixel and step) for
            # every field, each field scaled by its own gamma
            s0 = np.broadcast_to(s0, (nf,))
            s1 = np.broadcast_to(s1, (nf,))
            fbytes = 2 * pix * A.element_size()
            for f in range(nf):
                _lib.check(lib.nlse_add_noise(A.data_ptr() + f * fbytes, engine.dtype_code(A), 1, pix,
                                              float(s0[f]), float(s1[f]), seed, int(i), st),
                           "add_noise")

    @staticmethod
    def laser_excitation(simu, A, t, i, F_pump_r, F_pump_t, F_probe_r, F_probe_t) -> None:
        """Pump and probe source on the cavity field (ddgpe.py:127-156).

        Used as a host callback only when it cannot be fused (see
        _split_fused_callbacks).
        """
        dev = A.device
        fr = engine.to_device(F_pump_r, dev, A.dtype)
        qr = engine.to_device(F_probe_r, dev, A.dtype)
        ft = complex(np.asarray(_host(F_pump_t))[i])
        qt = complex(np.asarray(_host(F_probe_t))[i])
        A[..., 1, :, :] -= fr * ft * simu.delta_z * 1j
        A[..., 1, :, :] -= qr * qt * simu.delta_z * 1j

    def _build_propagator(self) -> np.ndarray:
        """Exciton (flat) and cavity (dispersive) propagators (ddgpe.py:204-224)."""
        propagator1 = np.exp(
            -1j * (self.omega_exc * (1 + 0 * self.Kxx**2) - self.omega_pump) * self.delta_z
        ).astype(np.complex64)
        propagator2 = np.exp(
            -1j * (self.omega_cav * np.sqrt(1 + (self.Kxx**2 + self.Kyy**2) / self.k_z**2)
                   - self.omega_pump) * self.delta_z
        ).astype(np.complex64)
        return np.array([propagator1, propagator2])

    def _prepare_output_array(self, E_in, normalize: bool) -> tuple:
        """Plain copy; the reference never normalises here (ddgpe.py:226-245)."""
        return super()._prepare_output_array(E_in, False)

    def _rabi_enabled(self, precision: str) -> bool:
        return precision == "single" and self.omega is not None

    def _nl_block(self, lead: tuple, precision: str, has_v: bool) -> np.ndarray:
        """Branch-specific arguments of DDGPE.split_step (ddgpe.py:288-457), as used there."""
        nf = int(np.prod(lead)) if lead else 1
        na = len(self._last_axes)
        pf = lambda x, name: engine.per_field(_host(x), lead, na, name)  # noqa: E731
        P = np.zeros((nf, _lib.NLSE_PARAM_STRIDE), dtype=np.float64)
        dz = self.delta_z  # complex for imaginary-time steps (nlse.py:505-508)
        g, g2, g12 = pf(self.g, "g"), pf(self.g2, "g2"), pf(self.g12, "g12")
        is1, is2 = pf(self.I_sat, "Isat"), pf(self.I_sat2, "Isat2")
        ga1, ga2 = pf(_host(self.gamma) / 2, "gamma"), pf(_host(self.gamma2) / 2, "gamma2")
        al1 = pf(_host(self.alpha) / 2, "alpha")
        one = np.ones(nf)

        def put(set_, comp, dzs, a, gs, vs):
            o = set_ * 16 + comp * 7
            P[:, o:o + 7] = np.stack([np.real(dzs) * one, a, gs, g12, is1, is2, vs * one], axis=1)
            P[:, 32 + set_] = np.imag(dzs)

        if precision == "double":
            if not has_v:  # ddgpe.py:300-321 and 366-387
                for s in (0, 1):
                    put(s, 0, dz / 2, ga1, g, 0.0)
                    put(s, 1, dz / 2, ga2, g, 0.0)
            else:  # ddgpe.py:323-346 (before) and 389-411 (after)
                put(1, 0, dz, ga1, g, 1.0)
                put(1, 1, dz, ga2, g2, 1.0)
                put(0, 0, dz, ga1, g, self.k / 2)
                put(0, 1, dz, ga2, g2, 1.0)
        else:
            if not has_v:  # ddgpe.py:413-434
                put(0, 0, dz, al1, g, 0.0)
                put(0, 1, dz, ga2, g2, 0.0)
            else:  # ddgpe.py:436-455
                put(0, 0, dz, ga1, g, 1.0)
                put(0, 1, dz, ga2, g2, 1.0)
        if self.omega is not None:
            w = pf(_host(self.omega) / 2, "omega")
            # the reference's cp.cos / cp.sin of the step, complex for a complex
            # step (kernels_gpu.py:155-156)
            cw, sw = np.cos(w * dz), np.sin(w * dz)
            P[:, 14], P[:, 15] = np.real(cw), np.real(sw)
            P[:, 34], P[:, 35] = np.imag(cw), np.imag(sw)
        P[:, 30], P[:, 31] = np.real(dz), np.imag(dz)
        return P

    def _split_fused_callbacks(self, callback, callback_args, A):
        """Fuse a leading DDGPE.laser_excitation callback into the step kernels."""
        if not isinstance(callback, list) or not callback:
            return None, callback, callback_args
        if getattr(callback[0], "__func__", callback[0]) is not DDGPE.laser_excitation:
            return None, callback, callback_args
        args = list(callback_args[0])
        if len(args) != 4:
            return None, callback, callback_args
        dev = A.device
        pix = tuple(A.shape[-2:])
        out = []
        for r, t in ((args[0], args[1]), (args[2], args[3])):
            rd = engine.to_device(r, dev, A.dtype)
            if tuple(rd.shape) != pix:
                return None, callback, callback_args  # per-field profiles: host callback
            td = engine.to_device(np.asarray(_host(t)).reshape(-1), dev, A.dtype)
            out += [rd, td]
        rest = callback[1:]
        rest_args = list(callback_args[1:])
        self._pump_len = int(min(out[1].numel(), out[3].numel()))
        return tuple(out), (rest if rest else None), rest_args

    def out_field(
        self,
        E_in,
        t: float,
        laser_excitation: Union[callable, None],
        plot: bool = False,
        precision: str = "single",
        verbose: bool = True,
        callback: Union[list[callable], callable] = None,
        callback_args: Union[list[tuple], tuple] = None,
    ) -> None:
        """Propagate to time t with the pump as callback 0 (ddgpe.py:519-565).

        Like the reference, returns None: results are read through callbacks.
        """
        if callback is None:
            callback = []
        if laser_excitation is None:
            callback.insert(0, self.laser_excitation)
        else:
            callback.insert(0, laser_excitation)
        super().out_field(E_in=E_in, z=t, plot=plot, precision=precision, verbose=verbose,
                          normalize=False, callback=callback, callback_args=callback_args)
