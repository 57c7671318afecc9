"""CPU oracle of the split-step path of Quantum-Optics-LKB/NLSE v2.3.0.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py may import this module,
and only as the checker or the timed CPU baseline.  The product
(nlse_gb300) never imports it.

This is a NumPy/SciPy restatement of the reference's GPU-path arithmetic
(backend="GPU", NLSE/kernels_gpu.py semantics), written from the
reference's behaviour.  Every function names the reference lines it
follows.  The one substitution is the FFT: scipy.fft (pocketfft) stands in
for VkFFT (pyvkfft 2024.1.2.post0, a dependency absent from the reference
tree); both compute the same unnormalised forward and 1/N-normalised
inverse C2C transform over the trailing axes.

The oracle is pinned against golden fields produced by running the
reference's own code (tests/golden/make_golden.py, which imports the
reference with NumPy stand-ins for CuPy/pyvkfft) and against the
reference's known-answer tests (identity at dz = 0, power conservation,
propagator closed forms, normalisation).

With cpu_kernels=True the nonlinear step follows the reference's CPU
kernels instead (NLSE/kernels_cpu.py: unsaturated loss in nl_prop); that
variant is the timed CPU baseline.
"""

from __future__ import annotations

import cmath
import math
from typing import Callable

import numpy as np
import scipy.fft as sfft
from scipy import signal, special
from scipy.constants import atomic_mass, c, epsilon_0, hbar

WORKERS = 1  # scipy.fft worker threads (the CPU baseline raises it)


# ---------------------------------------------------------------------------
# Elementwise kernels, GPU semantics (NLSE/kernels_gpu.py)
# ---------------------------------------------------------------------------
def square_mod(A: np.ndarray) -> np.ndarray:
    """|A|^2 via abs then square (kernels_gpu.py:179-190)."""
    return np.abs(A) ** 2


def nl_prop(A, A_sq, dz, alpha, V, g, Isat, cpu_kernels=False) -> None:
    """Saturated Kerr + loss + potential phase, in place (kernels_gpu.py:4-65).

    V may be None (nl_prop_without_V).  cpu_kernels: the loss is not
    saturated (kernels_cpu.py:28-33, 57-62).
    """
    sat = 1 / (1 + A_sq / Isat)
    arg = 1j * g * A_sq * sat
    if cpu_kernels:
        arg = arg + (-alpha)
    else:
        arg += -alpha * sat
    if V is not None:
        arg += 1j * V
    arg *= dz
    A *= np.exp(arg)


def nl_prop_c(A1, A_sq_1, A_sq_2, dz, alpha, V, g11, g12, Isat1, Isat2) -> None:
    """Two-component form with cross phase and joint saturation (kernels_gpu.py:68-139)."""
    sat = 1 / (1 + A_sq_1 * 1 / Isat1 + A_sq_2 * 1 / Isat2)
    arg = 1j * (g11 * A_sq_1 * sat + g12 * A_sq_2 * sat)
    arg += -alpha * sat
    if V is not None:
        arg += 1j * V
    arg *= dz
    A1 *= np.exp(arg)


def rabi_coupling(A1, A2, dz, omega) -> None:
    """Rabi rotation between the components (kernels_gpu.py:142-156).

    cos/sin are Python floats, so they round to the field precision as the
    CuPy fused kernel's scalars do.
    """
    if isinstance(omega * dz, complex):  # a complex step: complex cos and sin
        cw, sw = cmath.cos(omega * dz), cmath.sin(omega * dz)
    else:
        cw, sw = math.cos(omega * dz), math.sin(omega * dz)
    A1_old = A1.copy()
    A1[:] = cw * A1 - 1j * sw * A2
    A2[:] = cw * A2 - 1j * sw * A1_old


# ---------------------------------------------------------------------------
# Step counting of the z-loop (NLSE/nlse.py:568-585)
# ---------------------------------------------------------------------------
def count_steps(z, delta_z) -> int:
    """Iterations of `while abs(z_prop) < z: z_prop += delta_z` (nlse.py:570-585)."""
    z_prop, n = 0, 0
    while abs(z_prop) < z:
        z_prop += delta_z
        n += 1
    return n


# ---------------------------------------------------------------------------
# Solver restatements
# ---------------------------------------------------------------------------
class OracleNLSE:
    """Restatement of NLSE (NLSE/nlse.py:41-619), GPU path."""

    comps = 1

    def __init__(self, alpha, power, window, n2, V, L, NX=1024, NY=1024, Isat=np.inf,
                 nl_length=0, wvl=780e-9, cpu_kernels=False):
        # parameters and default step (nlse.py:93-114)
        self.cpu_kernels = cpu_kernels
        self.n2, self.V, self.wl = n2, V, wvl
        self.k = 2 * np.pi / self.wl
        self.L, self.alpha, self.power, self.I_sat = L, alpha, power, Isat
        self.NX, self.NY = NX, NY
        self.window = [window, window] if isinstance(window, (int, float)) else list(window)
        z_nl = 1 / (self.k * abs(self.n2 * self.power / min(self.window) ** 2))
        if isinstance(z_nl, np.ndarray):
            z_nl = float(z_nl.min())
        self.delta_z = 5e-3 * z_nl
        # float32 grid with float64 step, frequencies 2*pi*fftfreq (nlse.py:116-141)
        self.X, self.delta_X = np.linspace(-self.window[0] / 2, self.window[0] / 2, NX,
                                           endpoint=False, retstep=True, dtype=np.float32)
        self.Y, self.delta_Y = np.linspace(-self.window[1] / 2, self.window[1] / 2, NY,
                                           endpoint=False, retstep=True, dtype=np.float32)
        self.last_axes = (-2, -1)
        self.XX, self.YY = np.meshgrid(self.X, self.Y)
        self.Kx = 2 * np.pi * np.fft.fftfreq(NX, d=self.delta_X)
        self.Ky = 2 * np.pi * np.fft.fftfreq(NY, d=self.delta_Y)
        self.Kxx, self.Kyy = np.meshgrid(self.Kx, self.Ky)
        self.propagator = None
        self.nl_length = nl_length
        self.nl_profile = (k0_profile(nl_length, self.delta_X) if nl_length > 0
                           else np.ones((NY, NX), dtype=np.float32))

    # -- pieces ---------------------------------------------------------------
    def build_propagator(self):
        """nlse.py:188-197."""
        return np.exp(-1j * 0.5 * (self.Kxx**2 + self.Kyy**2) / self.k * self.delta_z
                      ).astype(np.complex64)

    def norm_integral(self, E):
        """Sum |E|^2 dX dY (c eps0 / 2) over the transform axes (nlse.py:293-301)."""
        s = ((E.real * E.real + E.imag * E.imag) * self.delta_X * self.delta_Y
             ).sum(axis=self.last_axes)
        return s * c * epsilon_0 / 2

    def prepare(self, E_in, normalize):
        """nlse.py:257-307."""
        A = np.zeros_like(E_in)
        if normalize:
            E_00 = (self.power / self.norm_integral(E_in)) ** 0.5
            A[:] = (E_00.T * E_in.T).T
        else:
            A[:] = E_in
        return A

    def fft(self, A):
        A[:] = sfft.fftn(A, axes=self.last_axes, workers=WORKERS)

    def ifft(self, A):
        A[:] = sfft.ifftn(A, axes=self.last_axes, workers=WORKERS)

    def convolve(self, A_sq):
        """Nonlocal response, linear 'same' convolution (nlse.py:406-408, 444-447)."""
        return signal.oaconvolve(A_sq, self.nl_profile, mode="same", axes=self.last_axes)

    def nonlinear(self, A, V, dz):
        """Squared modulus, optional convolution, nl_prop (nlse.py:443-487)."""
        A_sq = square_mod(A).astype(A.real.dtype)
        if self.nl_length > 0:
            A_sq[:] = self.convolve(A_sq)
        nl_prop(A, A_sq, dz, self.alpha / 2, None if V is None else self.k / 2 * V,
                self.k / 2 * self.n2 * c * epsilon_0, 2 * self.I_sat / (epsilon_0 * c),
                cpu_kernels=self.cpu_kernels)

    def split_step(self, A, V, propagator, precision="single"):
        """Lie ("single") or Strang ("double") step (nlse.py:372-487)."""
        if precision == "double":
            self.nonlinear(A, V, self.delta_z / 2)
        self.fft(A)
        A *= propagator
        self.ifft(A)
        self.nonlinear(A, V, self.delta_z / 2 if precision == "double" else self.delta_z)

    def out_field(self, E_in, z, precision="single", normalize=True,
                  callback: Callable | list | None = None, callback_args=()):
        """z-loop with callbacks (nlse.py:489-619); returns (A, number of steps)."""
        assert E_in.shape[self.last_axes[0]:] == self.XX.shape[self.last_axes[0]:]
        assert E_in.dtype in (np.complex64, np.complex128)
        if self.propagator is None:
            self.propagator = self.build_propagator()
        V = None if self.V is None else np.array(self.V, copy=True)
        A = self.prepare(E_in, normalize)
        n2_old = self.n2
        z_prop, i = 0, 0
        while abs(z_prop) < z:
            if z > self.L:
                self.n2 = 0
            self.split_step(A, V, self.propagator, precision)
            if callback is not None:
                if callable(callback):
                    callback(self, A, z, i, *callback_args)
                else:
                    for cb, ca in zip(callback, callback_args):
                        cb(self, A, z, i, *ca)
            z_prop += self.delta_z
            i += 1
        self.n2 = n2_old
        return A, i


def k0_profile(nl_length, delta_X):
    """Normalised K0 Bessel kernel of size (6d+1)^2, d = nl_length // dX (nlse.py:143-153)."""
    d = nl_length // delta_X
    r = np.arange(-3 * d, 3 * d + 1)
    xx, yy = np.meshgrid(r, r)
    prof = special.kn(0, np.hypot(xx, yy) / d)
    prof[prof.shape[0] // 2, prof.shape[1] // 2] = np.nanmax(prof[~np.isinf(prof)])
    return prof / prof.sum()


class OracleNLSE_1d(OracleNLSE):
    """Restatement of NLSE_1d (NLSE/nlse_1d.py:15-105)."""

    def __init__(self, alpha, power, window, n2, V, L, NX=1024, Isat=np.inf, nl_length=0,
                 wvl=780e-9, cpu_kernels=False):
        super().__init__(alpha, power, window, n2, V, L, NX=NX, NY=1024, Isat=Isat,
                         nl_length=nl_length, wvl=wvl, cpu_kernels=cpu_kernels)
        self.last_axes = (-1,)
        self.nl_profile = self.nl_profile[0]
        self.nl_profile = self.nl_profile / self.nl_profile.sum()

    def build_propagator(self):
        """Not cast to complex64 (nlse_1d.py:98-105)."""
        return np.exp(-1j * 0.5 * (self.Kx**2) / self.k * self.delta_z)

    def norm_integral(self, E):
        """Uses delta_X**2 (nlse_1d.py:86-91)."""
        s = ((E.real * E.real + E.imag * E.imag) * self.delta_X**2).sum(axis=self.last_axes)
        return s * (c * epsilon_0 / 2)


class OracleNLSE_3d(OracleNLSE):
    """Restatement of NLSE_3d (NLSE/nlse_3d.py:15-150)."""

    def __init__(self, alpha, energy, window, n2, D0, vg, V, L, NX=1024, NY=1024, NZ=1024,
                 Isat=np.inf, nl_length=0, wvl=780e-9, cpu_kernels=False):
        if len(window) == 2:
            window = [window[0], window[0], window[-1]]
        super().__init__(alpha, energy, window[0:2], n2, V, L, NX=NX, NY=NY, Isat=Isat,
                         nl_length=nl_length, wvl=wvl, cpu_kernels=cpu_kernels)
        self.energy = self.power
        self.NZ = NZ
        self.window_t = window[-1]
        self.power = self.energy / self.window_t
        z_nl = 1 / (self.k * abs(self.n2 * self.power / min(self.window[0:2]) ** 2))
        if isinstance(z_nl, np.ndarray):
            z_nl = z_nl.min()
        self.delta_z = 0.5e-2 * z_nl
        self.T, self.delta_T = np.linspace(-self.window_t / 2, self.window_t / 2, NZ,
                                           retstep=True)
        self.omega = 2 * np.pi * np.fft.fftfreq(NZ, self.delta_T)
        self.D0, self.vg = D0, vg
        self.XX, self.YY, self.TT = np.meshgrid(self.X, self.Y, self.T)
        self.Kxx, self.Kyy, self.Omega = np.meshgrid(self.Kx, self.Ky, self.omega)
        self.last_axes = (-3, -2, -1)

    def build_propagator(self):
        """2-D propagator (complex64) times the GVD factor, no dz on it (nlse_3d.py:105-114)."""
        prop_2d = super().build_propagator()
        return prop_2d * np.exp(-1j * self.D0 / 2 * self.Omega**2)

    def norm_integral(self, E):
        """nlse_3d.py:137-147."""
        s = ((E.real * E.real + E.imag * E.imag) * self.delta_X * self.delta_Y * self.delta_T
             ).sum(axis=self.last_axes)
        return s * (c * epsilon_0 / 2)

    def prepare(self, E_in, normalize):
        A = np.zeros_like(E_in)
        if normalize:
            E_00 = (self.energy / self.norm_integral(E_in)) ** 0.5
            A[:] = (E_00.T * E_in.T).T
        else:
            A[:] = E_in
        return A


class OracleGPE(OracleNLSE):
    """Restatement of GPE (NLSE/gpe.py:15-119)."""

    def __init__(self, gamma, N, window, g, V, m=87 * atomic_mass, NX=1024, NY=1024,
                 sat=np.inf, nl_length=0, cpu_kernels=False):
        super().__init__(gamma, N, window, g, V, 0, NX=NX, NY=NY, Isat=sat,
                         nl_length=nl_length, wvl=2 * np.pi / m, cpu_kernels=cpu_kernels)
        self.g, self.gamma, self.N, self.m, self.sat = g, self.alpha, self.power, self.k, sat
        self.delta_t = self.delta_z
        self.I_sat *= epsilon_0 * c / 2

    def build_propagator(self):
        """Uses delta_t, not delta_z (gpe.py:81-90)."""
        return np.exp(-1j * 0.5 * hbar * (self.Kxx**2 + self.Kyy**2) / self.m * self.delta_t
                      ).astype(np.complex64)

    def prepare(self, E_in, normalize):
        """Normalised to the atom number without c eps0 / 2 (gpe.py:92-119)."""
        A = np.array(E_in, copy=True)
        if normalize:
            s = ((E_in.real * E_in.real + E_in.imag * E_in.imag) * self.delta_X * self.delta_Y
                 ).sum(axis=self.last_axes)
            E_00 = (self.N / s) ** 0.5
            A[:] = (E_00.T * E_in.T).T
        return A


class OracleCNLSE(OracleNLSE):
    """Restatement of CNLSE (NLSE/cnlse.py:19-423)."""

    comps = 2

    def __init__(self, alpha, power, window, n2, n12, V, L, NX=1024, NY=1024, Isat=np.inf,
                 nl_length=0, wvl=780e-9, omega=None, cpu_kernels=False):
        super().__init__(alpha, power, window, n2, V, L, NX=NX, NY=NY, Isat=Isat,
                         nl_length=nl_length, wvl=wvl, cpu_kernels=cpu_kernels)
        self.I_sat2 = self.I_sat
        self.n12 = n12
        self.n22 = self.n2
        self.omega = omega
        self.alpha2 = self.alpha
        self.k2 = self.k
        self.power2 = self.power

    def build_propagator(self):
        """cnlse.py:179-190."""
        p1 = super().build_propagator()
        p2 = np.exp(-1j * 0.5 * (self.Kxx**2 + self.Kyy**2) / self.k2 * self.delta_z
                    ).astype(np.complex64)
        return np.array([p1, p2])

    def take(self, A):
        """cnlse.py:192-202."""
        return A[..., 0, :, :], A[..., 1, :, :]

    def prepare(self, E, normalize):
        """Per-component power normalisation (cnlse.py:99-148), batch-safe."""
        A = np.zeros_like(E)
        if normalize:
            integral = ((E.real * E.real + E.imag * E.imag) * self.delta_X * self.delta_Y
                        ).sum(axis=self.last_axes) * c * epsilon_0 / 2
            E_00 = (np.array([self.power, self.power2], dtype=E.dtype) / integral) ** 0.5
            A[:] = E_00[..., None, None] * E if self.last_axes == (-2, -1) else (
                E_00[..., None] * E)
        else:
            A[:] = E
        return A

    def nl_pair(self, A, V, dz, post):
        """Both components' nonlinear steps from the same |A|^2 (cnlse.py:288-421)."""
        A1, A2 = self.take(A)
        A_sq = square_mod(A).astype(A.real.dtype)
        s1, s2 = self.take(A_sq)
        if self.nl_length > 0:
            s1 = self.convolve(s1)
            s2 = self.convolve(s2)
        k, k2 = self.k, self.k2
        is1, is2 = 2 * self.I_sat / (epsilon_0 * c), 2 * self.I_sat2 / (epsilon_0 * c)
        nl_prop_c(A1, s1, s2, dz, self.alpha / 2, None if V is None else k / 2 * V,
                  k / 2 * self.n2 * c * epsilon_0, k / 2 * self.n12 * c * epsilon_0, is1, is2)
        nl_prop_c(A2, s2, s1, dz, self.alpha2 / 2, None if V is None else k2 / 2 * V,
                  k2 / 2 * self.n22 * c * epsilon_0, k2 / 2 * self.n12 * c * epsilon_0, is2, is1)

    def split_step(self, A, V, propagator, precision="single"):
        if precision == "double":
            self.nl_pair(A, V, self.delta_z / 2, False)
        self.fft(A)
        A *= propagator
        self.ifft(A)
        if precision == "double":
            self.nl_pair(A, V, self.delta_z / 2, True)
        else:
            self.nl_pair(A, V, self.delta_z, True)
            if self.omega is not None:
                A1, A2 = self.take(A)
                rabi_coupling(A1, A2, self.delta_z, self.omega / 2)


class OracleCNLSE_1d(OracleCNLSE):
    """Restatement of CNLSE_1d (NLSE/cnlse_1d.py:13-146)."""

    def __init__(self, alpha, power, window, n2, n12, V, L, NX=1024, Isat=np.inf, nl_length=0,
                 wvl=780e-9, omega=None, cpu_kernels=False):
        super().__init__(alpha, power, window, n2, n12, V, L, NX=NX, Isat=Isat,
                         nl_length=nl_length, wvl=wvl, omega=omega, cpu_kernels=cpu_kernels)
        self.last_axes = (-1,)
        # first row of the 2-D profile, renormalised (cnlse_1d.py:80-81)
        self.nl_profile = self.nl_profile[0]
        self.nl_profile = self.nl_profile / self.nl_profile.sum()

    def take(self, A):
        return A[..., 0, :], A[..., 1, :]

    def build_propagator(self):
        p1 = np.exp(-1j * 0.5 * (self.Kx**2) / self.k * self.delta_z)
        p2 = np.exp(-1j * 0.5 * (self.Kx**2) / self.k2 * self.delta_z)
        return np.array([p1, p2])

    def prepare(self, E, normalize):
        A = np.zeros_like(E)
        if normalize:
            integral = ((E.real * E.real + E.imag * E.imag) * self.delta_X**2
                        ).sum(axis=self.last_axes)
            integral *= c * epsilon_0 / 2
            E_00 = (np.array([self.power, self.power2], dtype=E.dtype) / integral) ** 0.5
            A[:] = E_00[..., None] * E
        else:
            A[:] = E
        return A


class OracleDDGPE(OracleCNLSE):
    """Restatement of DDGPE (NLSE/ddgpe.py:14-565), including its per-branch quirks."""

    def __init__(self, gamma, power, window, g, omega, T, omega_exc, omega_cav, detuning, k_z,
                 V=None, g12=0, NX=1024, NY=1024, Isat=np.inf, nl_length=0):
        super().__init__(gamma, power, window, -g, g12, V, T, NX=NX, NY=NY, Isat=Isat,
                         nl_length=nl_length, wvl=1e-30, omega=omega)
        self.g, self.g12, self.g2 = self.n2, self.n12, 0
        self.k_z, self.gamma, self.gamma2 = k_z, gamma, gamma
        self.omega_exc, self.omega_cav, self.detuning = omega_exc, omega_cav, detuning
        omega_lp = (omega_exc + omega_cav) / 2 - 0.5 * np.sqrt((omega_exc - omega_cav) ** 2
                                                               + omega**2)
        self.omega_pump = omega_lp + detuning

    def build_propagator(self):
        """ddgpe.py:204-224."""
        p1 = np.exp(-1j * (self.omega_exc * (1 + 0 * self.Kxx**2) - self.omega_pump)
                    * self.delta_z).astype(np.complex64)
        p2 = np.exp(-1j * (self.omega_cav * np.sqrt(1 + (self.Kxx**2 + self.Kyy**2)
                                                    / self.k_z**2) - self.omega_pump)
                    * self.delta_z).astype(np.complex64)
        return np.array([p1, p2])

    def prepare(self, E, normalize):
        """No normalisation (ddgpe.py:226-245)."""
        return np.array(E, copy=True)

    @staticmethod
    def laser_excitation(simu, A, t, i, F_pump_r, F_pump_t, F_probe_r, F_probe_t):
        """ddgpe.py:127-156."""
        A[..., 1, :, :] -= F_pump_r * F_pump_t[i] * simu.delta_z * 1j
        A[..., 1, :, :] -= F_probe_r * F_probe_t[i] * simu.delta_z * 1j

    def _pair(self, A1, A2, s1, s2, dz, V, a1, a2, v1, v2, g1, g2):
        nl_prop_c(A1, s1, s2, dz, a1, v1, g1, self.g12, self.I_sat, self.I_sat2)
        nl_prop_c(A2, s2, s1, dz, a2, v2, g2, self.g12, self.I_sat, self.I_sat2)

    def split_step(self, A, V, propagator, precision="single"):
        """The branch-specific arguments of ddgpe.py:247-457, verbatim in effect."""
        A1, A2 = self.take(A)
        dz = self.delta_z

        def sq():
            s = square_mod(A).astype(A.real.dtype)
            s1, s2 = self.take(s)
            if self.nl_length > 0:
                s1, s2 = self.convolve(s1), self.convolve(s2)
            return s1, s2

        if precision == "double":
            s1, s2 = sq()
            if V is None:  # ddgpe.py:300-321
                self._pair(A1, A2, s1, s2, dz / 2, None, self.gamma / 2, self.gamma2 / 2, None,
                           None, self.g, self.g)
            else:  # ddgpe.py:323-346
                self._pair(A1, A2, s1, s2, dz, None, self.gamma / 2, self.gamma2 / 2, V, V,
                           self.g, self.g2)
        self.fft(A)
        A *= propagator
        self.ifft(A)
        s1, s2 = sq()
        if precision == "double":
            if V is None:  # ddgpe.py:366-387
                self._pair(A1, A2, s1, s2, dz / 2, None, self.gamma / 2, self.gamma2 / 2, None,
                           None, self.g, self.g)
            else:  # ddgpe.py:389-411
                self._pair(A1, A2, s1, s2, dz, None, self.gamma / 2, self.gamma2 / 2,
                           self.k / 2 * V, V, self.g, self.g2)
        else:
            if V is None:  # ddgpe.py:413-434
                self._pair(A1, A2, s1, s2, dz, None, self.alpha / 2, self.gamma2 / 2, None,
                           None, self.g, self.g2)
            else:  # ddgpe.py:436-455
                self._pair(A1, A2, s1, s2, dz, None, self.gamma / 2, self.gamma2 / 2, V, V,
                           self.g, self.g2)
            if self.omega is not None:
                rabi_coupling(A1, A2, dz, self.omega / 2)

    def out_field(self, E_in, t, laser_excitation, precision="single", callback=None,
                  callback_args=None):
        """Pump inserted as callback 0, no normalisation (ddgpe.py:519-565)."""
        callback = list(callback) if callback else []
        callback_args = list(callback_args) if callback_args else []
        callback.insert(0, laser_excitation if laser_excitation is not None
                        else self.laser_excitation)
        return super().out_field(E_in, t, precision=precision, normalize=False,
                                 callback=callback, callback_args=callback_args)


# ---- counter-based noise (test oracle of nlse_add_noise) ----------------------
def philox4x32_10(c, k0, k1):
    """Philox4x32-10 (Salmon et al., SC 2011) on arrays of 4 uint32 counters
    c = (c0, c1, c2, c3) with key (k0, k1); returns the four output words."""
    M0, M1, W0, W1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57), 0x9E3779B9, 0xBB67AE85
    c0, c1, c2, c3 = (np.asarray(x, np.uint64) for x in c)
    k0, k1 = int(k0), int(k1)
    mask = np.uint64(0xFFFFFFFF)
    for _ in range(10):
        p0, p1 = M0 * c0, M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & mask
        hi1, lo1 = p1 >> np.uint64(32), p1 & mask
        c0, c1, c2, c3 = (hi1 ^ c1 ^ np.uint64(k0)), lo1, (hi0 ^ c3 ^ np.uint64(k1)), lo0
        k0, k1 = (k0 + W0) & 0xFFFFFFFF, (k1 + W1) & 0xFFFFFFFF
    return c0, c1, c2, c3


def ddgpe_noise(pix: int, seed: int, step: int):
    """Standard complex normals (component 0, component 1) per pixel for one step."""
    p = np.arange(pix, dtype=np.uint64)
    r = philox4x32_10((p & np.uint64(0xFFFFFFFF), np.full(pix, step, np.uint64),
                       p >> np.uint64(32), np.zeros(pix, np.uint64)),
                      seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    u = [(x.astype(np.float64) + 0.5) * 2.0**-32 for x in r]
    ra, rb = np.sqrt(-2 * np.log(u[0])), np.sqrt(-2 * np.log(u[2]))
    return (ra * np.cos(2 * np.pi * u[1]) + 1j * ra * np.sin(2 * np.pi * u[1]),
            rb * np.cos(2 * np.pi * u[3]) + 1j * rb * np.sin(2 * np.pi * u[3]))


# ---------------------------------------------------------------------------
# callbacks' nonlinear index change (NLSE/callbacks.py:57-112)
# ---------------------------------------------------------------------------
def delta_n(A, n2, I_sat):
    """evaluate_delta_n's record (NLSE/callbacks.py:79-82): NumPy evaluation of
    c*eps0/2*n2*|A|^2 / (1 + |A|^2/I_sat) with |A|^2 = re*re + im*im, every
    operation rounded on its own, Python-float parameters weak (field
    precision), float64 arrays and NumPy scalars strong."""
    a_sq = A.real * A.real + A.imag * A.imag
    return c * epsilon_0 / 2 * n2 * a_sq / (1 + a_sq / I_sat)


def adapt_peak(A, n2, I_sat):
    """Peak of adapt_delta_z's index change (NLSE/callbacks.py:108-110); the
    factor c*eps0/2 multiplies only the imaginary square there (operator
    precedence), and np.abs of a Python float is a float64 NumPy scalar."""
    a_sq = A.real * A.real + A.imag * A.imag * c * epsilon_0 / 2
    return (np.abs(n2) * a_sq / (1 + a_sq / I_sat)).max()


def adapt_delta_z(A, n2, I_sat, k):
    """The step adapt_delta_z sets (NLSE/callbacks.py:110-112)."""
    with np.errstate(divide="ignore"):
        z_nl = float(1 / (k * adapt_peak(A, n2, I_sat)))
    return np.abs(z_nl) / 12
