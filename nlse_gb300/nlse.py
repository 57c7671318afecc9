"""NLSE solver class: the drop-in for the reference's NLSE with backend="GPU".

Mirrors Quantum-Optics-LKB/NLSE v2.3.0, NLSE/nlse.py:41-681: same
constructor, attributes, helper methods and out_field semantics.  Device
arrays are torch CUDA tensors; the FFT, the propagator multiply and the
nonlinear operator run in libnlse_sm103 (no CuPy, VkFFT or cuFFT).
"""

from __future__ import annotations

import time
import warnings
from typing import Any, Callable, Union

import numpy as np
import torch
from scipy import special
from scipy.constants import c, epsilon_0

from . import _lib, autotune, callbacks, engine
from .engine import OperatorData, Plan

__BACKEND__ = "GPU"


def _gpu_available() -> bool:
    return torch.cuda.is_available()


def _is_device_array(x) -> bool:
    return isinstance(x, torch.Tensor) and x.is_cuda


def _host(x):
    """Host (NumPy) view of a parameter that may live on the device."""
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return x


def nonlinear_length(k: float, n2, power, w2: float):
    """1 / (k |n2 * power / w2|), minimised over the broadcast of n2 and power
    when either is an array (the default step of nlse.py:108-114 and
    nlse_3d.py:105-111), without forming that broadcast: a per-field n2
    (B, 1, 1) and power (B,) would make a (B, 1, B) array.  Every factor
    enters through its absolute value and rounding is monotone, so the
    minimum is the same expression evaluated at the largest |n2 * power|,
    which each operand reaches after a reduction over the axes the other one
    broadcasts along: the value is bit for bit the minimum of the array."""
    if not (isinstance(n2, np.ndarray) or isinstance(power, np.ndarray)):
        return 1 / (k * abs(n2 * power / w2))
    # NumPy's absolute value keeps each operand's type, and a Python scalar
    # stays a Python scalar (weak in NumPy's promotion, as in the product)
    a = np.abs(n2) if isinstance(n2, (np.ndarray, np.generic)) else abs(n2)
    b = np.abs(power) if isinstance(power, (np.ndarray, np.generic)) else abs(power)
    if isinstance(a, np.ndarray) and isinstance(b, np.ndarray):
        nd = max(a.ndim, b.ndim)
        a = a.reshape((1,) * (nd - a.ndim) + a.shape)
        b = b.reshape((1,) * (nd - b.ndim) + b.shape)
        np.broadcast_shapes(a.shape, b.shape)  # incompatible shapes raise as the product would
        for ax in range(nd):
            if a.shape[ax] == 1 and b.shape[ax] > 1:
                b = b.max(axis=ax, keepdims=True)
            elif b.shape[ax] == 1 and a.shape[ax] > 1:
                a = a.max(axis=ax, keepdims=True)
    return (1 / (k * ((a * b) / w2))).min()


def count_steps(z: float, delta_z) -> int:
    """Number of iterations of `while abs(z_prop) < z: z_prop += delta_z`.

    Reproduces the float accumulation of the reference z-loop
    (NLSE/nlse.py:568-585) exactly, so the step count matches it.
    """
    z_prop = 0
    n = 0
    if delta_z == 0:
        if abs(z_prop) < z:
            raise ValueError("delta_z = 0 with z > 0 never terminates")
        return 0
    while abs(z_prop) < z:
        z_prop += delta_z
        n += 1
    return n


_PIPE_STREAMS: dict = {}


def _pipeline_streams(dev: torch.device) -> tuple:
    """The upload and download streams of the host pipeline on one device."""
    key = str(dev)
    if key not in _PIPE_STREAMS:
        _PIPE_STREAMS[key] = (torch.cuda.Stream(dev), torch.cuda.Stream(dev))
    return _PIPE_STREAMS[key]


def pipeline_split(nf: int, nbytes: int, nsteps: int, max_steps: int, min_bytes: int):
    """Field bounds of the host pipeline's chunks for a batch of nf fields of
    nbytes in all, propagated over nsteps steps, or None (not pipelined): the
    first and the last field alone, the others together."""
    if nf < 2 or nbytes < min_bytes or nsteps > max_steps:
        return None
    return [0, 1, nf] if nf < 4 else [0, 1, nf - 1, nf]


class NLSE:
    """A class to solve NLSE"""

    __CUPY_AVAILABLE__ = _gpu_available()  # name kept from the reference: "GPU backend usable"
    __GPU_AVAILABLE__ = __CUPY_AVAILABLE__
    __PYOPENCL_AVAILABLE__ = False

    _comps = 1  # field components stacked before the transform axes

    def __init__(
        self,
        alpha: float,
        power: float,
        window: Union[float, tuple, list],
        n2: float,
        V: Union[np.ndarray, None],
        L: float,
        NX: int = 1024,
        NY: int = 1024,
        Isat: float = np.inf,
        nl_length: float = 0,
        wvl: float = 780e-9,
        backend: str = __BACKEND__,
    ) -> None:
        """Instantiate the simulation (NLSE/nlse.py:47-155).

        Solves d/dz psi = -1/2k0 (d2/dx2 + d2/dy2) psi + k0 dn psi + k0 n2 |psi|^2 psi.

        Args:
            alpha: linear loss (1/m); power: power in W; window: transverse window
            in m (float or (wx, wy)); n2: nonlinear index (m^2/W); V: potential or
            None; L: medium length (m); NX, NY: grid points; Isat: saturation
            intensity (W/m^2); nl_length: nonlocal length (m); wvl: wavelength (m);
            backend: "GPU" (the only backend of this engine).
        """
        self.backend = backend
        self.n2 = n2
        self.V = V
        self.wl = wvl
        self.k = 2 * np.pi / self.wl
        self.L = L
        self.alpha = alpha
        self.power = power
        self.I_sat = Isat
        self.NX = NX
        self.NY = NY
        if isinstance(window, (float, int)):
            self.window = [window, window]
        elif isinstance(window, (tuple, list)):
            self.window = window
        else:
            self.window = list(window)
        # default step: 1/200 of the nonlinear length (nlse.py:108-114)
        z_nl = nonlinear_length(self.k, self.n2, self.power, min(self.window) ** 2)
        if isinstance(self.n2, np.ndarray) or isinstance(self.power, np.ndarray):
            if np.broadcast_shapes(np.shape(self.n2), np.shape(self.power)) != ():
                z_nl = float(z_nl)  # the minimum of an array, as a Python float
        self.delta_z = 5e-3 * z_nl
        # float32 transverse grid, float64 step (nlse.py:116-131)
        self.X, self.delta_X = np.linspace(
            -self.window[0] / 2, self.window[0] / 2, num=NX, endpoint=False, retstep=True,
            dtype=np.float32)
        self.Y, self.delta_Y = np.linspace(
            -self.window[1] / 2, self.window[1] / 2, num=NY, endpoint=False, retstep=True,
            dtype=np.float32)
        self._last_axes = (-2, -1)
        self.XX, self.YY = np.meshgrid(self.X, self.Y)
        self.Kx = 2 * np.pi * np.fft.fftfreq(self.NX, d=self.delta_X)
        self.Ky = 2 * np.pi * np.fft.fftfreq(self.NY, d=self.delta_Y)
        self.Kxx, self.Kyy = np.meshgrid(self.Kx, self.Ky)
        self.propagator = None
        self.plans = None
        self.nl_length = nl_length
        if self.nl_length > 0:
            self.nl_profile = self._k0_profile(self.nl_length, self.delta_X)
        else:
            self.nl_profile = np.ones((self.NY, self.NX), dtype=np.float32)

    @staticmethod
    def _k0_profile(nl_length: float, delta_X: float) -> np.ndarray:
        """Normalised K0 Bessel nonlocal kernel of size (6d+1)^2 (nlse.py:143-153).

        With nl_length < delta_X, d = 0 and the kernel is NaN, as in the
        reference (every field it enters becomes NaN); a RuntimeWarning says
        so at construction instead of leaving it to the results."""
        d = nl_length // delta_X
        if d == 0:
            warnings.warn(f"nl_length = {nl_length:g} m is below the grid step {delta_X:g} m: "
                          "the K0 nonlocal kernel is NaN (as in the reference); use nl_length "
                          ">= the grid step or set nl_profile", RuntimeWarning, stacklevel=3)
        r = np.arange(-3 * d, 3 * d + 1)
        xx, yy = np.meshgrid(r, r)
        prof = special.kn(0, np.hypot(xx, yy) / d)
        finite = prof[np.logical_not(np.isinf(prof))]
        prof[prof.shape[0] // 2, prof.shape[1] // 2] = np.nanmax(finite) if finite.size else np.nan
        prof /= prof.sum()
        return prof

    # -- backend ------------------------------------------------------------
    @property
    def backend(self) -> str:
        return self.__backend

    @backend.setter
    def backend(self, value: str) -> None:
        """Select the backend (nlse.py:162-186).  This engine is the GPU backend."""
        if value not in ["CPU", "GPU", "CL"]:
            raise ValueError("Backend must be 'CPU', 'GPU' or 'CL'")
        if value != "GPU":
            raise ValueError(
                f"backend {value!r} is not provided: this engine is the GPU backend only")
        self.__backend = "GPU"

    @property
    def _device(self) -> torch.device:
        return torch.device("cuda", torch.cuda.current_device())

    # -- construction helpers (overridden by the subclasses) ------------------
    def _build_propagator(self) -> np.ndarray:
        """exp(-i (Kx^2+Ky^2)/(2k) dz) in FP64, cast to complex64 (nlse.py:188-197)."""
        return np.exp(
            -1j * 0.5 * (self.Kxx**2 + self.Kyy**2) / self.k * self.delta_z
        ).astype(np.complex64)

    def _build_fft_plan(self, A) -> list:
        """One plan for both directions, as the reference's GPU path (nlse.py:199-218)."""
        lead = self._lead_shape(tuple(A.shape))
        n_axes = len(self._last_axes)
        shape = tuple(A.shape[-n_axes:])
        dtype = engine.dtype_code(A) if isinstance(A, torch.Tensor) else (
            0 if np.dtype(A.dtype) == np.complex64 else 1)
        nf = int(np.prod(lead)) if lead else 1
        return [Plan.get(n_axes, shape, nf, self._comps, dtype, self._device)]

    def _lead_shape(self, shape: tuple) -> tuple:
        """Leading (batch) dimensions of a field shape."""
        k = len(self._last_axes) + (1 if self._comps == 2 else 0)
        return tuple(shape[: len(shape) - k])

    def _norm_coef(self) -> float:
        """Integration weight of sum(|E|^2) in the power normalisation (nlse.py:293-301)."""
        return self.delta_X * self.delta_Y * c * epsilon_0 / 2

    def _norm_target(self, lead: tuple) -> np.ndarray:
        """Per-segment target of the normalisation (the power)."""
        return engine.per_field(self.power, lead, 0, "power")

    def _prepare_output_array(self, E_in, normalize: bool) -> tuple:
        """Device copy of E_in, normalised to the power, and the |A|^2 twin (nlse.py:257-307)."""
        dev = self._device
        src = engine.to_device(E_in, dev)
        A = torch.empty_like(src)
        # split_step's |A|^2 argument: the fused kernels form |A|^2 in registers and
        # never read it, so it is not zero-filled
        A_sq = torch.empty(A.shape, dtype=A.real.dtype, device=dev)
        if normalize:
            lead = self._lead_shape(tuple(A.shape))
            nseg = int(np.prod(lead)) * self._comps if lead else self._comps
            sums = engine.power(src, nseg)
            target = torch.from_numpy(np.array(self._norm_target(lead), dtype=np.float64)
                                      .reshape(-1)).to(dev)
            engine.normalize(src, A, nseg, sums, target, self._norm_coef())
        else:
            A.copy_(src)
        return A, A_sq

    _DEVICE_ATTRS = ("power", "n2", "alpha", "I_sat")

    def _send_arrays_to_gpu(self) -> None:
        """Move the potential, propagator and array parameters to the device (nlse.py:309-342).

        Records which of them were host arrays: only those go back to the host
        afterwards (device tensors a caller supplied stay where they are)."""
        dev = self._device
        host = {}
        for name in ("V", "nl_profile", "propagator"):
            v = getattr(self, name, None)
            if v is not None:
                t = engine.to_device(v, dev)
                if not _is_device_array(v):
                    host[name] = (v, t, t._version)
                setattr(self, name, t)
        for name in self._DEVICE_ATTRS:
            v = getattr(self, name, None)
            if isinstance(v, np.ndarray):
                t = engine.to_device(v, dev)
                host[name] = (v, t, t._version)
                setattr(self, name, t)
        self._host_attrs = host

    def _retrieve_arrays_from_gpu(self) -> None:
        """Bring the arrays that were host arrays back to NumPy (nlse.py:344-370).

        A device copy that nothing changed in place (its torch version counter
        is the one it had when sent) gives back the caller's own host array,
        which holds the same values, without a copy; a changed one is copied."""
        for name, (orig, t, ver) in getattr(self, "_host_attrs", {}).items():
            v = getattr(self, name, None)
            if v is t and t._version == ver:
                setattr(self, name, orig)
            elif _is_device_array(v):
                setattr(self, name, engine.to_host(v).numpy())
        self._host_attrs = {}

    # -- the split-step operator --------------------------------------------
    def _nl_block(self, lead: tuple, precision: str, has_v: bool) -> np.ndarray:
        """Per-field parameters of the nonlinear steps (nlse.py:404-487).

        Row layout: see include/nlse_gb300.h (NLSE_PARAM_STRIDE).
        """
        nf = int(np.prod(lead)) if lead else 1
        na = len(self._last_axes)
        P = np.zeros((nf, _lib.NLSE_PARAM_STRIDE), dtype=np.float64)
        dz = self.delta_z
        # a coefficient that varies over the grid goes to a plane (_coef_planes);
        # its per-field slot is then not read
        cg, ca, ci = self._nl_coefs()
        g = 0.0 if engine.varies_on_grid(cg, na) else engine.per_field(cg, lead, na, "n2")
        alpha = 0.0 if engine.varies_on_grid(ca, na) else engine.per_field(ca, lead, na, "alpha")
        isat = np.inf if engine.varies_on_grid(ci, na) else engine.per_field(ci, lead, na, "Isat")
        vs = self.k / 2
        for s, dzs in ((0, dz / 2 if precision == "double" else dz), (1, dz / 2)):
            o = s * 16
            P[:, o + 0] = np.real(dzs)
            P[:, 32 + s] = np.imag(dzs)
            P[:, o + 1] = alpha
            P[:, o + 2] = g
            P[:, o + 3] = 0.0
            P[:, o + 4] = isat
            P[:, o + 5] = np.inf
            P[:, o + 6] = vs
        return P

    def _nl_coefs(self) -> tuple:
        """The nonlinear step's coefficients as the reference forms them for
        nl_prop (nlse.py:411-428): g = k/2 n2 c eps0, alpha/2, Isat' = 2 Isat/(eps0 c),
        scalars or arrays that broadcast against the field."""
        return (self.k / 2 * _host(self.n2) * c * epsilon_0, _host(self.alpha) / 2,
                2 * _host(self.I_sat) / (epsilon_0 * c))

    def _coef_planes(self, lead: tuple, grid: tuple, real_dtype, dev) -> tuple:
        """Planes [3][map fields][pixels] (g, alpha/2, 1/Isat') of the coefficients
        that vary over the grid -- the reference broadcasts n2, alpha and Isat
        arrays elementwise in nl_prop (nlse.py:309-328, kernels_gpu.py:4-65) --
        and the mask of the planes present; (None, 0) when none does."""
        na = len(self._last_axes)
        planes, mask = [None, None, None], 0
        for i, x in enumerate(self._nl_coefs()):
            if engine.varies_on_grid(x, na):
                if self._comps != 1:
                    raise NotImplementedError("coefficients varying over the grid are "
                                              "supported for one-component fields")
                p = engine.coef_plane(x, lead, grid)
                planes[i] = 1.0 / p if i == 2 else p
                mask |= 1 << i
        if not mask:
            return None, 0
        nmf = max(p.shape[0] for p in planes if p is not None)
        pix = int(np.prod(grid))
        out = np.zeros((3, nmf, pix), dtype=np.float64)
        for i, p in enumerate(planes):
            if p is not None:
                out[i] = np.broadcast_to(p, (nmf, pix))
        return torch.from_numpy(out).to(device=dev, dtype=real_dtype), mask

    def _prop_layout(self, prop: torch.Tensor) -> int:
        """Element stride between the components' propagators (0: shared)."""
        return 0

    def _operator(self, A: torch.Tensor, V, propagator, precision: str,
                  pump: tuple | None = None, plan: Plan | None = None) -> OperatorData:
        if precision not in ("single", "double"):
            raise ValueError("precision must be 'single' or 'double'")
        dev = A.device
        lead = self._lead_shape(tuple(A.shape))
        na = len(self._last_axes)
        prop = engine.to_device(propagator, dev)
        if prop.dtype not in (torch.complex64, torch.complex128):
            prop = prop.to(torch.complex128 if A.dtype == torch.complex128 else torch.complex64)
        Vd, vstride = None, 0
        if V is not None:
            Vd = engine.to_device(V, dev)
            if Vd.is_complex() and not bool(torch.any(Vd.imag != 0)):
                Vd = Vd.real.contiguous()
            if A.dtype == torch.complex64:
                Vd = Vd.to(torch.complex64 if Vd.is_complex() else torch.float32)
            pix_shape = tuple(A.shape[-na:])
            if tuple(Vd.shape[-na:]) != pix_shape:
                raise ValueError(f"V of shape {tuple(Vd.shape)} does not match the grid {pix_shape}")
            vlead = tuple(Vd.shape[:-na])
            if vlead and int(np.prod(vlead)) > 1:
                if vlead != lead:
                    Vd = Vd.expand(*lead, *pix_shape).contiguous()
                vstride = int(np.prod(pix_shape))
            Vd = Vd.contiguous()
        params = torch.from_numpy(self._nl_block(lead, precision, V is not None)).to(dev)
        khat = None
        plan = plan if plan is not None else self._build_fft_plan(A)[0]
        if self.nl_length > 0:
            # nonlocal response: the reference convolves |A|^2 with nl_profile
            # ("same" mode) before each nonlinear step (nlse.py:406-408, 444-447)
            if na == 3:
                raise NotImplementedError("nonlocal response of 3-D fields")
            pads, khat = engine.nonlocal_spectrum(self.nl_profile, tuple(A.shape[-na:]), A.dtype,
                                                  dev)
            plan.set_nonlocal(pads)
        else:
            plan.set_nonlocal(None)
        maps, mask = self._coef_planes(lead, tuple(A.shape[-na:]), A.real.dtype, dev)
        return OperatorData(prop=prop.contiguous(), params=params,
                            scheme=1 if precision == "double" else 0,
                            rabi=self._rabi_enabled(precision), V=Vd, v_fstride=vstride,
                            prop_cstride=self._prop_layout(prop), pump=pump, nl_khat=khat,
                            maps=maps, maps_mask=mask)

    def _rabi_enabled(self, precision: str) -> bool:
        return False

    def split_step(
        self,
        A: torch.Tensor,
        A_sq: torch.Tensor,
        V,
        propagator,
        plans: list,
        precision: str = "single",
    ) -> None:
        """One propagation step, in place on A (nlse.py:372-487).

        A_sq is accepted for signature compatibility; |A|^2 is formed inside
        the fused kernels and never stored.
        """
        op = self._operator(A, V, propagator, precision, plan=plans[0])
        engine.propagate(plans[0], A, op, 1, 0, graph=False)

    # -- pump hooks (DDGPE) ---------------------------------------------------
    def _split_fused_callbacks(self, callback, callback_args, A):
        """Separate callbacks the engine runs on the device from the host ones."""
        return None, callback, callback_args

    def out_field(
        self,
        E_in,
        z: float,
        plot: bool = False,
        precision: str = "single",
        verbose: bool = True,
        normalize: bool = True,
        callback: Union[list[Callable], Callable] = None,
        callback_args: Union[list[tuple], tuple] = (),
    ):
        """Propagate the field over a distance z (nlse.py:489-619).

        Without callbacks the whole z-loop is one nlse_propagate call replayed
        from a CUDA graph; with only the norm / sample callbacks the loop and
        their recordings are one graph (results copied out at the end); with
        other callbacks each step is one call followed by the callbacks on the
        live device field, as in the reference loop.
        Returns the field in proper units (V/m): a NumPy array for NumPy input,
        a torch tensor for torch input.
        """
        assert tuple(E_in.shape[self._last_axes[0]:]) == tuple(
            self.XX.shape[self._last_axes[0]:]), "Shape mismatch"
        in_dtype = E_in.dtype
        assert in_dtype in (np.complex64, np.complex128, torch.complex64, torch.complex128), (
            "Type mismatch, E_in should be complex64 or complex128")
        if callback is None:
            bounds = self._pipeline_bounds(E_in, count_steps(z, self.delta_z))
            if bounds is not None:
                return self._out_field_pipelined(E_in, z, precision, verbose, normalize, bounds)
        if self.propagator is None:
            self.propagator = self._build_propagator()
        self._send_arrays_to_gpu()
        V = None if self.V is None else self.V.clone()
        A, A_sq = self._prepare_output_array(E_in, normalize)
        self.plans = self._build_fft_plan(A)
        if plot:
            warnings.warn("plotting is not part of this engine; plot=True is ignored")
        n2_old = self.n2
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
        t0 = time.perf_counter()
        pump, callback, callback_args = self._split_fused_callbacks(callback, callback_args, A)
        try:
            if z > self.L:
                self.n2 = 0
            plen = None if pump is None else min(pump[1].numel(), pump[3].numel())
            recs = None if callback is None else callbacks.device_plan(
                self, callback, callback_args)
            if recs is not None:
                # device callbacks: nodes of one graph over the whole loop, or
                # graph segments between the updates of an adaptive step
                n = count_steps(z, self.delta_z)
                adaptive = any(k == "adapt" for k, _, _ in recs)
                if plen is not None and n > plen and not adaptive:
                    raise IndexError(f"the pump time profile has {plen} entries, the loop "
                                     f"runs {n} steps")
                done = n == 0
                if adaptive:
                    # the step count follows the adapted step: segments between updates
                    op = self._operator(A, V, self.propagator, precision, pump, self.plans[0])
                    autotune.maybe_tune(self.plans[0], A, op)
                    lead = self._lead_shape(tuple(A.shape))
                    has_v = V is not None

                    def refresh(op=op, lead=lead, has_v=has_v):
                        op.params.copy_(torch.from_numpy(self._nl_block(lead, precision, has_v)))

                    done = callbacks.run_adaptive(self, self.plans[0], A, op, z, recs, refresh,
                                                  plen)
                elif n > 0:
                    op = self._operator(A, V, self.propagator, precision, pump, self.plans[0])
                    autotune.maybe_tune(self.plans[0], A, op)
                    done = callbacks.run_in_graph(self, self.plans[0], A, op, n, recs)
                if done:
                    callback = None
            if callback is None and recs is not None:
                pass  # ran above
            elif callback is None:
                n = count_steps(z, self.delta_z)
                if plen is not None and n > plen:
                    raise IndexError(f"the pump time profile has {plen} entries, the loop "
                                     f"runs {n} steps")
                if n > 0:
                    op = self._operator(A, V, self.propagator, precision, pump, self.plans[0])
                    autotune.maybe_tune(self.plans[0], A, op)
                    engine.propagate(self.plans[0], A, op, n, 0, graph=True)
            else:
                z_prop = 0
                i = 0
                op = None
                key = None
                while abs(z_prop) < z:
                    if z > self.L:
                        self.n2 = 0
                    if plen is not None and i >= plen:
                        raise IndexError(f"pump time profile index {i} out of range ({plen})")
                    k = self._op_key()
                    if op is None or k != key:
                        op = self._operator(A, V, self.propagator, precision, pump,
                                            self.plans[0])
                        key = k
                    engine.propagate(self.plans[0], A, op, 1, i, graph=False)
                    if isinstance(callback, Callable):
                        callback(self, A, z, i, *callback_args)
                    elif isinstance(callback, list) and callback and isinstance(callback[0], Callable):
                        for cb, ca in zip(callback, callback_args):
                            cb(self, A, z, i, *ca)
                    else:
                        raise ValueError("callbacks should be a callable or a list of callables")
                    z_prop += self.delta_z
                    i += 1
        finally:
            self.n2 = n2_old
        end.record()
        if verbose:
            end.synchronize()
            print(f"\nTime spent to solve : {start.elapsed_time(end) * 1e-3} s (GPU) /"
                  f" {time.perf_counter() - t0} s (CPU)\n")
        self._retrieve_arrays_from_gpu()
        if isinstance(E_in, np.ndarray):
            return engine.to_host(A).numpy()
        if isinstance(E_in, torch.Tensor) and not E_in.is_cuda:
            return engine.to_host(A)
        return A

    # host batches of at least this size go through the copy/compute pipeline
    PIPELINE_MIN_BYTES = 64 << 20

    # Longest loop that is pipelined: the pipeline hides the host link (268 MB
    # each way for 8 fields of 2048^2 complex64: 1.3 ms up, 1.45 ms down) but
    # runs its chunks at a smaller batch, which costs more per step than a
    # whole-batch loop; for that batch the two break even near 120 steps
    # (20 steps: 9.6 against 11.8 ms per call; 200 steps: 78.7 against 77.1).
    PIPELINE_MAX_STEPS = 100

    def _pipeline_bounds(self, E_in, nsteps: int):
        """Field bounds of the host-to-host pipeline's chunks, or None.

        A page-locked host batch of 2-D fields (this class, no nonlocal
        response) of at least PIPELINE_MIN_BYTES, propagated over at most
        PIPELINE_MAX_STEPS steps, is split by fields: the first and the last
        field alone, the others together, so that only one field's upload
        and one field's download are not hidden behind a propagation."""
        if type(self) is not NLSE or self.nl_length > 0 or nsteps > self.PIPELINE_MAX_STEPS:
            return None
        if not (isinstance(E_in, torch.Tensor) and not E_in.is_cuda and E_in.is_pinned()
                and E_in.is_contiguous()):
            return None
        lead = self._lead_shape(tuple(E_in.shape))
        nf = int(np.prod(lead)) if lead else 1
        return pipeline_split(nf, E_in.numel() * E_in.element_size(), nsteps,
                              self.PIPELINE_MAX_STEPS, self.PIPELINE_MIN_BYTES)

    def _out_field_pipelined(self, E_in: torch.Tensor, z: float, precision: str, verbose: bool,
                             normalize: bool, bounds: list) -> torch.Tensor:
        """out_field of a page-locked host batch with the host link and the
        device overlapped: the batch is split into field chunks; chunk i is
        uploaded on one stream, normalised and propagated (its own plan and
        captured loop) on the current stream, and downloaded into page-locked
        memory on a third stream while chunk i + 1 is propagated.  Every field
        is computed exactly as in the unsplit call with the same kernel variant
        (fields are independent)."""
        dev = self._device
        if self.propagator is None:
            self.propagator = self._build_propagator()
        self._send_arrays_to_gpu()
        V = None if self.V is None else self.V.clone()
        shape = tuple(E_in.shape)
        lead = self._lead_shape(shape)
        nf = int(np.prod(lead))
        grid = shape[len(lead):]
        host_in = E_in.reshape(nf, *grid)
        A = torch.empty((nf, *grid), dtype=E_in.dtype, device=dev)
        stage = torch.empty_like(A) if normalize else A
        out = torch.empty((nf, *grid), dtype=E_in.dtype, pin_memory=True)
        dtype = engine.dtype_code(A)
        plans = [Plan.get(2, grid, b1 - b0, 1, dtype, dev, slot=i)
                 for i, (b0, b1) in enumerate(zip(bounds, bounds[1:]))]
        big = max(range(len(plans)), key=lambda i: bounds[i + 1] - bounds[i])
        cur = torch.cuda.current_stream(dev)
        s_in, s_out = _pipeline_streams(dev)
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(cur)
        t0 = time.perf_counter()
        n2_old = self.n2
        try:
            if z > self.L:
                self.n2 = 0
            n = count_steps(z, self.delta_z)
            op = self._operator(A, V, self.propagator, precision, None, plans[0])
            target = None
            if normalize:
                target = torch.from_numpy(np.array(self._norm_target(lead), dtype=np.float64)
                                          .reshape(-1)).to(dev)
            # uploads: all chunks back to back on s_in, after this stream's set-up
            s_in.wait_stream(cur)
            loaded = []
            with torch.cuda.stream(s_in):
                for b0, b1 in zip(bounds, bounds[1:]):
                    stage[b0:b1].copy_(host_in[b0:b1], non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(s_in)
                    loaded.append(ev)
            for i, (b0, b1) in enumerate(zip(bounds, bounds[1:])):
                cur.wait_event(loaded[i])
                Ac = A[b0:b1]
                if normalize:
                    sums = engine.power(stage[b0:b1], b1 - b0)
                    engine.normalize(stage[b0:b1], Ac, b1 - b0, sums, target[b0:b1],
                                     self._norm_coef())
                if n > 0:
                    # every chunk runs the kernel variant tuned for the largest
                    # one (tuned once per process, on that chunk's buffer)
                    if not getattr(plans[big], "_tuned", False):
                        cur.wait_event(loaded[big])
                        autotune.maybe_tune(plans[big], A[bounds[big]:bounds[big + 1]], op)
                    if i != big:
                        v = plans[big].get_variant()
                        plans[i].set_variant(v["rows"], v["cols"], v["rows_cap"], v["cols_cap"])
                    engine.propagate(plans[i], Ac, op, n, 0, graph=True, field0=b0)
                done = torch.cuda.Event()
                done.record(cur)
                s_out.wait_event(done)
                with torch.cuda.stream(s_out):
                    out[b0:b1].copy_(Ac, non_blocking=True)
            cur.wait_stream(s_out)
        finally:
            self.n2 = n2_old
        end.record(cur)
        end.synchronize()
        if verbose:
            print(f"\nTime spent to solve : {start.elapsed_time(end) * 1e-3} s (GPU) /"
                  f" {time.perf_counter() - t0} s (CPU)\n")
        self._retrieve_arrays_from_gpu()
        return out.reshape(shape)

    def _op_key(self):
        """Snapshot of the attributes the operator depends on (callbacks may change them)."""
        def k(x):
            if isinstance(x, torch.Tensor):
                return ("t", x.data_ptr(), x._version)
            if isinstance(x, np.ndarray):
                return ("a", x.tobytes())
            return x
        return tuple(k(getattr(self, n, None)) for n in self._OP_ATTRS)

    _OP_ATTRS = ("delta_z", "n2", "alpha", "I_sat", "k")

    def plot_field(self, A_plot, z: float) -> None:
        """Plotting is not provided (matplotlib is not a dependency of this engine)."""
        raise NotImplementedError("plot_field is not part of this engine")
