"""Device-side engine: plans, operators and the calls into libnlse_sm103.

Fields and parameters live in torch CUDA tensors owned by Python; the C
library receives raw pointers and the current CUDA stream.  Nothing here
computes on the host beyond the small per-field parameter blocks.
"""

from __future__ import annotations

import ctypes as ct
import itertools
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib

_DT = {torch.complex64: _lib.NLSE_C64, torch.complex128: _lib.NLSE_C128}
_versions = itertools.count(1)


def dtype_code(t: torch.Tensor) -> int:
    try:
        return _DT[t.dtype]
    except KeyError:
        raise TypeError(f"field dtype must be complex64 or complex128, got {t.dtype}") from None


def stream_handle(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def require_cuda(t: torch.Tensor, name: str = "field") -> None:
    if not (isinstance(t, torch.Tensor) and t.is_cuda):
        raise TypeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be C-contiguous")


class Plan:
    """A libnlse_sm103 plan for one field geometry (the VkFFTApp analogue)."""

    _cache: dict = {}

    def __init__(self, ndim: int, shape: tuple, nfields: int, comps: int, dtype: int,
                 device: torch.device):
        self.lib = _lib.load()
        self.ndim, self.shape, self.nfields = ndim, tuple(int(s) for s in shape), int(nfields)
        self.comps, self.dtype, self.device = int(comps), int(dtype), device
        d = _lib.Desc()
        d.ndim = ndim
        for i, s in enumerate(self.shape):
            d.shape[i] = s
        d.nfields = self.nfields
        d.comps = self.comps
        d.dtype = dtype
        h = ct.c_void_p()
        with torch.cuda.device(device):
            _lib.check(self.lib.nlse_plan_create(ct.byref(h), ct.byref(d)), "plan")
        self.handle = h
        self.shape0 = self.shape

    @classmethod
    def get(cls, ndim, shape, nfields, comps, dtype, device, slot: int = 0) -> "Plan":
        """The cached plan of this geometry; slot > 0 gives further plans of the
        same geometry (each keeps its own captured loop)."""
        key = (ndim, tuple(shape), int(nfields), int(comps), int(dtype), str(device), int(slot))
        p = cls._cache.get(key)
        if p is None:
            p = cls(ndim, shape, nfields, comps, dtype, device)
            cls._cache[key] = p
        return p

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.nlse_plan_destroy(h)
            except Exception:
                pass

    def set_nonlocal(self, pads: tuple | None) -> None:
        """Give the plan its zero-padded nonlocal grid (None removes it)."""
        pads = tuple(int(x) for x in pads) if pads else None
        if getattr(self, "_nl_pads", None) == pads:
            return
        py, px = (0, 0) if pads is None else ((1, pads[0]) if len(pads) == 1 else pads)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.nlse_plan_set_nonlocal(self.handle, py, px), "nonlocal grid")
        self._nl_pads = pads

    def set_kernels(self, rows_tma: bool, cols_tma: bool) -> None:
        """Choose the 2-D passes' kernel variants (nlse_plan_set_kernels)."""
        _lib.check(self.lib.nlse_plan_set_kernels(self.handle, int(rows_tma), int(cols_tma)),
                   "kernel variant")

    def set_variant(self, rows: int, cols: int, rows_cap: int = 0, cols_cap: int = 0) -> None:
        """Choose the 2-D passes' variants and CTAs per SM (nlse_plan_set_variant)."""
        _lib.check(self.lib.nlse_plan_set_variant(self.handle, int(rows), int(cols), int(rows_cap),
                                                  int(cols_cap)), "kernel variant")

    def get_variant(self) -> dict:
        """Current variant codes, CTA caps and the available variants (code lists)."""
        v = [ct.c_int32() for _ in range(4)]
        m = [ct.c_uint32() for _ in range(2)]
        _lib.check(self.lib.nlse_plan_get_variant(self.handle, *[ct.byref(x) for x in v],
                                                  *[ct.byref(x) for x in m]), "kernel variant")
        return {"rows": v[0].value, "cols": v[1].value, "rows_cap": v[2].value,
                "cols_cap": v[3].value,
                "rows_avail": [i for i in range(32) if m[0].value >> i & 1],
                "cols_avail": [i for i in range(32) if m[1].value >> i & 1]}

    def get_kernels(self) -> tuple:
        """(rows_tma, cols_tma, rows_tma available, cols_tma available)."""
        v = [ct.c_int32() for _ in range(4)]
        _lib.check(self.lib.nlse_plan_get_kernels(self.handle, *[ct.byref(x) for x in v]),
                   "kernel variant")
        return tuple(bool(x.value) for x in v)

    def status(self) -> None:
        """Synchronise and raise if a kernel of this plan gave up a bounded wait."""
        with torch.cuda.device(self.device):
            _lib.check(self.lib.nlse_plan_status(self.handle, stream_handle(self.device)),
                       "plan status")

    # -- transforms -------------------------------------------------------
    def fft(self, A: torch.Tensor, B: torch.Tensor | None = None) -> torch.Tensor:
        """Forward transform over the plan axes (VkFFTApp.fft)."""
        return self._fft(A, B, 0)

    def ifft(self, A: torch.Tensor, B: torch.Tensor | None = None) -> torch.Tensor:
        """Normalised inverse transform (VkFFTApp.ifft with norm=1)."""
        return self._fft(A, B, 1)

    def _fft(self, A, B, inverse):
        require_cuda(A)
        if B is not None and B.data_ptr() != A.data_ptr():
            B.copy_(A)
            A = B
        with torch.cuda.device(A.device):
            _lib.check(self.lib.nlse_fft(self.handle, A.data_ptr(), inverse,
                                         stream_handle(A.device)), "fft")
        return A


@dataclass
class OperatorData:
    """Device buffers of one split-step operator and its C descriptor."""

    prop: torch.Tensor
    params: torch.Tensor
    scheme: int
    rabi: bool = False
    V: torch.Tensor | None = None
    v_fstride: int = 0
    prop_cstride: int = 0
    pump: tuple | None = None  # (pump_r, pump_t, probe_r, probe_t) device tensors or None
    nl_khat: torch.Tensor | None = None  # nonlocal kernel spectrum on the padded grid
    maps: torch.Tensor | None = None  # [3][map fields][pixels] g, alpha/2, 1/Isat' planes
    maps_mask: int = 0
    keep: list = field(default_factory=list)
    # unique per operator: tells the plan its cached copy of the propagator is stale
    version: int = field(default_factory=lambda: next(_versions))

    def struct(self, field0: int = 0) -> _lib.Operator:
        """The C descriptor; field0 > 0 describes fields field0, field0 + 1, ... of
        the batch the operator was built for (per-field parameters, potentials
        and coefficient planes start at that field)."""
        o = _lib.Operator()
        if self.V is not None:
            o.V = self.V.data_ptr() + field0 * int(self.v_fstride) * self.V.element_size()
            o.v_complex = int(self.V.is_complex())
            o.v_f32 = int(self.V.dtype in (torch.float32, torch.complex64))
            o.v_fstride = int(self.v_fstride)
        o.prop = self.prop.data_ptr()
        o.prop_c128 = int(self.prop.dtype == torch.complex128)
        o.prop_cstride = int(self.prop_cstride)
        o.params = self.params.data_ptr() + field0 * _lib.NLSE_PARAM_STRIDE * 8
        o.scheme = int(self.scheme)
        o.rabi = int(bool(self.rabi))
        if self.pump is not None:
            pr, pt, qr, qt = self.pump
            if pr is not None:
                o.pump_r, o.pump_t = pr.data_ptr(), pt.data_ptr()
            if qr is not None:
                o.probe_r, o.probe_t = qr.data_ptr(), qt.data_ptr()
        o.prop_version = int(self.version)
        if self.nl_khat is not None:
            o.nl_khat = self.nl_khat.data_ptr()
        if self.maps is not None and self.maps_mask:
            o.maps_plane = int(self.maps.shape[1] * self.maps.shape[2])
            o.maps_fstride = int(self.maps.shape[2]) if self.maps.shape[1] > 1 else 0
            o.nl_maps = self.maps.data_ptr() + field0 * o.maps_fstride * self.maps.element_size()
            o.maps_mask = int(self.maps_mask)
        if field0 and self.pump is not None:
            raise ValueError("a field offset of an operator with pump terms")
        return o


def propagate(plan: Plan, A: torch.Tensor, op: OperatorData, nsteps: int, step0: int = 0,
              graph: bool = False, field0: int = 0) -> None:
    """Advance A in place by nsteps split steps (nlse_propagate); A holds the
    fields field0, field0 + 1, ... of the batch op was built for."""
    require_cuda(A)
    s = op.struct(field0)
    flags = _lib.NLSE_RUN_GRAPH if graph else 0
    with torch.cuda.device(A.device):
        _lib.check(plan.lib.nlse_propagate(plan.handle, A.data_ptr(), ct.byref(s), int(nsteps),
                                           int(step0), flags, stream_handle(A.device)),
                   "propagate")


def run_pass(plan: Plan, A: torch.Tensor, op: OperatorData, which: int, step: int = 0) -> None:
    """Enqueue one pass of the step sequence (nlse_pass)."""
    require_cuda(A)
    s = op.struct()
    with torch.cuda.device(A.device):
        _lib.check(plan.lib.nlse_pass(plan.handle, A.data_ptr(), ct.byref(s), int(which),
                                      int(step), stream_handle(A.device)), "pass")


def nonlinear(plan: Plan, A: torch.Tensor, op: OperatorData, asq: torch.Tensor | None = None,
              step: int = 0) -> None:
    """Nonlinear step only (parameter set 0), pointwise (nlse_nonlinear)."""
    require_cuda(A)
    s = op.struct()
    with torch.cuda.device(A.device):
        _lib.check(plan.lib.nlse_nonlinear(plan.handle, A.data_ptr(),
                                           asq.data_ptr() if asq is not None else None,
                                           ct.byref(s), int(step), stream_handle(A.device)),
                   "nonlinear")


def power(A: torch.Tensor, nseg: int) -> torch.Tensor:
    """FP64 sums of |A|^2 over nseg equal contiguous segments (device tensor)."""
    require_cuda(A)
    lib = _lib.load()
    n = A.numel()
    if nseg <= 0 or n % nseg:
        raise ValueError("segments must tile the array")
    seg = n // nseg
    out = torch.empty(nseg, dtype=torch.float64, device=A.device)
    wsb = lib.nlse_power_workspace_size(nseg, seg)
    ws = torch.empty(max(1, wsb // 8), dtype=torch.float64, device=A.device)
    with torch.cuda.device(A.device):
        _lib.check(lib.nlse_power(A.data_ptr(), dtype_code(A), nseg, seg, out.data_ptr(),
                                  ws.data_ptr(), wsb, stream_handle(A.device)), "power")
    return out


def delta_n(A: torch.Tensor, pix: int, coef: torch.Tensor, isat: torch.Tensor, flags: int,
            out: torch.Tensor) -> None:
    """evaluate_delta_n's index change of A into out (nlse_delta_n); coef and
    isat: FP64 device values per segment of pix points."""
    require_cuda(A)
    nseg = A.numel() // pix
    want = torch.float64 if (flags or A.dtype == torch.complex128) else torch.float32
    if out.dtype != want or out.numel() != A.numel() or not out.is_contiguous():
        raise ValueError(f"delta_n output must be a contiguous {want} array of the field's size")
    with torch.cuda.device(A.device):
        _lib.check(_lib.load().nlse_delta_n(A.data_ptr(), dtype_code(A), nseg, pix,
                                            coef.data_ptr(), isat.data_ptr(), int(flags),
                                            out.data_ptr(), stream_handle(A.device)), "delta_n")


def delta_n_max(A: torch.Tensor, pix: int, n2abs: torch.Tensor, isat: torch.Tensor, c: float,
                eps0: float, flags: int, out: torch.Tensor) -> None:
    """adapt_delta_z's peak index change of A into the FP64 device scalar out
    (nlse_delta_n_max); stream-ordered, nothing is read back here."""
    require_cuda(A)
    nseg = A.numel() // pix
    if out.dtype != torch.float64 or out.numel() < 1:
        raise ValueError("delta_n_max writes one float64 value")
    with torch.cuda.device(A.device):
        _lib.check(_lib.load().nlse_delta_n_max(A.data_ptr(), dtype_code(A), nseg, pix,
                                                n2abs.data_ptr(), isat.data_ptr(), float(c),
                                                float(eps0), int(flags), out.data_ptr(),
                                                stream_handle(A.device)), "delta_n_max")


def normalize(src: torch.Tensor, dst: torch.Tensor, nseg: int, sums: torch.Tensor,
              target: torch.Tensor, coef: float) -> None:
    """dst = src * sqrt(target / (sums * coef)) per segment (nlse_normalize)."""
    require_cuda(src)
    require_cuda(dst)
    lib = _lib.load()
    seg = src.numel() // nseg
    with torch.cuda.device(src.device):
        _lib.check(lib.nlse_normalize(src.data_ptr(), dst.data_ptr(), dtype_code(src), nseg, seg,
                                      sums.data_ptr(), target.data_ptr(), float(coef),
                                      stream_handle(src.device)), "normalize")


def square_mod(A: torch.Tensor, out: torch.Tensor) -> None:
    require_cuda(A)
    require_cuda(out)
    lib = _lib.load()
    with torch.cuda.device(A.device):
        _lib.check(lib.nlse_square_mod(A.data_ptr(), out.data_ptr(), dtype_code(A), A.numel(),
                                       stream_handle(A.device)), "square_mod")


def per_field(x, lead: tuple, n_axes: int, name: str) -> np.ndarray:
    """Broadcast a scalar or per-field parameter to one float64 value per field.

    The reference broadcasts parameter arrays against the field with NumPy
    rules; per-field values are arrays whose trailing n_axes dimensions are 1
    (e.g. n2 of shape (B, 1, 1) for (B, NY, NX) fields).
    """
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    a = np.asarray(x)
    if np.iscomplexobj(a):
        if np.any(a.imag != 0):
            raise NotImplementedError(f"complex {name} is not supported")
        a = a.real
    a = a.astype(np.float64)
    if a.ndim > 0:
        if a.ndim >= n_axes and n_axes > 0:
            tail = a.shape[a.ndim - n_axes:]
            if any(t != 1 for t in tail):
                raise NotImplementedError(
                    f"{name} varies across the transverse grid (shape {a.shape}); only per-field "
                    "values with trailing singleton axes are supported")
            a = a.reshape(a.shape[: a.ndim - n_axes])
        elif n_axes > 0:
            raise NotImplementedError(
                f"{name} of shape {a.shape} would broadcast along the grid axes")
    try:
        b = np.broadcast_to(a, lead)
    except ValueError:
        raise ValueError(f"{name} of shape {np.shape(x)} does not broadcast to fields {lead}") from None
    return np.ascontiguousarray(b).reshape(-1)


def varies_on_grid(x, n_axes: int) -> bool:
    """Whether a parameter, broadcast with NumPy's rules against fields whose
    last n_axes axes are the grid, changes along a grid axis (its own trailing
    n_axes dimensions, right-aligned, are not all 1)."""
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    shape = np.shape(x)
    tail = shape[max(0, len(shape) - n_axes):]
    return any(t != 1 for t in tail)


def coef_plane(x, lead: tuple, grid: tuple) -> np.ndarray:
    """A grid-varying parameter broadcast to the fields: (1, pixels) when it is
    the same for every field, else (fields, pixels); float64."""
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    a = np.asarray(x, dtype=np.float64)
    full = tuple(lead) + tuple(grid)
    try:
        b = np.broadcast_to(a, full)
    except ValueError:
        raise ValueError(f"parameter of shape {a.shape} does not broadcast to fields {full}") from None
    pix = int(np.prod(grid))
    own_lead = a.shape[:max(0, a.ndim - len(grid))]
    if all(s == 1 for s in own_lead):
        return np.ascontiguousarray(b.reshape(-1, pix)[:1])
    return np.ascontiguousarray(b).reshape(-1, pix)


def next_pow2(n: int) -> int:
    p = 1
    while p < n:
        p *= 2
    return p


def nonlocal_spectrum(profile, grid: tuple, dtype: torch.dtype, device) -> tuple:
    """Padded grid and kernel spectrum of the linear "same" convolution.

    scipy's oaconvolve(a, k, mode="same") output i is the full convolution at
    i + (M-1)//2 for an M-point kernel.  With the kernel placed on a cyclic
    grid of P >= N + M - 1 - (M-1)//2 points so that its element (M-1)//2
    sits at the origin, the cyclic convolution equals that output on the N
    points of the field (no wrap-around reaches them).  The spectrum is the
    project FFT of that placed kernel.
    """
    k = profile.detach().cpu().numpy() if isinstance(profile, torch.Tensor) else np.asarray(profile)
    k = np.asarray(k, dtype=np.float64)
    if k.ndim != len(grid):
        raise ValueError(f"nonlocal kernel of {k.ndim} axes for a {len(grid)}-axis field")
    pads = tuple(next_pow2(n + m - 1 - (m - 1) // 2) for n, m in zip(grid, k.shape))
    placed = np.zeros(pads, dtype=np.float64)
    placed[tuple(slice(0, m) for m in k.shape)] = k
    placed = np.roll(placed, shift=[-((m - 1) // 2) for m in k.shape], axis=tuple(range(k.ndim)))
    khat = torch.from_numpy(placed.astype(np.complex128)).to(device=device, dtype=dtype)
    plan = Plan.get(len(pads), pads, 1, 1, dtype_code(khat), device)
    plan.fft(khat)
    return pads, khat.contiguous()


PINNED_MIN_BYTES = 8 << 20


def to_host(t: torch.Tensor) -> torch.Tensor:
    """A new host tensor with the values of t.

    Large results land in page-locked memory from torch's caching host
    allocator: the device copy then runs at the host link's rate and no
    second host copy is needed (a copy into newly mapped pageable memory runs
    at a tenth of that, its page faults included).  A freed result's block
    is reused by the next result of the same size; release_staging() returns
    the cached blocks to the system."""
    if not t.is_cuda or t.numel() * t.element_size() < PINNED_MIN_BYTES:
        return t.cpu()
    t = t.contiguous()
    out = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    out.copy_(t)  # waits for the producing stream, then copies at the pinned rate
    return out


def release_staging() -> None:
    """Return the page-locked blocks cached for host results to the system
    (blocks still held by live results are kept)."""
    empty = getattr(torch._C, "_host_emptyCache", None)
    if empty is not None:
        empty()


def to_device(x, device, dtype=None) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x.to(device)
    else:
        t = torch.from_numpy(np.ascontiguousarray(x)).to(device)
    if dtype is not None:
        t = t.to(dtype)
    return t.contiguous()


INF = math.inf
