"""ctypes binding of libnlse_sm103 (include/nlse_gb300.h).

The library is built in-tree by ``nlse_gb300._build.build()``.  Loading fails
loudly when it is missing: there is no fallback implementation.
"""

from __future__ import annotations

import ctypes as ct
import threading
from pathlib import Path

from . import _build

NLSE_C64 = 0
NLSE_C128 = 1
NLSE_RUN_GRAPH = 1
NLSE_PARAM_STRIDE = 40
PASS_FORWARD, PASS_LINEAR, PASS_INV_NL_FWD, PASS_INV_NL = 0, 1, 2, 3
# kernel variants of the 2-D passes (nlse_plan_set_variant)
ROWS_LINE, ROWS_TMA, ROWS_PAIR, ROWS_PAIR8, ROWS_DEEP = 0, 1, 2, 3, 4
COLS_TILE, COLS_TMA, COLS_PAIR, COLS_PAIR8, COLS_DEEP = 0, 1, 2, 3, 4
DN_COEF_F64, DN_ISAT_F64 = 1, 2

OK = 0
ERR_ARG = -1
ERR_UNSUPPORTED = -2
ERR_CUDA = -3
ERR_STATE = -4
ERR_TIMEOUT = -5


class Desc(ct.Structure):
    _fields_ = [
        ("ndim", ct.c_int32),
        ("shape", ct.c_int64 * 3),
        ("nfields", ct.c_int64),
        ("comps", ct.c_int32),
        ("dtype", ct.c_int32),
    ]


class Operator(ct.Structure):
    _fields_ = [
        ("V", ct.c_void_p),
        ("v_complex", ct.c_int32),
        ("v_f32", ct.c_int32),
        ("v_fstride", ct.c_int64),
        ("prop", ct.c_void_p),
        ("prop_c128", ct.c_int32),
        ("prop_cstride", ct.c_int64),
        ("params", ct.c_void_p),
        ("scheme", ct.c_int32),
        ("rabi", ct.c_int32),
        ("pump_r", ct.c_void_p),
        ("pump_t", ct.c_void_p),
        ("probe_r", ct.c_void_p),
        ("probe_t", ct.c_void_p),
        ("prop_version", ct.c_int64),
        ("nl_khat", ct.c_void_p),
        ("nl_maps", ct.c_void_p),
        ("maps_fstride", ct.c_int64),
        ("maps_plane", ct.c_int64),
        ("maps_mask", ct.c_int32),
    ]


# (name, restype, argtypes) for every symbol declared in include/nlse_gb300.h
SIGNATURES = [
    ("nlse_abi_version", ct.c_int, []),
    ("nlse_last_error", ct.c_char_p, []),
    ("nlse_plan_create", ct.c_int, [ct.POINTER(ct.c_void_p), ct.POINTER(Desc)]),
    ("nlse_plan_destroy", ct.c_int, [ct.c_void_p]),
    ("nlse_plan_status", ct.c_int, [ct.c_void_p, ct.c_void_p]),
    ("nlse_plan_set_nonlocal", ct.c_int, [ct.c_void_p, ct.c_int64, ct.c_int64]),
    ("nlse_plan_set_kernels", ct.c_int, [ct.c_void_p, ct.c_int32, ct.c_int32]),
    ("nlse_plan_get_kernels", ct.c_int, [ct.c_void_p] + [ct.POINTER(ct.c_int32)] * 4),
    ("nlse_plan_set_variant", ct.c_int, [ct.c_void_p, ct.c_int32, ct.c_int32, ct.c_int32,
                                         ct.c_int32]),
    ("nlse_plan_get_variant", ct.c_int, [ct.c_void_p] + [ct.POINTER(ct.c_int32)] * 4
     + [ct.POINTER(ct.c_uint32)] * 2),
    ("nlse_group_create", ct.c_int, [ct.POINTER(ct.c_void_p)]),
    ("nlse_group_destroy", ct.c_int, [ct.c_void_p]),
    ("nlse_group_fused", ct.c_int, [ct.c_void_p]),
    (
        "nlse_group_propagate",
        ct.c_int,
        [ct.c_void_p, ct.c_int32, ct.POINTER(ct.c_void_p), ct.POINTER(ct.c_void_p),
         ct.POINTER(Operator), ct.POINTER(ct.c_int64), ct.c_void_p],
    ),
    (
        "nlse_propagate",
        ct.c_int,
        [ct.c_void_p, ct.c_void_p, ct.POINTER(Operator), ct.c_int64, ct.c_int64, ct.c_int32,
         ct.c_void_p],
    ),
    (
        "nlse_pass",
        ct.c_int,
        [ct.c_void_p, ct.c_void_p, ct.POINTER(Operator), ct.c_int32, ct.c_int64, ct.c_void_p],
    ),
    ("nlse_fft", ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_void_p]),
    (
        "nlse_nonlinear",
        ct.c_int,
        [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.POINTER(Operator), ct.c_int64, ct.c_void_p],
    ),
    ("nlse_power_workspace_size", ct.c_size_t, [ct.c_int64, ct.c_int64]),
    (
        "nlse_power",
        ct.c_int,
        [ct.c_void_p, ct.c_int32, ct.c_int64, ct.c_int64, ct.c_void_p, ct.c_void_p, ct.c_size_t,
         ct.c_void_p],
    ),
    (
        "nlse_power_noalloc",
        ct.c_int,
        [ct.c_void_p, ct.c_int32, ct.c_int64, ct.c_int64, ct.c_void_p, ct.c_void_p],
    ),
    (
        "nlse_normalize",
        ct.c_int,
        [ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_int64, ct.c_int64, ct.c_void_p, ct.c_void_p,
         ct.c_double, ct.c_void_p],
    ),
    ("nlse_square_mod", ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_int64, ct.c_void_p]),
    (
        "nlse_add_noise",
        ct.c_int,
        [ct.c_void_p, ct.c_int32, ct.c_int64, ct.c_int64, ct.c_double, ct.c_double, ct.c_uint64,
         ct.c_int64, ct.c_void_p],
    ),
    ("nlse_wait_selftest", ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_void_p]),
    (
        "nlse_delta_n",
        ct.c_int,
        [ct.c_void_p, ct.c_int32, ct.c_int64, ct.c_int64, ct.c_void_p, ct.c_void_p, ct.c_int32,
         ct.c_void_p, ct.c_void_p],
    ),
    (
        "nlse_delta_n_max",
        ct.c_int,
        [ct.c_void_p, ct.c_int32, ct.c_int64, ct.c_int64, ct.c_void_p, ct.c_void_p, ct.c_double,
         ct.c_double, ct.c_int32, ct.c_void_p, ct.c_void_p],
    ),
] + [
    # surrogate kernels (nlse_fno.h): p = pointer (device pointer or stream), l = int64,
    # i = int32, f = float
    (name, ct.c_int, [{"p": ct.c_void_p, "l": ct.c_int64, "i": ct.c_int32, "f": ct.c_float}[c]
                      for c in sig])
    for name, sig in [
        ("nlse_fno_lift_rows", "lpppppppp"),
        ("nlse_fno_cols_analysis", "lpfippp"),
        ("nlse_fno_mix", "lppppp"),
        ("nlse_fno_cols_synthesis", "lppp"),
        ("nlse_fno_layer_rows", "lppppipppppppp"),
        ("nlse_fno_proj_bwd", "lpppppp"),
        ("nlse_fno_layer_rows_bwd", "lpppippppppp"),
        ("nlse_fno_lift_bwd", "lpppppp"),
        ("nlse_fno_mix_wgrad", "lpppp"),
        ("nlse_fno_reduce", "pllpp"),
        ("nlse_fno_pack_spectral", "pppp"),
        ("nlse_fno_pack_conv", "pppp"),
        ("nlse_fno_loss", "lpppppp"),
        ("nlse_fno_adam", "pppplffffifp"),
        ("nlse_fno_gemm_selftest", "pppiipp"),
    ]
]

_lock = threading.Lock()
_lib = None


def load(path: str | Path | None = None) -> ct.CDLL:
    """Load (once) and return the library, with prototypes set."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else _build.lib_path()
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build it with nlse_gb300._build.build() "
                "(nvcc, sm_103a); the engine has no CPU fallback"
            )
        lib = ct.CDLL(str(p))
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.nlse_abi_version() != 2:
            raise RuntimeError("libnlse_sm103 ABI version mismatch")
        _lib = lib
        return lib


def last_error() -> str:
    return load().nlse_last_error().decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    """Raise the Python exception matching a negative status."""
    if rc == OK:
        return
    msg = f"{what}: {last_error()}" if what else last_error()
    if rc == ERR_ARG:
        raise ValueError(msg)
    if rc == ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)
