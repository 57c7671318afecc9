"""Replay the golden fixtures (tests/golden/*.npz) on the oracle or the product.

Each case rebuilds the solver the way tests/golden/make_golden.py built the
reference one, from the stored inputs, and returns the final field.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
from scipy.constants import atomic_mass

GOLDEN = Path(__file__).resolve().parent / "golden"
WAIST, WAIST2, POWER, N2, ISAT, ALPHA, L = 2.23e-3, 70e-6, 1.05, -1.6e-9, 1e5, 20, 10e-3
WINDOW = 4 * WAIST

FIXTURES = sorted(p.stem for p in GOLDEN.glob("*.npz")
                  if not p.stem.startswith(("kernels_", "step_counts", "callbacks_")))


def load(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


_REFERENCE = None  # the reference package, when a generation script installs it


def set_reference(module) -> None:
    """Let run(..., kind="reference") build the reference package's own classes
    (used by the fixture generation scripts, never by the tests)."""
    global _REFERENCE
    _REFERENCE = module


def _classes(kind: str) -> dict:
    if kind == "reference":
        from functools import partial

        R = _REFERENCE
        return {k: partial(getattr(R, k), backend="GPU")
                for k in ("NLSE", "NLSE_1d", "NLSE_3d", "CNLSE", "CNLSE_1d", "GPE", "DDGPE")}
    if kind == "oracle":
        from oracle import nlse_oracle as o

        return dict(NLSE=o.OracleNLSE, NLSE_1d=o.OracleNLSE_1d, NLSE_3d=o.OracleNLSE_3d,
                    CNLSE=o.OracleCNLSE, CNLSE_1d=o.OracleCNLSE_1d, GPE=o.OracleGPE,
                    DDGPE=o.OracleDDGPE)
    import nlse_gb300 as p

    return dict(NLSE=p.NLSE, NLSE_1d=p.NLSE_1d, NLSE_3d=p.NLSE_3d, CNLSE=p.CNLSE,
                CNLSE_1d=p.CNLSE_1d, GPE=p.GPE, DDGPE=p.DDGPE)


def _out(kind, sim, E, z, precision, **kw):
    if kind == "reference":
        kw.pop("cpu", None)
        return sim.out_field(E, z, precision=precision, verbose=False, **kw)
    if kind == "oracle":
        if "cpu" in kw:
            kw.pop("cpu")
        return sim.out_field(E, z, precision=precision, **kw)[0]
    kw.pop("cpu", None)
    return sim.out_field(E, z, precision=precision, verbose=False, **kw)


def _z(z: float, dz: float, steps: int | None) -> float:
    """Propagation length: the fixture's own, or one that runs `steps` loop steps."""
    return z if steps is None else (steps - 0.5) * dz


def run(name: str, kind: str, upcast: bool = False, steps: int | None = None):
    """Final field of fixture `name` computed by `kind` ("oracle", "product" or,
    in the generation scripts, "reference").

    upcast: run the complex64 case in complex128 (same inputs, same
    complex64-rounded propagator), the FP64 reference of its rounding error.
    steps: stop after this many loop steps instead of the fixture's length
    (the short-horizon cases).
    """
    f = load(name)
    C = _classes(kind)
    E = f["E_in"].astype(np.complex128) if upcast else f["E_in"]
    if name.startswith("nlse2d"):
        N, NY, dz, z, _, nl_length = f["meta"]
        N, NY = int(N), int(NY)
        window = WINDOW if NY == N else [WINDOW, WINDOW * NY / N]
        kw = dict(NX=N, NY=NY, Isat=ISAT, nl_length=float(nl_length))
        if kind == "oracle" and "cpu" in name:
            kw["cpu_kernels"] = True
        sim = C["NLSE"](ALPHA, f["power"][()] if f["power"].ndim == 0 else f["power"], window,
                        f["n2"][()] if f["n2"].ndim == 0 else f["n2"], None, L, **kw)
        sim.delta_z = float(dz)
        sim.V = None if f["V"].size == 0 else f["V"].copy()
        return _out(kind, sim, E, _z(float(z), float(dz), steps), str(f["precision"]))
    if name.startswith("maps"):
        # n2, alpha, Isat as arrays over the grid (or per field), set after construction
        sim = C["NLSE"](ALPHA, POWER, WINDOW, N2, None, L, NX=64, NY=64, Isat=ISAT)
        sim.n2 = f["n2"] if f["n2"].ndim else f["n2"][()]
        sim.alpha = f["alpha"] if f["alpha"].ndim else f["alpha"][()]
        sim.I_sat = f["isat"] if f["isat"].ndim else f["isat"][()]
        sim.delta_z = 5e-5
        sim.V = f["V"].copy()
        return _out(kind, sim, E, _z(L, 5e-5, steps), str(f["precision"]))
    if name.startswith("nlse1d"):
        sim = C["NLSE_1d"](ALPHA, POWER, WINDOW, N2, None, L, NX=256, Isat=ISAT)
        sim.delta_z = 5e-5
        sim.V = f["V"].copy()
        return _out(kind, sim, E, _z(L, 5e-5, steps), "double" if "double" in name else "single")
    if name.startswith("nlse3d"):
        sim = C["NLSE_3d"](alpha=ALPHA, energy=1.05 * 2e-6, window=np.array([WINDOW, 16e-6]),
                           n2=N2, D0=1e-16, vg=3e7, V=None, L=L, NX=16, NY=16, NZ=8, Isat=ISAT)
        sim.delta_z = 2.5e-4
        return _out(kind, sim, E, _z(L, 2.5e-4, steps), "double" if "double" in name else "single")
    if name.startswith("cnlsenl"):
        sim = C["CNLSE"](ALPHA, 0.5, WINDOW, N2, -0.8e-9, None, 20e-3, NX=64, NY=64, Isat=ISAT,
                         nl_length=100e-6)
        sim.nl_profile = f["nl_profile"].copy()
        sim.delta_z = 5e-5
        sim.power2 = 0.05
        sim.n22 = -1.6e-9
        return _out(kind, sim, E, _z(2e-3, 5e-5, steps), "double" if "double" in name else "single")
    if name.startswith("cnlse1d"):
        sim = C["CNLSE_1d"](ALPHA, POWER, WINDOW, N2, -1e-10, None, L, NX=128, Isat=ISAT)
        sim.delta_z = 5e-5
        sim.power2 = 10e-3
        return _out(kind, sim, E, _z(L, 5e-5, steps), "double" if "double" in name else "single")
    if name.startswith("cnlse"):
        omega = float(f["meta"][3])
        sim = C["CNLSE"](ALPHA, 0.5, WINDOW, N2, -0.8e-9, None, 20e-3, NX=32, NY=32, Isat=ISAT,
                         omega=None if omega < 0 else omega)
        # (a complex step: imaginary-time evolution with the Rabi rotation)
        sim.delta_z = complex(f["dz"][()]) if "dz" in f else 5e-5
        sim.power2 = 0.05
        sim.n22 = -1.2e-9
        sim.k2 = 2 * np.pi / 795e-9
        sim.V = f["V"].copy()
        return _out(kind, sim, E, _z(20e-3, 5e-5, steps), "double" if "double" in name else "single")
    if name.startswith("gpe"):
        sim = C["GPE"](gamma=0.5, N=2e5, window=40e-6, g=1e3 / 2e5 * 1e-12, V=None,
                       m=87 * atomic_mass, NX=32, NY=32, sat=1e15)
        sim.delta_z = 1e-5
        sim.delta_t = 1e-5
        return _out(kind, sim, E, _z(2e-4, 1e-5, steps), "double" if "double" in name else "single")
    if name.startswith("ddgpe"):
        h = 0.654
        sim = C["DDGPE"](gamma=0.07 / h, power=1.0, window=64.0, g=1e-2 / h, omega=5.07 / h,
                         T=2.0, omega_exc=1484.44 / h, omega_cav=1482.76 / h,
                         detuning=0.17 / h, k_z=27.0, NX=32, NY=32)
        sim.delta_z = complex(f["dz"][()]) if "dz" in f else 0.1 / 32
        if f["V"].size:
            sim.V = f["V"].copy()
        final = {}

        def grab(simu, A, z, i):
            final["A"] = A.clone() if hasattr(A, "clone") else np.array(A, copy=True)

        args = [[f["Fr"], f["Ft"], f["Pr"], f["Pt"]], []]
        prec = "double" if "double" in name else "single"
        zd = _z(2.0, 0.1 / 32, steps)
        if kind == "oracle":
            sim.out_field(E, zd, sim.laser_excitation, precision=prec, callback=[grab],
                          callback_args=args)
        else:
            sim.out_field(E, zd, sim.laser_excitation, precision=prec, verbose=False,
                          callback=[grab], callback_args=args)
        a = final["A"]
        return a.cpu().numpy() if hasattr(a, "cpu") else a
    raise KeyError(name)


def tolerance(name: str) -> float:
    """rel-L2 bound against a complex128 fixture (complex64 ones: see c64_check)."""
    return 1e-12 if "c128" in name else 1e-5


C64_SLACK = 2.0  # complex64 result: at most this many times the reference's own c64 error
SPREAD_SLACK = 2.0  # complex64 result: at most this many times the reference's FFT spread


def spread(name: str) -> float:
    """How far the reference's own result for `name` moves when only its FFT
    changes: max rel-L2 of the NumPy- and torch-FFT runs against the scipy-FFT
    fixture (tests/golden/spread/, make_parity.py)."""
    from tests.cases import rel_l2

    ref = load(name)["out"]
    with np.load(GOLDEN / "spread" / f"{name}.npz") as z:
        return max(rel_l2(z["out_numpy"], ref), rel_l2(z["out_torch"], ref))


SHORT = sorted(p.stem for p in (GOLDEN / "short").glob("*.npz"))


def load_short(name: str) -> dict:
    """Short-horizon fixture: the reference stopped after `steps` loop steps with
    the scipy FFT (out), the NumPy FFT (out_numpy) and torch's (out_torch)."""
    with np.load(GOLDEN / "short" / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def c64_check(name: str, got) -> dict:
    """Acceptance of a complex64 result of a full-length case.

    Over hundreds of nonlinear steps complex64 rounding is amplified: the
    reference's own result moves by ref_fft_spread (1.6e-6 .. 6.5e-5) when only
    its FFT changes, so no complex64 implementation can be held to 1e-5 there.
    A result is accepted when (1) its distance to the reference fixture is at
    most SPREAD_SLACK * ref_fft_spread (or 1e-5), and (2) its error against the
    FP64 run of the same inputs is at most C64_SLACK times the reference's own
    (or 1e-5).  Returns the numbers for reporting."""
    from tests.cases import rel_l2

    ref = load(name)["out"]
    truth = run(name, "oracle", upcast=True)
    err_ref = rel_l2(ref, truth)
    err_got = rel_l2(got, truth)
    err_vs_ref = rel_l2(got, ref)
    spr = spread(name)
    return {"err_ref_vs_fp64": err_ref, "err_vs_fp64": err_got, "err_vs_ref": err_vs_ref,
            "ref_fft_spread": spr,
            "ok": err_got <= max(C64_SLACK * err_ref, 1e-5)
            and err_vs_ref <= max(SPREAD_SLACK * spr, 1e-5)}
