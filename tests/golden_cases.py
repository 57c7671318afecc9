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


def _classes(kind: str) -> dict:
    if kind == "oracle":
        from oracle import nlse_oracle as o

        return dict(NLSE=o.OracleNLSE, NLSE_1d=o.OracleNLSE_1d, NLSE_3d=o.OracleNLSE_3d,
                    CNLSE=o.OracleCNLSE, CNLSE_1d=o.OracleCNLSE_1d, GPE=o.OracleGPE,
                    DDGPE=o.OracleDDGPE)
    import nlse_gb300 as p

    return dict(NLSE=p.NLSE, NLSE_1d=p.NLSE_1d, NLSE_3d=p.NLSE_3d, CNLSE=p.CNLSE,
                CNLSE_1d=p.CNLSE_1d, GPE=p.GPE, DDGPE=p.DDGPE)


def _out(kind, sim, E, z, precision, **kw):
    if kind == "oracle":
        if "cpu" in kw:
            kw.pop("cpu")
        return sim.out_field(E, z, precision=precision, **kw)[0]
    kw.pop("cpu", None)
    return sim.out_field(E, z, precision=precision, verbose=False, **kw)


def run(name: str, kind: str, upcast: bool = False):
    """Final field of fixture `name` computed by `kind` ("oracle" or "product").

    upcast: run the complex64 case in complex128 (same inputs, same
    complex64-rounded propagator), the FP64 reference of its rounding error.
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
        return _out(kind, sim, E, float(z), str(f["precision"]))
    if name.startswith("nlse1d"):
        sim = C["NLSE_1d"](ALPHA, POWER, WINDOW, N2, None, L, NX=256, Isat=ISAT)
        sim.delta_z = 5e-5
        sim.V = f["V"].copy()
        return _out(kind, sim, E, L, "double" if "double" in name else "single")
    if name.startswith("nlse3d"):
        sim = C["NLSE_3d"](alpha=ALPHA, energy=1.05 * 2e-6, window=np.array([WINDOW, 16e-6]),
                           n2=N2, D0=1e-16, vg=3e7, V=None, L=L, NX=16, NY=16, NZ=8, Isat=ISAT)
        sim.delta_z = 2.5e-4
        return _out(kind, sim, E, L, "double" if "double" in name else "single")
    if name.startswith("cnlsenl"):
        sim = C["CNLSE"](ALPHA, 0.5, WINDOW, N2, -0.8e-9, None, 20e-3, NX=64, NY=64, Isat=ISAT,
                         nl_length=100e-6)
        sim.nl_profile = f["nl_profile"].copy()
        sim.delta_z = 5e-5
        sim.power2 = 0.05
        sim.n22 = -1.6e-9
        return _out(kind, sim, E, 2e-3, "double" if "double" in name else "single")
    if name.startswith("cnlse1d"):
        sim = C["CNLSE_1d"](ALPHA, POWER, WINDOW, N2, -1e-10, None, L, NX=128, Isat=ISAT)
        sim.delta_z = 5e-5
        sim.power2 = 10e-3
        return _out(kind, sim, E, L, "double" if "double" in name else "single")
    if name.startswith("cnlse"):
        omega = float(f["meta"][3])
        sim = C["CNLSE"](ALPHA, 0.5, WINDOW, N2, -0.8e-9, None, 20e-3, NX=32, NY=32, Isat=ISAT,
                         omega=None if omega < 0 else omega)
        sim.delta_z = 5e-5
        sim.power2 = 0.05
        sim.n22 = -1.2e-9
        sim.k2 = 2 * np.pi / 795e-9
        sim.V = f["V"].copy()
        return _out(kind, sim, E, 20e-3, "double" if "double" in name else "single")
    if name.startswith("gpe"):
        sim = C["GPE"](gamma=0.5, N=2e5, window=40e-6, g=1e3 / 2e5 * 1e-12, V=None,
                       m=87 * atomic_mass, NX=32, NY=32, sat=1e15)
        sim.delta_z = 1e-5
        sim.delta_t = 1e-5
        return _out(kind, sim, E, 2e-4, "double" if "double" in name else "single")
    if name.startswith("ddgpe"):
        h = 0.654
        sim = C["DDGPE"](gamma=0.07 / h, power=1.0, window=64.0, g=1e-2 / h, omega=5.07 / h,
                         T=2.0, omega_exc=1484.44 / h, omega_cav=1482.76 / h,
                         detuning=0.17 / h, k_z=27.0, NX=32, NY=32)
        sim.delta_z = 0.1 / 32
        if f["V"].size:
            sim.V = f["V"].copy()
        final = {}

        def grab(simu, A, z, i):
            final["A"] = A.clone() if hasattr(A, "clone") else np.array(A, copy=True)

        args = [[f["Fr"], f["Ft"], f["Pr"], f["Pt"]], []]
        prec = "double" if "double" in name else "single"
        if kind == "oracle":
            sim.out_field(E, 2.0, sim.laser_excitation, precision=prec, callback=[grab],
                          callback_args=args)
        else:
            sim.out_field(E, 2.0, sim.laser_excitation, precision=prec, verbose=False,
                          callback=[grab], callback_args=args)
        a = final["A"]
        return a.cpu().numpy() if hasattr(a, "cpu") else a
    raise KeyError(name)


def tolerance(name: str) -> float:
    """rel-L2 bound against a complex128 fixture (complex64 ones: see c64_check)."""
    return 1e-12 if "c128" in name else 1e-5


C64_SLACK = 2.0  # complex64 result: at most this many times the reference's own c64 error


def c64_check(name: str, got) -> dict:
    """Error budget of a complex64 result against the FP64 run of the same inputs.

    The reference's complex64 arithmetic is itself off its FP64 run by err_ref
    (rounding amplified over hundreds of nonlinear steps); a complex64 result is
    accepted when its own error against FP64 is at most C64_SLACK * err_ref (or
    below 1e-5).  Returns the numbers for reporting.
    """
    from tests.cases import rel_l2

    ref = load(name)["out"]
    truth = run(name, "oracle", upcast=True)
    err_ref = rel_l2(ref, truth)
    err_got = rel_l2(got, truth)
    return {"err_ref_vs_fp64": err_ref, "err_vs_fp64": err_got, "err_vs_ref": rel_l2(got, ref),
            "ok": err_got <= max(C64_SLACK * err_ref, 1e-5)}
