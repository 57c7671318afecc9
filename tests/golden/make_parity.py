"""Parity fixtures beside make_golden.py's, computed by the reference package itself.

Runs Quantum-Optics-LKB/NLSE v2.3.0 unmodified through make_golden.py's
import stand-ins.  The FFT behind the VkFFTApp stand-in is selectable: scipy's
pocketfft (make_golden.py's choice), NumPy's pocketfft or torch's CPU FFT
(oneMKL on x86).  The three are equally valid complex64 FFTs that differ only
in rounding (about 1.5e-7 rel-L2 per transform of a random 256^2 array).

Parts (each writes .npz files under tests/golden/):

  spread    every golden case re-run with the NumPy and torch FFTs at the
            case's own length -> spread/<case>.npz {out_numpy, out_torch}:
            how far the reference's own results move when only the FFT's
            rounding changes.
  short     every complex64 case stopped after 20 loop steps, with all three
            FFTs -> short/<case>.npz {out, out_numpy, out_torch, steps}.
  ddgpe128  the four DDGPE cases with complex128 fields and pump profiles
            -> ddgpe_c128_<branch>.npz
            (replayed by the golden tests like every other fixture).
  imagtime  CNLSE with Rabi coupling and DDGPE (pump, probe, potential,
            Rabi coupling) with a complex delta_z, complex128
            -> cnlse_c128_single_rabi_cdz.npz, ddgpe_c128_single_V_cdz.npz
            (+ spread/).
  maps      NLSE 2-D with n2, alpha and Isat varying over the grid -> maps_*.npz
            (golden fixtures; run before spread and short, which cover them).
  fullsize  the benchmark configurations at their stated sizes (outputs
            subsampled on a regular grid, FP64 power of the whole field):
              nlse2048   2048^2 noisy beam, dz = 2e-5 m, 501 steps, "single";
              cnlse1024  CNLSE 1024^2, two components, Gaussian nonlocal kernel
                         (sigma 100 um, 67^2 support), 400 steps, "single";
              mixed      field 0 of each grid size of the 164-field batch
                         (tests/cases.py mixed_batch, seed 11; per-field power
                         (1,) and n2 (1, 1, 1) float64 arrays, so the
                         reference evaluates the complex64 nonlinear step in
                         FP64), 201 steps;
            each in complex128 and complex64, each with the three FFTs
            -> fullsize/<case>_<c128|c64>_single.npz
            (fullsize:nlse2048,c128 picks cases and/or one dtype)

Usage: python tests/golden/make_parity.py REFERENCE_ROOT [part ...]
       (or NLSE_REFERENCE_ROOT=...; default: every part)
"""

from __future__ import annotations

import os
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

import make_golden as mg  # noqa: E402

SHORT_STEPS = 20
WORKERS = os.cpu_count() or 1


# ---------------------------------------------------------------------------
# FFT backends behind the VkFFTApp / pyfftw stand-ins
# ---------------------------------------------------------------------------
class ScipyFFT:
    """scipy.fft (pocketfft), all host threads (threads split lines: same result)."""

    @staticmethod
    def fftn(x, axes):
        return mg.sfft_orig.fftn(x, axes=axes, workers=WORKERS)

    @staticmethod
    def ifftn(x, axes):
        return mg.sfft_orig.ifftn(x, axes=axes, workers=WORKERS)


class NumpyFFT:
    @staticmethod
    def fftn(x, axes):
        return np.fft.fftn(np.asarray(x), axes=axes)

    @staticmethod
    def ifftn(x, axes):
        return np.fft.ifftn(np.asarray(x), axes=axes)


class TorchFFT:
    @staticmethod
    def fftn(x, axes):
        import torch

        return torch.fft.fftn(torch.from_numpy(np.ascontiguousarray(x)), dim=axes).numpy()

    @staticmethod
    def ifftn(x, axes):
        import torch

        return torch.fft.ifftn(torch.from_numpy(np.ascontiguousarray(x)), dim=axes).numpy()


BACKENDS = {"scipy": ScipyFFT, "numpy": NumpyFFT, "torch": TorchFFT}


def use_fft(kind: str) -> None:
    mg.sfft = BACKENDS[kind]


def save(path: Path, **arrays) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, **arrays)
    print(f"  {path.relative_to(HERE)}: " + ", ".join(f"{k}{np.shape(v)}" for k, v in arrays.items()),
          flush=True)


# ---------------------------------------------------------------------------
# parts on the golden cases
# ---------------------------------------------------------------------------
def _cases():
    from tests import golden_cases as gc

    return gc, [n for n in gc.FIXTURES if "cpu" not in n]


def part_spread() -> None:
    gc, names = _cases()
    for name in names:
        outs = {}
        for kind in ("numpy", "torch"):
            use_fft(kind)
            outs[f"out_{kind}"] = gc.run(name, "reference")
        use_fft("scipy")
        save(HERE / "spread" / f"{name}.npz", **outs)


def part_short() -> None:
    gc, names = _cases()
    for name in names:
        if "c128" in name or "beyond_L" in name:
            continue
        outs = {}
        for kind in ("scipy", "numpy", "torch"):
            use_fft(kind)
            outs["out" if kind == "scipy" else f"out_{kind}"] = gc.run(name, "reference",
                                                                      steps=SHORT_STEPS)
        use_fft("scipy")
        save(HERE / "short" / f"{name}.npz", steps=np.array(SHORT_STEPS), **outs)


def part_ddgpe128() -> None:
    """The DDGPE cases with complex128 fields and complex128 pump and probe
    profiles: the reference forms the pump term F_r * F_t[i] * dz * 1j in the
    profiles' precision, so complex128 profiles keep the whole step in FP64."""
    gc, _ = _cases()
    use_fft("scipy")
    for branch in ("single_noV", "single_V", "double_noV", "double_V"):
        src = gc.load(f"ddgpe_c64_{branch}")
        arrays = dict(src)
        arrays["E_in"] = src["E_in"].astype(np.complex128)
        for k in ("Fr", "Ft", "Pr", "Pt"):
            arrays[k] = src[k].astype(np.complex128)
        name = f"ddgpe_c128_{branch}"
        np.savez_compressed(HERE / f"{name}.npz", **{**arrays, "out": np.zeros(0)})
        out = gc.run(name, "reference")
        assert out.dtype == np.complex128
        arrays["out"] = out
        save(HERE / f"{name}.npz", **arrays)


def part_imagtime() -> None:
    """CNLSE with Rabi coupling and DDGPE with a complex delta_z (imaginary-time
    evolution, NLSE/nlse.py:505-508): the cnlse_c128_single_rabi inputs with
    dz = (1 - 0.4j) 5e-5 and the ddgpe_c128_single_V inputs with dz =
    (1 - 0.3j) 0.1/32 -- the reference's rabi_coupling then takes the complex
    cosine and sine of the step (kernels_gpu.py:155-156) and the DDGPE source
    term the complex product F dz i (ddgpe.py:155-156)
    -> cnlse_c128_single_rabi_cdz.npz, ddgpe_c128_single_V_cdz.npz and their
    spread/ entries."""
    gc, _ = _cases()
    for name, src, dz in (("cnlse_c128_single_rabi_cdz", "cnlse_c128_single_rabi", (1 - 0.4j) * 5e-5),
                          ("ddgpe_c128_single_V_cdz", "ddgpe_c128_single_V", (1 - 0.3j) * 0.1 / 32)):
        use_fft("scipy")
        arrays = dict(gc.load(src))
        arrays["dz"] = np.array(dz)
        np.savez_compressed(HERE / f"{name}.npz", **{**arrays, "out": np.zeros(0)})
        arrays["out"] = gc.run(name, "reference")
        save(HERE / f"{name}.npz", **arrays)
        outs = {}
        for kind in ("numpy", "torch"):
            use_fft(kind)
            outs[f"out_{kind}"] = gc.run(name, "reference")
        use_fft("scipy")
        save(HERE / "spread" / f"{name}.npz", **outs)


def part_maps() -> None:
    """NLSE 2-D with n2, alpha and Isat varying over the grid (the reference
    broadcasts them in nl_prop; float64 arrays make it evaluate the step in
    FP64), 64^2, 201 steps: complex64 "single" and complex128 "double", and a
    three-field batch with a per-field n2 and an Isat map."""
    from tests import golden_cases as gc

    use_fft("scipy")
    N = 64
    sim = _R.NLSE(mg.ALPHA, mg.POWER, mg.WINDOW, mg.N2, None, mg.L, NX=N, NY=N, Isat=mg.ISAT,
                  backend="GPU")
    XX, YY = sim.XX.astype(np.float64), sim.YY.astype(np.float64)
    n2 = mg.N2 * (1 + 0.5 * np.exp(-(XX ** 2 + YY ** 2) / (1.5e-3) ** 2))
    alpha = mg.ALPHA * (1 + 0.5 * XX / mg.WINDOW)
    isat = mg.ISAT * (1 + 4 * (YY / mg.WINDOW) ** 2)
    E = mg.gauss(sim.XX, sim.YY)
    V = mg.well(sim.XX, sim.YY).astype(np.complex64)
    for name, dt, prec, B in (("maps_c64_single", np.complex64, "single", 0),
                              ("maps_c128_double", np.complex128, "double", 0),
                              ("maps_c64_batch3", np.complex64, "single", 3)):
        E_in = (np.broadcast_to(E, (B, N, N)) if B else E).astype(dt)
        f = dict(E_in=E_in, V=V,
                 n2=n2 if not B else np.linspace(-1.6e-9, -4e-10, B).reshape(B, 1, 1),
                 alpha=alpha if not B else np.asarray(mg.ALPHA), isat=isat,
                 precision=np.array(prec))
        np.savez_compressed(HERE / f"{name}.npz", **f, out=np.zeros(0))
        out = gc.run(name, "reference")
        save(HERE / f"{name}.npz", **f, out=out)


# ---------------------------------------------------------------------------
# full-size configurations
# ---------------------------------------------------------------------------
def _builders():
    from tests import cases

    return cases


def subsample(E):
    return _builders().subsample(E)


def power_fp64(E):
    return _builders().power_fp64(E)


def nlse2048_inputs(R_NLSE, dtype):
    return _builders().nlse2048_inputs(R_NLSE, dtype)


def cnlse1024_inputs(R_CNLSE, dtype):
    return _builders().cnlse1024_inputs(R_CNLSE, dtype)


def mixed_inputs(R_NLSE, dtype, group: int):
    return _builders().mixed_field0(R_NLSE, dtype, group)


def part_fullsize(which=("nlse2048", "cnlse1024", "mixed")) -> None:
    kinds = ("scipy", "numpy", "torch")
    dtypes = [d for d, t in ((np.complex128, "c128"), (np.complex64, "c64")) if t in which]
    dtypes = dtypes or [np.complex128, np.complex64]
    cases_ = [c for c in ("nlse2048", "cnlse1024", "mixed") if c in which]
    which = cases_ or ("nlse2048", "cnlse1024", "mixed")
    from functools import partial
    from types import SimpleNamespace

    # the reference's GPU path (its constructors pick the CPU backend by default here)
    R = SimpleNamespace(NLSE=partial(_R.NLSE, backend="GPU"), CNLSE=partial(_R.CNLSE, backend="GPU"))
    if "nlse2048" in which:
        for dtype in dtypes:
            outs = {}
            for kind in kinds:
                use_fft(kind)
                sim, E = nlse2048_inputs(R.NLSE, dtype)
                t = time.time()
                out = sim.out_field(E, 10e-3, precision="single", verbose=False)
                print(f"  nlse2048 {np.dtype(dtype).name} {kind}: {time.time() - t:.0f} s",
                      flush=True)
                outs[f"sub_{kind}"] = subsample(out)
                outs[f"power_{kind}"] = power_fp64(out)
            use_fft("scipy")
            tag = "c128" if dtype == np.complex128 else "c64"
            save(HERE / "fullsize" / f"nlse2048_{tag}_single.npz", N=np.array(2048), seed=np.array(0),
                 dz=np.array(2e-5), z=np.array(10e-3), **outs)
    if "cnlse1024" in which:
        for dtype in dtypes:
            outs = {}
            for kind in kinds:
                use_fft(kind)
                sim, E = cnlse1024_inputs(R.CNLSE, dtype)
                t = time.time()
                out = sim.out_field(E, 20e-3, precision="single", verbose=False)
                print(f"  cnlse1024 {np.dtype(dtype).name} {kind}: {time.time() - t:.0f} s",
                      flush=True)
                outs[f"sub_{kind}"] = subsample(out)
                outs[f"power_{kind}"] = power_fp64(out)
            use_fft("scipy")
            tag = "c128" if dtype == np.complex128 else "c64"
            save(HERE / "fullsize" / f"cnlse1024_{tag}_single.npz", N=np.array(1024),
                 dz=np.array(5e-5), z=np.array(20e-3), **outs)
    if "mixed" in which:
        for g, N in enumerate((256, 512, 1024, 2048)):
            for dtype in dtypes:
                outs = {}
                for kind in kinds:
                    use_fft(kind)
                    sim, E = mixed_inputs(R.NLSE, dtype, g)
                    t = time.time()
                    out = sim.out_field(E, 10e-3, precision="single", verbose=False)
                    print(f"  mixed {N} {np.dtype(dtype).name} {kind}: {time.time() - t:.0f} s",
                          flush=True)
                    outs[f"sub_{kind}"] = subsample(out)
                    outs[f"power_{kind}"] = power_fp64(out)
                use_fft("scipy")
                tag = "c128" if dtype == np.complex128 else "c64"
                save(HERE / "fullsize" / f"mixed{N}_{tag}_single.npz", N=np.array(N),
                     group=np.array(g), **outs)


_R = None


def main() -> None:
    global _R
    parts = [a for a in sys.argv[1:] if a in ("spread", "short", "ddgpe128", "maps", "imagtime",
                                              "fullsize")
             or a.startswith("fullsize:")]
    args = [a for a in sys.argv[1:] if a not in parts]
    sys.argv = [sys.argv[0]] + args
    ref = mg._reference_root().resolve()
    os.chdir(tempfile.mkdtemp(prefix="nlse_parity_"))
    _R = mg.load_reference(ref)
    mg.sfft_orig = mg.sfft
    use_fft("scipy")
    from tests import golden_cases as gc

    gc.set_reference(_R)
    print(f"reference NLSE {_R.__version__} from {ref}")
    for part in parts or ["maps", "spread", "short", "ddgpe128", "imagtime", "fullsize"]:
        t = time.time()
        if part == "maps":
            part_maps()
        elif part == "spread":
            part_spread()
        elif part == "short":
            part_short()
        elif part == "ddgpe128":
            part_ddgpe128()
        elif part == "imagtime":
            part_imagtime()
        elif part.startswith("fullsize"):
            sel = part.split(":", 1)[1].split(",") if ":" in part else ("nlse2048", "cnlse1024",
                                                                        "mixed")
            part_fullsize(tuple(sel))
        print(f"part {part}: {time.time() - t:.0f} s", flush=True)


if __name__ == "__main__":
    main()
