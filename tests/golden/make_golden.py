"""Generate the golden fixtures by running the reference package itself.

Runs Quantum-Optics-LKB/NLSE v2.3.0 unmodified, from a source checkout
given on the command line or in NLSE_REFERENCE_ROOT, with import stand-ins
for the third-party modules that are absent here:

  cupy           NumPy arrays (an ndarray subclass with .get()), cp.fuse = identity
  cupyx.scipy.signal.oaconvolve -> scipy.signal.oaconvolve
  pyvkfft.cuda.VkFFTApp        -> scipy.fft.fftn / ifftn over the trailing ndim axes
                                  (unnormalised forward, 1/N inverse: norm=1)
  pyfftw         FFTW objects on scipy.fft (CPU path only), aligned allocators
  numba          njit = identity, prange = range (CPU path only)
  matplotlib     stub (plot=False everywhere)

So the fixtures hold the reference's own split-step/out_field arithmetic in
NumPy semantics; only the FFT implementation is substituted.  Output:
tests/golden/*.npz (inputs, parameters and outputs of each case).

Usage: python tests/golden/make_golden.py REFERENCE_ROOT
       (or NLSE_REFERENCE_ROOT=REFERENCE_ROOT python tests/golden/make_golden.py)
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np
import scipy.fft as sfft
import scipy.signal as ssig

OUT = Path(__file__).resolve().parent
def _reference_root() -> Path:
    import os

    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NLSE_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT (the NLSE source checkout; "
                         "or set NLSE_REFERENCE_ROOT)")
    return Path(root)


# ---------------------------------------------------------------------------
# import stand-ins
# ---------------------------------------------------------------------------
class _CpArray(np.ndarray):
    def get(self):
        return np.asarray(self).copy()


def _install_shims() -> None:
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt

    nb = types.ModuleType("numba")

    def njit(*a, **k):
        if a and callable(a[0]):
            return a[0]
        return lambda f: f

    nb.njit = njit
    nb.prange = range
    sys.modules["numba"] = nb

    fw = types.ModuleType("pyfftw")
    fw.config = types.SimpleNamespace(NUM_THREADS=1, PLANNER_EFFORT="FFTW_ESTIMATE")
    fw.interfaces = types.SimpleNamespace(cache=types.SimpleNamespace(enable=lambda: None))
    fw.simd_alignment = 16
    fw.zeros_aligned = lambda shape, dtype=np.complex64, n=None: np.zeros(shape, dtype=dtype)
    fw.empty_aligned = lambda shape, dtype=np.complex64, n=None: np.zeros(shape, dtype=dtype)
    fw.import_wisdom = lambda w: None
    fw.export_wisdom = lambda: ()

    class FFTW:
        def __init__(self, a, b, direction="FFTW_FORWARD", threads=1, axes=(-1,)):
            self.direction, self.axes = direction, axes
            self.output_shape = b.shape

        def __call__(self, input_array=None, output_array=None, normalise_idft=True):
            if self.direction == "FFTW_FORWARD":
                output_array[...] = sfft.fftn(input_array, axes=self.axes)
            else:
                output_array[...] = sfft.ifftn(input_array, axes=self.axes)
            return output_array

    fw.FFTW = FFTW
    sys.modules["pyfftw"] = fw

    cp = types.ModuleType("cupy")
    cp.ndarray = _CpArray
    cp.asarray = lambda x, dtype=None: np.asarray(x, dtype=dtype).view(_CpArray)
    cp.array = lambda x, dtype=None: np.array(x, dtype=dtype).view(_CpArray)
    cp.zeros_like = lambda a, dtype=None: np.zeros_like(np.asarray(a), dtype=dtype).view(_CpArray)
    cp.empty_like = lambda a, dtype=None: np.zeros_like(np.asarray(a), dtype=dtype).view(_CpArray)
    cp.ones = lambda *a, **k: np.ones(*a, **k).view(_CpArray)
    cp.zeros = lambda *a, **k: np.zeros(*a, **k).view(_CpArray)

    def fuse(*a, **k):
        if a and callable(a[0]):
            return a[0]
        return lambda f: f

    cp.fuse = fuse
    for name in ("exp", "abs", "angle", "multiply", "max", "allclose", "sqrt"):
        setattr(cp, name, getattr(np, name))

    # Inside cp.fuse a Python-scalar expression such as cos(omega * dz) stays a
    # weakly typed scalar and rounds to the array precision when it meets an
    # array (rabi_coupling); np.cos would return a strongly typed float64.
    def _weak(f):
        def g(x, *a, **k):
            if np.ndim(x) == 0 and not a and not k:
                y = f(x)
                return complex(y) if np.iscomplexobj(y) else float(y)
            return f(x, *a, **k)
        return g

    cp.cos = _weak(np.cos)
    cp.sin = _weak(np.sin)
    cp.newaxis = np.newaxis
    cp.random = np.random

    class _Event:
        def record(self):
            pass

        def synchronize(self):
            pass

    cp.cuda = types.SimpleNamespace(Event=_Event, get_elapsed_time=lambda a, b: 0.0,
                                    get_current_stream=lambda: None)
    sys.modules["cupy"] = cp

    cx = types.ModuleType("cupyx")
    cxs = types.ModuleType("cupyx.scipy")
    cxss = types.ModuleType("cupyx.scipy.signal")
    cxss.oaconvolve = ssig.oaconvolve
    cx.scipy = cxs
    cxs.signal = cxss
    sys.modules["cupyx"] = cx
    sys.modules["cupyx.scipy"] = cxs
    sys.modules["cupyx.scipy.signal"] = cxss

    pv = types.ModuleType("pyvkfft")
    pvc = types.ModuleType("pyvkfft.cuda")

    class VkFFTApp:
        def __init__(self, shape, dtype, ndim=2, stream=None, inplace=True, norm=1, tune=False):
            self.shape0 = tuple(shape[-ndim:])
            self.axes = tuple(range(-ndim, 0))

        def fft(self, src, dst):
            dst[...] = sfft.fftn(src, axes=self.axes)

        def ifft(self, src, dst):
            dst[...] = sfft.ifftn(src, axes=self.axes)

    pvc.VkFFTApp = VkFFTApp
    pv.cuda = pvc
    sys.modules["pyvkfft"] = pv
    sys.modules["pyvkfft.cuda"] = pvc


def load_reference(root: Path | None = None):
    _install_shims()
    sys.path.insert(0, str(root if root is not None else _reference_root()))
    import NLSE  # noqa: N811  (the reference package)

    return NLSE


# ---------------------------------------------------------------------------
# cases
# ---------------------------------------------------------------------------
WAIST, WAIST2, POWER, N2, ISAT, ALPHA, L = 2.23e-3, 70e-6, 1.05, -1.6e-9, 1e5, 20, 10e-3
WINDOW = 4 * WAIST


def gauss(XX, YY, w=WAIST):
    return np.exp(-(XX**2 + YY**2) / w**2)


def well(XX, YY):
    return -1e-4 * np.exp(-(XX**2 + YY**2) / WAIST2**2)


class Counter:
    def __init__(self):
        self.n = 0

    def __call__(self, simu, A, z, i):
        self.n = i + 1


def save(name, **arrays):
    np.savez_compressed(OUT / f"{name}.npz", **arrays)
    print(f"  {name}: " + ", ".join(f"{k}{np.shape(v)}" for k, v in arrays.items()))


def run_nlse2d(R, name, N, dtype, precision, noise=0.0, with_v=True, dz=5e-5, NY=None,
               batch=None, nl_length=0, backend="GPU", z=L, seed=0):
    NY = NY or N
    window = WINDOW if NY == N else [WINDOW, WINDOW * NY / N]
    n2, power = N2, POWER
    if batch:
        n2 = np.linspace(-1.6e-9, -4e-10, batch).reshape(batch, 1, 1)
        power = np.linspace(0.5, 2.0, batch)
    sim = R.NLSE(ALPHA, power, window, n2, None, L, NX=N, NY=NY, Isat=ISAT,
                 nl_length=nl_length, backend=backend)
    sim.delta_z = dz
    E = gauss(sim.XX, sim.YY).astype(np.complex128)
    if batch:
        E = np.broadcast_to(E, (batch, NY, N)).copy()
    if noise:
        rng = np.random.default_rng(seed)
        E = E * (1 + noise * (rng.standard_normal(E.shape) + 1j * rng.standard_normal(E.shape)))
    E = E.astype(dtype)
    V = well(sim.XX, sim.YY).astype(np.complex64) if with_v else None
    sim.V = None if V is None else V.copy()
    cnt = Counter()
    out = sim.out_field(E, z, precision=precision, verbose=False, callback=cnt)
    save(name, E_in=E, V=np.zeros(0) if V is None else V, out=out,
         meta=np.array([N, NY, dz, z, cnt.n, nl_length]), n2=np.asarray(n2),
         power=np.asarray(power), precision=np.array(precision))


def run_callbacks(R, name, N, dtype, precision, batch=None, adapt_every=0, every=4, z=2e-3,
                  dz=5e-5):
    """out_field with the reference's own callbacks: sample + evaluate_delta_n +
    norm every `every` steps, or sample + adapt_delta_z every `adapt_every`
    steps (sample first, so the samples hold the field each update saw)."""
    from NLSE import callbacks as rcb

    n2, power = N2, POWER
    if batch:
        n2 = np.linspace(-1.6e-9, -4e-10, batch).reshape(batch, 1, 1)
        power = np.linspace(0.5, 2.0, batch)
    sim = R.NLSE(ALPHA, power, WINDOW, n2, None, L, NX=N, NY=N, Isat=ISAT, backend="GPU")
    sim.delta_z = dz
    E = gauss(sim.XX, sim.YY).astype(np.complex128)
    if batch:
        E = np.broadcast_to(E, (batch, N, N)).copy()
    E = E.astype(dtype)
    sim.V = well(sim.XX, sim.YY).astype(np.complex64)
    cnt = Counter()
    if adapt_every:
        nrec = 64
        samples = np.zeros((nrec,) + E.shape, dtype=dtype)
        dzs = []
        out = sim.out_field(E, z, precision=precision, verbose=False,
                            callback=[rcb.sample, rcb.adapt_delta_z, cnt],
                            callback_args=[(adapt_every, samples), (adapt_every, dzs), ()])
        nrec = (cnt.n - 1) // adapt_every + 1
        save(name, E_in=E, V=sim.V, out=out, samples=samples[:nrec], dzs=np.array(dzs),
             meta=np.array([N, dz, z, cnt.n, adapt_every, sim.k]), n2=np.asarray(n2),
             power=np.asarray(power), precision=np.array(precision))
        return
    nrec = (int(round(z / dz)) + every) // every + 1
    samples = np.zeros((nrec,) + E.shape, dtype=dtype)
    rdt = np.float64 if (batch or dtype == np.complex128) else np.float32
    dn = np.zeros((nrec,) + E.shape, dtype=rdt)
    norms = np.zeros(nrec)
    out = sim.out_field(E, z, precision=precision, verbose=False,
                        callback=[rcb.sample, rcb.evaluate_delta_n, rcb.norm, cnt],
                        callback_args=[(every, samples), (every, dn), (every, norms), ()])
    nrec = (cnt.n - 1) // every + 1
    save(name, E_in=E, V=sim.V, out=out, samples=samples[:nrec], delta_n=dn[:nrec],
         norms=norms[:nrec], meta=np.array([N, dz, z, cnt.n, every, sim.k]), n2=np.asarray(n2),
         power=np.asarray(power), precision=np.array(precision))


def run_cnlse1d(R, name, dtype, precision):
    sim = R.CNLSE_1d(ALPHA, POWER, WINDOW, N2, -1e-10, None, L, NX=128, Isat=ISAT,
                     backend="GPU")
    sim.delta_z = 5e-5
    sim.power2 = 10e-3
    E = np.array([gauss(sim.X, 0), gauss(sim.X, 0, WAIST / 3)]).astype(dtype)
    out = sim.out_field(E, L, precision=precision, verbose=False)
    save(name, E_in=E, out=out, meta=np.array([128, 5e-5, L]))


def run_gpe(R, name, dtype, precision):
    from scipy.constants import atomic_mass

    sim = R.GPE(gamma=0.5, N=2e5, window=40e-6, g=1e3 / 2e5 * 1e-12, V=None,
                m=87 * atomic_mass, NX=32, NY=32, sat=1e15, backend="GPU")
    sim.delta_z = 1e-5
    sim.delta_t = 1e-5
    E = np.exp(-(sim.XX**2 + sim.YY**2) / (5e-6) ** 2).astype(dtype)
    out = sim.out_field(E, 2e-4, precision=precision, verbose=False)
    save(name, E_in=E, out=out, meta=np.array([32, 1e-5, 2e-4]))


def run_cnlse_nonlocal(R, name, dtype, precision):
    """CNLSE with a Gaussian nonlocal kernel (the 1024^2 coupled configuration's
    physics at 64^2; the kernel set through nl_profile, sigma 100 um)."""
    sim = R.CNLSE(ALPHA, 0.5, WINDOW, N2, -0.8e-9, None, 20e-3, NX=64, NY=64, Isat=ISAT,
                  nl_length=100e-6, backend="GPU")
    r = np.arange(-10, 11) * sim.delta_X
    kern = np.exp(-(r[:, None] ** 2 + r[None, :] ** 2) / (2 * (100e-6) ** 2))
    kern = kern / kern.sum()
    sim.nl_profile = kern
    sim.delta_z = 5e-5
    sim.power2 = 0.05
    sim.n22 = -1.6e-9
    E = np.array([gauss(sim.XX, sim.YY, 1.5e-3), gauss(sim.XX, sim.YY, 0.5e-3)]).astype(dtype)
    out = sim.out_field(E, 2e-3, precision=precision, verbose=False)
    save(name, E_in=E, out=out, nl_profile=kern, meta=np.array([64, 5e-5, 2e-3]))


def main() -> None:
    import os
    import tempfile

    # the reference's CPU path writes an FFTW wisdom file into the working directory
    ref = _reference_root().resolve()
    os.chdir(tempfile.mkdtemp(prefix="nlse_golden_"))
    R = load_reference(ref)
    print(f"reference NLSE {R.__version__} from {ref}")
    # NLSE 2-D: the benchmark physics at 64^2
    run_nlse2d(R, "nlse2d_c64_single", 64, np.complex64, "single")
    run_nlse2d(R, "nlse2d_c128_double", 64, np.complex128, "double")
    run_nlse2d(R, "nlse2d_c64_double", 64, np.complex64, "double")
    run_nlse2d(R, "nlse2d_c128_single", 64, np.complex128, "single")
    run_nlse2d(R, "nlse2d_c64_noise_noV", 64, np.complex64, "single", noise=0.01, with_v=False,
               dz=2e-5)
    run_nlse2d(R, "nlse2d_c128_noise_noV_double", 64, np.complex128, "double", noise=0.01,
               with_v=False, dz=2e-5)
    run_nlse2d(R, "nlse2d_c64_rect", 64, np.complex64, "single", NY=32)
    run_nlse2d(R, "nlse2d_c64_batch3", 32, np.complex64, "single", batch=3)
    run_nlse2d(R, "nlse2d_c64_beyond_L", 32, np.complex64, "single", z=1.5 * L)
    run_nlse2d(R, "nlse2d_c64_nonlocal", 64, np.complex64, "single", nl_length=300e-6,
               dz=1e-4)
    run_nlse2d(R, "nlse2d_c128_nonlocal_double", 64, np.complex128, "double", nl_length=300e-6,
               dz=1e-4)
    # the reference's callbacks (NLSE/callbacks.py) inside out_field
    run_callbacks(R, "callbacks_c64_delta_n", 32, np.complex64, "single")
    run_callbacks(R, "callbacks_c64_batch_delta_n", 32, np.complex64, "single", batch=3)
    run_callbacks(R, "callbacks_c128_delta_n", 32, np.complex128, "double")
    run_callbacks(R, "callbacks_c64_adapt", 32, np.complex64, "single", adapt_every=4)
    run_callbacks(R, "callbacks_c128_adapt", 32, np.complex128, "single", adapt_every=3)

    # the reference's CPU path (numba kernels run as Python loops: tiny case)
    run_nlse2d(R, "nlse2d_cpu_c128_single", 16, np.complex128, "single", backend="CPU", dz=1e-3)

    # NLSE_1d
    for dt, prec, tag in ((np.complex64, "single", "c64_single"),
                          (np.complex128, "double", "c128_double")):
        sim = R.NLSE_1d(ALPHA, POWER, WINDOW, N2, None, L, NX=256, Isat=ISAT, backend="GPU")
        sim.delta_z = 5e-5
        E = np.stack([gauss(sim.X, 0), gauss(sim.X, 0, w=WAIST / 2)]).astype(dt)
        sim.V = well(sim.X, 0).astype(np.complex64)
        out = sim.out_field(E, L, precision=prec, verbose=False)
        save(f"nlse1d_{tag}", E_in=E, V=sim.V, out=out, meta=np.array([256, 5e-5, L]))

    # NLSE_3d (x, y, t)
    for dt, prec, tag in ((np.complex64, "single", "c64_single"),
                          (np.complex128, "double", "c128_double")):
        sim = R.NLSE_3d(alpha=ALPHA, energy=1.05 * 2e-6, window=np.array([WINDOW, 16e-6]),
                        n2=N2, D0=1e-16, vg=3e7, V=None, L=L, NX=16, NY=16, NZ=8, Isat=ISAT,
                        backend="GPU")
        sim.delta_z = 2.5e-4
        E = (np.exp(-(sim.XX**2 + sim.YY**2) / WAIST**2) * np.exp(-(sim.TT**2) / (2e-6) ** 2)
             ).astype(dt)
        out = sim.out_field(E, L, precision=prec, verbose=False)
        save(f"nlse3d_{tag}", E_in=E, out=out, meta=np.array([16, 16, 8, 2.5e-4, L]))

    # CNLSE with Rabi coupling and a potential
    for dt, prec, tag, omega in ((np.complex64, "single", "c64_single_rabi", 2e3),
                                 (np.complex128, "double", "c128_double", None),
                                 (np.complex128, "single", "c128_single_rabi", 2e3)):
        sim = R.CNLSE(ALPHA, 0.5, WINDOW, N2, -0.8e-9, None, 20e-3, NX=32, NY=32, Isat=ISAT,
                      omega=omega, backend="GPU")
        sim.delta_z = 5e-5
        sim.power2 = 0.05
        sim.n22 = -1.2e-9
        sim.k2 = 2 * np.pi / 795e-9
        sim.V = well(sim.XX, sim.YY).astype(np.complex64)
        E = np.array([gauss(sim.XX, sim.YY, 1.5e-3), gauss(sim.XX, sim.YY, 0.5e-3)]).astype(dt)
        out = sim.out_field(E, 20e-3, precision=prec, verbose=False)
        save(f"cnlse_{tag}", E_in=E, V=sim.V, out=out,
             meta=np.array([32, 5e-5, 20e-3, -1 if omega is None else omega]))

    # CNLSE_1d and GPE, complex64 "single" and complex128 "double"
    run_cnlse1d(R, "cnlse1d_c64_single", np.complex64, "single")
    run_cnlse1d(R, "cnlse1d_c128_double", np.complex128, "double")
    run_gpe(R, "gpe_c64_single", np.complex64, "single")
    run_gpe(R, "gpe_c128_double", np.complex128, "double")
    run_cnlse_nonlocal(R, "cnlsenl_c64_single", np.complex64, "single")
    run_cnlse_nonlocal(R, "cnlsenl_c128_double", np.complex128, "double")

    # DDGPE with the pump as callback 0 (and the branch-specific arguments)
    for prec, with_v, tag in (("single", False, "single_noV"), ("single", True, "single_V"),
                              ("double", False, "double_noV"), ("double", True, "double_V")):
        h = 0.654  # meV ps
        sim = R.DDGPE(gamma=0.07 / h, power=1.0, window=64.0, g=1e-2 / h, omega=5.07 / h,
                      T=2.0, omega_exc=1484.44 / h, omega_cav=1482.76 / h,
                      detuning=0.17 / h, k_z=27.0, NX=32, NY=32, backend="GPU")
        sim.delta_z = 0.1 / 32
        t = np.arange(0, 2.0 + sim.delta_z, step=sim.delta_z, dtype=np.float32)
        E0 = np.zeros((2, 32, 32), dtype=np.complex64)
        rng = np.random.default_rng(3)
        E0 += (0.01 * (rng.standard_normal(E0.shape) + 1j * rng.standard_normal(E0.shape))
               ).astype(np.complex64)
        Fr = (2.0 * np.exp(-((sim.XX**2 + sim.YY**2) / 20.0**2))).astype(np.complex64)
        Ft = np.clip(t / 1.0, 0, 1).astype(np.complex64)
        Pr = (0.1 * np.exp(-((sim.XX - 5) ** 2 + sim.YY**2) / 4.0**2)).astype(np.complex64)
        Pt = np.exp(-((t - 1.0) ** 2) / 0.1).astype(np.complex64)
        if with_v:
            sim.V = (0.5 * np.exp(-(sim.XX**2 + sim.YY**2) / 10.0**2)).astype(np.complex64)
        final = {}

        def grab(simu, A, z, i):
            final["A"] = np.array(A, copy=True)
            final["n"] = i + 1

        sim.out_field(E0, 2.0, sim.laser_excitation, precision=prec, verbose=False,
                      callback=[grab], callback_args=[[Fr, Ft, Pr, Pt], []])
        save(f"ddgpe_c64_{tag}", E_in=E0, Fr=Fr, Ft=Ft, Pr=Pr, Pt=Pt,
             V=np.zeros(0) if sim.V is None else np.asarray(sim.V), out=final["A"],
             meta=np.array([32, 0.1 / 32, 2.0, final["n"]]))

    # elementwise kernels of the GPU path on random inputs
    from NLSE import kernels_gpu as kg

    rng = np.random.default_rng(11)
    for dt in (np.complex64, np.complex128):
        tag = "c64" if dt == np.complex64 else "c128"
        rdt = np.float32 if dt == np.complex64 else np.float64
        A = (rng.standard_normal((3, 17, 16)) + 1j * rng.standard_normal((3, 17, 16))).astype(dt)
        B = (rng.standard_normal((3, 17, 16)) + 1j * rng.standard_normal((3, 17, 16))).astype(dt)
        V = (1e-3 * (rng.standard_normal((17, 16)) + 1j * rng.standard_normal((17, 16)))
             ).astype(np.complex64)
        sq_a = np.abs(A) ** 2
        sq_b = np.abs(B) ** 2
        o1 = A.copy()
        kg.nl_prop(o1, sq_a.astype(rdt), 0.3, 0.7, 5.0 * V, 2.5, 1.7)
        o2 = A.copy()
        kg.nl_prop_without_V(o2, sq_a.astype(rdt), 0.3, 0.7, 2.5, 1.7)
        o3 = A.copy()
        kg.nl_prop_c(o3, sq_a.astype(rdt), sq_b.astype(rdt), 0.3, 0.7, 5.0 * V, 2.5, -1.5, 1.7,
                     0.9)
        o4 = A.copy()
        kg.nl_prop_without_V_c(o4, sq_a.astype(rdt), sq_b.astype(rdt), 0.3, 0.7, 2.5, -1.5, 1.7,
                               0.9)
        r1, r2 = A.copy(), B.copy()
        kg.rabi_coupling(r1, r2, 0.3, 1.3)
        save(f"kernels_{tag}", A=A, B=B, V=V, nl_prop=o1, nl_prop_without_V=o2, nl_prop_c=o3,
             nl_prop_without_V_c=o4, rabi1=r1, rabi2=r2, square_mod=sq_a.astype(rdt))

    # step counts of the z-loop for the benchmark configurations (no field needed)
    counts = []
    for z, dz in ((10e-3, 5e-5), (10e-3, 2e-5), (20e-3, 5e-5), (1e-3, 1e-5), (2e-3, 1e-4)):
        zp, n = 0, 0
        while abs(zp) < z:
            zp += dz
            n += 1
        counts.append((z, dz, n))
    save("step_counts", counts=np.array(counts))


if __name__ == "__main__":
    main()
