"""evaluate_delta_n / adapt_delta_z on the GPU (NLSE/callbacks.py:57-112).

* nlse_delta_n and nlse_delta_n_max against the oracle on the same field:
  bit-exact (the kernels evaluate NumPy's expression operation by operation,
  in the precisions NumPy's promotion gives), for every parameter type.
* out_field with the callbacks against the reference's own records
  (tests/golden/callbacks_*.npz): index change, norms, samples, the adapted
  steps and the step count -- complex64 within 1e-4 (rel-L2; the fields
  differ by FFT rounding over the loop), complex128 within 1e-10.
* The device forms (graph nodes; segments between adaptive updates) against
  the per-step host loop (NLSE_DEVICE_CALLBACKS=0): identical when every step
  records, within 1e-5 when steps are fused.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import callbacks as cb  # noqa: E402
from nlse_gb300 import engine  # noqa: E402
from oracle import nlse_oracle as o  # noqa: E402
from scipy.constants import c, epsilon_0  # noqa: E402
from tests import golden_cases as gc  # noqa: E402
from tests.cases import rel_l2  # noqa: E402
from tests.test_callbacks_dn import CASES, _field  # noqa: E402


class _Simu:
    def __init__(self, n2, isat, na):
        self.n2, self.I_sat = n2, isat
        self._last_axes = tuple(range(-na, 0))


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_kernels_equal_oracle_bit_for_bit(case, dtype):
    n2, isat, shape, na = CASES[case]
    A = _field(shape, dtype, 100 + case)
    dA = torch.from_numpy(A).cuda()
    simu = _Simu(n2, isat, na)
    rec = []
    cb.evaluate_delta_n(simu, dA, 0.0, 0, 1, _Rec(rec))
    got = rec[0].cpu().numpy()
    ref = o.delta_n(A, n2, isat)
    assert got.dtype == ref.dtype and np.array_equal(got, ref)
    st = cb.index_change_setup(simu, dA, adapt=True)
    buf = torch.empty(1, dtype=torch.float64, device="cuda")
    engine.delta_n_max(dA, st[0], st[1], st[2], c, epsilon_0, st[3], buf)
    assert buf.item() == float(o.adapt_peak(A, n2, isat))


class _Rec:
    """A destination that keeps what the callback stores (device tensors)."""

    def __init__(self, out):
        self.out = out

    def __setitem__(self, idx, v):
        self.out.append(v)


def test_peak_propagates_nan():
    A = _field((16, 16), np.complex64, 7)
    A[3, 5] = np.nan
    dA = torch.from_numpy(A).cuda()
    st = cb.index_change_setup(_Simu(gc.N2, gc.ISAT, 2), dA, adapt=True)
    buf = torch.empty(1, dtype=torch.float64, device="cuda")
    engine.delta_n_max(dA, st[0], st[1], st[2], c, epsilon_0, st[3], buf)
    assert np.isnan(buf.item()) and np.isnan(o.adapt_peak(A, gc.N2, gc.ISAT))


def _sim(f, batch):
    N, dz = int(f["meta"][0]), float(f["meta"][1])
    n2 = f["n2"] if batch else gc.N2
    power = f["power"] if batch else gc.POWER
    sim = ng.NLSE(gc.ALPHA, power, gc.WINDOW, n2, None, gc.L, NX=N, NY=N, Isat=gc.ISAT)
    sim.delta_z = dz
    sim.V = f["V"].copy()
    return sim


@pytest.mark.parametrize("name", ["callbacks_c64_delta_n", "callbacks_c64_batch_delta_n",
                                  "callbacks_c128_delta_n"])
def test_delta_n_records_match_reference(name, monkeypatch):
    monkeypatch.setenv("NLSE_DEVICE_CALLBACKS", "1")
    f = gc.load(name)
    sim = _sim(f, "batch" in name)
    every, z = int(f["meta"][4]), float(f["meta"][2])
    nrec = f["delta_n"].shape[0]
    samples = np.zeros_like(f["samples"])
    dn = np.zeros_like(f["delta_n"])
    norms = np.zeros(nrec)
    out = sim.out_field(f["E_in"], z, precision=str(f["precision"]), verbose=False,
                        callback=[ng.sample, ng.evaluate_delta_n, ng.norm],
                        callback_args=[(every, samples), (every, dn), (every, norms)])
    tol = 1e-10 if "c128" in name else 1e-4
    assert rel_l2(out, f["out"]) <= tol
    assert rel_l2(samples, f["samples"]) <= tol
    assert rel_l2(dn, f["delta_n"]) <= tol
    np.testing.assert_allclose(norms, f["norms"], rtol=1e-12 if "c128" in name else 1e-5)
    # each record is the oracle's value of the recorded field, bit for bit
    n2 = f["n2"] if "batch" in name else gc.N2
    assert np.array_equal(dn, o.delta_n(samples, n2, gc.ISAT))


@pytest.mark.parametrize("name", ["callbacks_c64_adapt", "callbacks_c128_adapt"])
def test_adapted_steps_match_reference(name, monkeypatch):
    monkeypatch.setenv("NLSE_DEVICE_CALLBACKS", "1")
    f = gc.load(name)
    sim = _sim(f, False)
    u, z = int(f["meta"][4]), float(f["meta"][2])
    samples = np.zeros_like(f["samples"])
    dzs = []
    out = sim.out_field(f["E_in"], z, precision=str(f["precision"]), verbose=False,
                        callback=[ng.sample, ng.adapt_delta_z],
                        callback_args=[(u, samples), (u, dzs)])
    assert len(dzs) == len(f["dzs"])  # same step count
    tol = 1e-10 if "c128" in name else 1e-5
    np.testing.assert_allclose(np.array(dzs, dtype=np.float64), f["dzs"], rtol=tol)
    assert rel_l2(out, f["out"]) <= (1e-10 if "c128" in name else 1e-4)
    # every update is the oracle's step for the field it saw, bit for bit
    k = float(f["meta"][5])
    got = np.array(dzs[1::u])
    ref = [o.adapt_delta_z(s, gc.N2, gc.ISAT, k) for s in samples[:len(got)]]
    assert np.array_equal(got, np.array(ref))


def _loop(monkeypatch, device, every, u, dtype=np.complex64, N=64, z=3e-3):
    monkeypatch.setenv("NLSE_DEVICE_CALLBACKS", "1" if device else "0")
    sim = ng.NLSE(gc.ALPHA, gc.POWER, gc.WINDOW, gc.N2, None, gc.L, NX=N, NY=N, Isat=gc.ISAT)
    sim.delta_z = 5e-5
    sim.V = (-1e-4 * np.exp(-(sim.XX**2 + sim.YY**2) / gc.WAIST2**2)).astype(np.complex64)
    E = np.exp(-(sim.XX**2 + sim.YY**2) / gc.WAIST**2).astype(dtype)
    dn = np.zeros((64, N, N), np.float32 if dtype == np.complex64 else np.float64)
    norms = np.zeros(64)
    cbs, args = [ng.evaluate_delta_n, ng.norm], [(every, dn), (every, norms)]
    dzs = []
    if u:
        cbs.append(ng.adapt_delta_z)
        args.append((u, dzs))
    out = sim.out_field(E, z, verbose=False, callback=cbs, callback_args=args)
    return out, dn, norms, np.array(dzs, dtype=np.float64)


def test_device_records_equal_host_loop_step_by_step(monkeypatch):
    a = _loop(monkeypatch, True, 1, 0, z=1e-3)
    b = _loop(monkeypatch, False, 1, 0, z=1e-3)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_adaptive_segments_equal_host_loop(monkeypatch, dtype):
    a = _loop(monkeypatch, True, 3, 5, dtype)
    b = _loop(monkeypatch, False, 3, 5, dtype)
    assert len(a[3]) == len(b[3]) > 10
    tol = 1e-5 if dtype == np.complex64 else 1e-12
    np.testing.assert_allclose(a[3], b[3], rtol=tol)
    assert rel_l2(a[0], b[0]) <= tol
    assert rel_l2(a[1], b[1]) <= tol
    np.testing.assert_allclose(a[2], b[2], rtol=tol)
