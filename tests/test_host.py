"""Host-side logic of nlse_gb300 and the C ABI surface (no GPU needed)."""

import ctypes as ct
import re
from pathlib import Path

import numpy as np
import pytest
from scipy.constants import c, epsilon_0

import nlse_gb300 as ng
from nlse_gb300 import _build, _lib, engine
from oracle import nlse_oracle as orc
from tests import cases

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "nlse_gb300.h"


def _declared_symbols():
    text = "\n".join(h.read_text() for h in sorted(HEADER.parent.glob("*.h")))
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char\*|void)\s+(nlse_\w+)\(", text,
                                 re.M)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    syms = _declared_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s
    assert {s for s, _, _ in _lib.SIGNATURES} == set(syms)


def test_abi_version_and_error_reporting(lib):
    assert lib.nlse_abi_version() == 2
    h = ct.c_void_p()
    d = _lib.Desc()
    d.ndim = 2
    d.shape[0], d.shape[1] = 100, 64  # not a power of two
    d.nfields, d.comps, d.dtype = 1, 1, 0
    d.ndim = 4
    assert lib.nlse_plan_create(ct.byref(h), ct.byref(d)) == _lib.ERR_ARG
    assert lib.nlse_power_workspace_size(3, 4096) == 3 * 8
    assert lib.nlse_power(None, 0, 1, 1, None, None, 0, None) == _lib.ERR_ARG


def test_backend_is_gpu_only():
    with pytest.raises(ValueError):
        ng.NLSE(20, 1.05, 1e-2, -1e-9, None, 1e-2, NX=8, NY=8, backend="CPU")
    with pytest.raises(ValueError):
        ng.NLSE(20, 1.05, 1e-2, -1e-9, None, 1e-2, NX=8, NY=8, backend="XYZ")


@pytest.mark.parametrize("N", [64, 2048])
def test_build_propagator_closed_forms(N):
    """The reference's propagator KATs (tests/test_nlse.py:32-50 and per class)."""
    s = ng.NLSE(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N, NY=N,
                Isat=cases.ISAT)
    p = s._build_propagator()
    assert p.dtype == np.complex64
    assert np.allclose(p, np.exp(-1j * 0.5 * (s.Kxx**2 + s.Kyy**2) / s.k * s.delta_z))
    o = orc.OracleNLSE(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N,
                       NY=N, Isat=cases.ISAT)
    np.testing.assert_array_equal(p, o.build_propagator())
    s1 = ng.NLSE_1d(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, None, cases.L, NX=N)
    p1 = s1._build_propagator()
    assert p1.dtype == np.complex128
    assert np.allclose(p1, np.exp(-1j * 0.5 * s1.Kx**2 / s1.k * s1.delta_z))
    cn = ng.CNLSE(cases.ALPHA, cases.POWER, cases.WINDOW, cases.N2, -1e-10, None, cases.L,
                  NX=N, NY=N)
    cn.k2 = 2 * np.pi / 795e-9
    pc = cn._build_propagator()
    assert pc.shape == (2, N, N)
    assert np.allclose(pc[1], np.exp(-1j * 0.5 * (cn.Kxx**2 + cn.Kyy**2) / cn.k2 * cn.delta_z))


def test_nlse3d_and_gpe_and_ddgpe_propagators():
    s = ng.NLSE_3d(alpha=20, energy=1.05 * 2e-6, window=np.array([8.92e-3, 16e-6]), n2=-1.6e-9,
                   D0=1e-16, vg=3e7, V=None, L=1e-2, NX=16, NY=16, NZ=8, Isat=1e5)
    p = s._build_propagator()
    th = np.exp(-1j * 0.5 * (s.Kxx**2 + s.Kyy**2) / s.k * s.delta_z)
    th = th * np.exp(-1j * s.D0 / 2 * s.Omega**2)
    assert p.shape == (16, 16, 8) and p.dtype == np.complex128 and np.allclose(p, th)
    from scipy.constants import hbar

    g = ng.GPE(gamma=0, N=2e5, window=40e-6, g=1e-20, V=None, NX=32, NY=32)
    g.delta_t = 1e-7
    pg = g._build_propagator()
    assert np.allclose(pg, np.exp(-1j * 0.5 * hbar * (g.Kxx**2 + g.Kyy**2) / g.m * 1e-7))
    h = 0.654
    d = ng.DDGPE(0.07 / h, 1.0, 64.0, 1e-2 / h, 5.07 / h, 2.0, 1484.44 / h, 1482.76 / h,
                 0.17 / h, 27.0, NX=16, NY=16)
    pd = d._build_propagator()
    assert np.allclose(pd[0], np.exp(-1j * (d.omega_exc - d.omega_pump) * d.delta_z))


def test_default_delta_z_and_grid_match_oracle():
    for N in (32, 256):
        s = ng.NLSE(20, 1.05, 8.92e-3, -1.6e-9, None, 1e-2, NX=N, NY=N)
        o = orc.OracleNLSE(20, 1.05, 8.92e-3, -1.6e-9, None, 1e-2, NX=N, NY=N)
        assert s.delta_z == o.delta_z
        np.testing.assert_array_equal(s.XX, o.XX)
        assert s.delta_X == o.delta_X


def test_count_steps_matches_reference_loop():
    assert ng.count_steps(10e-3, 5e-5) == 201
    assert ng.count_steps(10e-3, 2e-5) == 501
    assert ng.count_steps(20e-3, 5e-5) == 400
    assert ng.count_steps(0, 5e-5) == 0
    for z, dz in ((1e-3, 1e-5), (2e-3, 1e-4), (3.3e-3, 7e-5)):
        assert ng.count_steps(z, dz) == orc.count_steps(z, dz)


def test_per_field_broadcasting():
    assert engine.per_field(2.0, (3,), 2, "x").tolist() == [2.0, 2.0, 2.0]
    v = engine.per_field(np.arange(3.0).reshape(3, 1, 1), (3,), 2, "x")
    assert v.tolist() == [0.0, 1.0, 2.0]
    assert engine.per_field(np.arange(4.0), (4,), 0, "power").tolist() == [0, 1, 2, 3]
    with pytest.raises(NotImplementedError):
        engine.per_field(np.ones((3, 8, 8)), (3,), 2, "n2")  # varies over the grid
    with pytest.raises(ValueError):
        engine.per_field(np.ones((2, 1, 1)), (3,), 2, "n2")


def test_grid_varying_coefficients_become_planes():
    """n2, alpha and Isat arrays over the grid (the reference broadcasts them in
    nl_prop) become per-pixel planes g, alpha/2, 1/Isat'; per-field and scalar
    ones stay in the parameter block."""
    import torch

    assert not engine.varies_on_grid(np.ones((3, 1, 1)), 2)
    assert engine.varies_on_grid(np.ones((16,)), 2)          # broadcasts along x
    assert engine.varies_on_grid(np.ones((16, 1)), 2)        # along y
    assert engine.coef_plane(np.arange(4.0), (3,), (2, 4)).shape == (1, 8)
    assert engine.coef_plane(np.ones((3, 2, 4)), (3,), (2, 4)).shape == (3, 8)
    N = 16
    n2map = -1.6e-9 * (1 + 0.1 * np.arange(N * N).reshape(N, N) / (N * N))
    isat = np.full((N, N), 1e5)
    isat[:, : N // 2] = 2e5
    # (a grid-shaped n2 with a (B,) power does not broadcast in the reference's
    # default-step expression either; the power stays scalar here)
    s = ng.NLSE(20, 1.0, 8.92e-3, n2map, None, 1e-2, NX=N, NY=N, Isat=isat)
    s.alpha = np.full((2, 1, 1), 20.0)                        # per field: stays in the block
    s.delta_z = 5e-5
    P = s._nl_block((2,), "single", False)
    assert np.all(P[:, 1] == 10.0) and np.all(P[:, 4] == np.inf) and np.all(P[:, 2] == 0.0)
    maps, mask = s._coef_planes((2,), (N, N), torch.float64, "cpu")
    assert mask == 0b101 and tuple(maps.shape) == (3, 1, N * N)
    g = s.k / 2 * n2map * c * epsilon_0
    np.testing.assert_array_equal(maps[0, 0].numpy(), g.reshape(-1))
    np.testing.assert_array_equal(maps[2, 0].numpy(), (1 / (2 * isat / (epsilon_0 * c))).reshape(-1))
    # two-component fields keep the error
    cn = ng.CNLSE(20, 1.0, 8.92e-3, n2map, -1e-10, None, 1e-2, NX=N, NY=N, Isat=1e5)
    with pytest.raises(NotImplementedError):
        cn._nl_block((), "single", False)


def test_nlse_parameter_block_formulas():
    s = ng.NLSE(20, 1.05, 8.92e-3, -1.6e-9, None, 1e-2, NX=16, NY=16, Isat=1e5)
    s.delta_z = 5e-5
    P = s._nl_block((), "single", True)
    assert P.shape == (1, _lib.NLSE_PARAM_STRIDE)
    assert P[0, 0] == 5e-5 and P[0, 1] == 10.0
    assert P[0, 2] == s.k / 2 * s.n2 * c * epsilon_0
    assert P[0, 4] == 2 * s.I_sat / (epsilon_0 * c) and np.isinf(P[0, 5])
    assert P[0, 6] == s.k / 2
    D = s._nl_block((), "double", True)
    assert D[0, 0] == 2.5e-5 and D[0, 16] == 2.5e-5


def test_ddgpe_parameter_block_follows_branch_arguments():
    h = 0.654
    d = ng.DDGPE(0.07 / h, 1.0, 64.0, 1e-2 / h, 5.07 / h, 2.0, 1484.44 / h, 1482.76 / h,
                 0.17 / h, 27.0, NX=16, NY=16)
    d.delta_z = 0.01
    P = d._nl_block((), "single", False)
    assert P[0, 1] == d.alpha / 2 and P[0, 8] == d.gamma2 / 2 and P[0, 9] == d.g2
    assert P[0, 11] == d.I_sat and P[0, 12] == d.I_sat2
    assert np.isclose(P[0, 14], np.cos(d.omega / 2 * 0.01)) and P[0, 30] == 0.01
    D = d._nl_block((), "double", True)
    assert D[0, 16] == 0.01 and D[0, 22] == 1.0  # before the linear step: full dz, raw V
    assert D[0, 6] == d.k / 2 and D[0, 13] == 1.0  # after: k/2*V on the exciton only
    D = d._nl_block((), "double", False)
    assert D[0, 9] == d.g  # both components use g in this branch


def test_cnlse_parameter_block():
    cn = ng.CNLSE(20, 0.5, 8.92e-3, -1.6e-9, -0.8e-9, None, 2e-2, NX=16, NY=16, Isat=1e5,
                  omega=2e3)
    cn.n22 = -1.2e-9
    cn.k2 = 2 * np.pi / 795e-9
    P = cn._nl_block((), "single", False)
    assert P[0, 3] == cn.k / 2 * cn.n12 * c * epsilon_0
    assert P[0, 9] == cn.k2 / 2 * cn.n22 * c * epsilon_0
    assert P[0, 10] == cn.k2 / 2 * cn.n12 * c * epsilon_0
    assert P[0, 13] == cn.k2 / 2
    assert np.isclose(P[0, 15], np.sin(1e3 * cn.delta_z))
    assert cn._rabi_enabled("single") and not cn._rabi_enabled("double")


def _arg_error_cases(lib):
    z = ct.c_void_p(None)
    fake = ct.c_void_p(16)  # never dereferenced: every call below fails its argument check first
    return [
        ("add_noise null field", lambda: lib.nlse_add_noise(z, 0, 1, 16, 0.1, 0.1, 1, 0, z)),
        ("add_noise bad dtype", lambda: lib.nlse_add_noise(fake, 7, 1, 16, 0.1, 0.1, 1, 0, z)),
        ("add_noise negative step",
         lambda: lib.nlse_add_noise(fake, 0, 1, 16, 0.1, 0.1, 1, -1, z)),
        ("delta_n null coef", lambda: lib.nlse_delta_n(fake, 0, 1, 16, z, fake, 0, fake, z)),
        ("delta_n bad flags", lambda: lib.nlse_delta_n(fake, 0, 1, 16, fake, fake, 4, fake, z)),
        ("delta_n empty", lambda: lib.nlse_delta_n(fake, 0, 0, 16, fake, fake, 0, fake, z)),
        ("delta_n_max bad dtype",
         lambda: lib.nlse_delta_n_max(fake, 3, 1, 16, fake, fake, 1.0, 1.0, 0, fake, z)),
        ("wait_selftest zero limit", lambda: lib.nlse_wait_selftest(fake, fake, 0, z)),
        ("wait_selftest over 1 s", lambda: lib.nlse_wait_selftest(fake, fake, 2_000_000_000, z)),
        ("set_kernels null plan", lambda: lib.nlse_plan_set_kernels(z, 1, 1)),
        ("propagate null plan", lambda: lib.nlse_propagate(z, fake, None, 1, 0, 0, z)),
        ("pass null plan", lambda: lib.nlse_pass(z, fake, None, 0, 0, z)),
        ("normalize null", lambda: lib.nlse_normalize(z, z, 0, 1, 1, z, z, 1.0, z)),
        ("square_mod bad dtype", lambda: lib.nlse_square_mod(fake, fake, 9, 16, z)),
        ("fno_lift_rows empty batch",
         lambda: lib.nlse_fno_lift_rows(0, fake, fake, fake, fake, fake, fake, fake, z)),
        ("fno_mix empty batch", lambda: lib.nlse_fno_mix(0, fake, fake, fake, fake, z)),
        ("fno_loss empty batch", lambda: lib.nlse_fno_loss(0, fake, fake, fake, fake, fake, z)),
        # 32769 segments of 8193 elements need 65,538 partial sums: two over the static array
        ("power_noalloc over capacity",
         lambda: lib.nlse_power_noalloc(fake, 0, 32769, 8193, fake, z)),
        ("power_noalloc 1024 partials x 65 segments",
         lambda: lib.nlse_power_noalloc(fake, 0, 65, 1024 * 8192, fake, z)),
    ]


def test_entry_points_reject_bad_arguments_before_any_device_work(lib):
    for name, call in _arg_error_cases(lib):
        rc = call()
        assert rc == _lib.ERR_ARG, (name, rc, _lib.last_error())
        assert _lib.last_error(), name


def _declared_arities():
    """Parameter count of every nlse_* prototype in include/*.h."""
    text = "\n".join(h.read_text() for h in sorted(HEADER.parent.glob("*.h")))
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)  # comments out
    out = {}
    for m in re.finditer(r"(?:int|size_t|const char\s*\*|void)\s+(nlse_\w+)\s*\(([^)]*)\)\s*;",
                         text):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_the_header_prototypes():
    ar = _declared_arities()
    assert len(ar) >= 10
    for name, _, argtypes in _lib.SIGNATURES:
        assert ar[name] == len(argtypes), (name, ar[name], len(argtypes))


def test_ctypes_structs_have_the_c_layout(tmp_path):
    """nlse_desc and nlse_operator as gcc lays them out (include/nlse_gb300.h)
    against the ctypes structures the Python host passes."""
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = {"nlse_desc": _lib.Desc, "nlse_operator": _lib.Operator}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "nlse_gb300.h"',
             "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{HEADER.parent}", str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True,
                               text=True).stdout.splitlines():
        cname, fname, v = line.split()
        got[(cname, fname)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == ct.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_surrogate_constants_match_the_header():
    """nlse_gb300.fno's sizes against the #defines of include/nlse_fno.h."""
    from nlse_gb300 import fno

    text = (HEADER.parent / "nlse_fno.h").read_text()
    d = {k: int(v) for k, v in re.findall(r"#define NLSE_FNO_(\w+)\s+(\d+)", text)}
    assert (fno.N, fno.C, fno.NM) == (d["N"], d["C"], d["MODES"])
    assert (fno.PART_LAYER, fno.PART_PROJ, fno.PART_LIFT) == (
        d["PART_LAYER"], d["PART_PROJ"], d["PART_LIFT"])
    assert d["PART_LAYER"] == d["C"] * d["C"] + d["C"] and d["PART_PROJ"] == 2 * d["C"] + 2


def test_pipeline_split_policy():
    """Host pipeline chunks: first and last field alone, only for short loops
    of large enough batches."""
    from nlse_gb300.nlse import NLSE, pipeline_split

    mx, mn = NLSE.PIPELINE_MAX_STEPS, NLSE.PIPELINE_MIN_BYTES
    assert pipeline_split(8, 1 << 28, 20, mx, mn) == [0, 1, 7, 8]
    assert pipeline_split(4, 1 << 28, mx, mx, mn) == [0, 1, 3, 4]
    assert pipeline_split(3, 1 << 28, 20, mx, mn) == [0, 1, 3]
    assert pipeline_split(2, 1 << 28, 20, mx, mn) == [0, 1, 2]
    assert pipeline_split(1, 1 << 28, 20, mx, mn) is None
    assert pipeline_split(8, mn - 1, 20, mx, mn) is None
    assert pipeline_split(8, 1 << 28, mx + 1, mx, mn) is None
