"""Every golden fixture (fields computed by the reference's own code) replayed on the GPU."""

import numpy as np
import pytest

from nlse_gb300 import _lib

from tests import golden_cases as gc
from tests.cases import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SKIP = {
    # the reference's CPU-path kernels (unsaturated loss) are not the GPU path
    "nlse2d_cpu_c128_single": "CPU-path semantics",
}


@pytest.mark.parametrize("name", gc.FIXTURES)
def test_product_matches_reference_fixture(name):
    if name in SKIP:
        pytest.skip(SKIP[name])
    got = gc.run(name, "product")
    ref = gc.load(name)["out"]
    assert got.shape == ref.shape and got.dtype == ref.dtype
    if "c128" in name:
        err = rel_l2(got, ref)
        assert err <= gc.tolerance(name), err
    else:
        r = gc.c64_check(name, got)
        print(name, r)
        assert r["ok"], r


@pytest.mark.parametrize("name", gc.SHORT)
def test_product_matches_reference_at_20_steps(name):
    """complex64 against the reference's own complex64 result after 20 steps:
    rel-L2 <= 1e-5 (the reference's FFT spread there is ~1e-6)."""
    f = gc.load_short(name)
    got = gc.run(name, "product", steps=int(f["steps"]))
    ref = f["out"]
    assert got.shape == ref.shape and got.dtype == ref.dtype
    err = rel_l2(got, ref)
    spr = max(rel_l2(f["out_numpy"], ref), rel_l2(f["out_torch"], ref))
    print(f"{name} ({int(f['steps'])} steps): product vs reference {err:.2e}, "
          f"reference FFT spread {spr:.2e}")
    assert err <= 1e-5, err


@pytest.mark.parametrize("tag", ["c64", "c128"])
def test_elementwise_kernels_match_reference(tag):
    """nlse_nonlinear against kernels_gpu.nl_prop / nl_prop_c / rabi_coupling outputs."""
    import nlse_gb300 as ng  # noqa: F401
    from nlse_gb300 import engine
    from nlse_gb300.engine import OperatorData, Plan

    f = gc.load(f"kernels_{tag}")
    A, B, V = f["A"], f["B"], f["V"]
    dt = 0 if tag == "c64" else 1
    tol = 2e-6 if tag == "c64" else 1e-14
    dev = torch.device("cuda", 0)
    prop = torch.ones(1, dtype=torch.complex64, device=dev)

    def params(rows):
        P = np.zeros((A.shape[0], _lib.NLSE_PARAM_STRIDE))
        for k, row in rows.items():
            P[:, k:k + len(row)] = row
        return torch.from_numpy(P).to(dev)

    # nl_prop (one component): dz 0.3, alpha 0.7, V' = 5 V, g 2.5, Isat 1.7
    plan1 = Plan.get(2, (17, 16), 3, 1, dt, dev)
    for key, with_v in (("nl_prop", True), ("nl_prop_without_V", False)):
        a = torch.from_numpy(A.copy()).to(dev)
        op = OperatorData(prop=prop, params=params({0: [0.3, 0.7, 2.5, 0.0, 1.7, np.inf, 5.0]}),
                          scheme=0, V=torch.from_numpy(V).to(dev) if with_v else None)
        engine.nonlinear(plan1, a, op)
        assert rel_l2(a.cpu().numpy(), f[key]) < tol, key

    # nl_prop_c on component 0 of a two-component field (B as the partner)
    plan2 = Plan.get(2, (17, 16), 3, 2, dt, dev)
    for key, with_v in (("nl_prop_c", True), ("nl_prop_without_V_c", False)):
        ab = torch.from_numpy(np.stack([A, B], axis=1).copy()).to(dev)
        P = params({0: [0.3, 0.7, 2.5, -1.5, 1.7, 0.9, 5.0], 7: [0, 0, 0, 0, np.inf, np.inf, 0]})
        op = OperatorData(prop=prop, params=P, scheme=0,
                          V=torch.from_numpy(V).to(dev) if with_v else None)
        engine.nonlinear(plan2, ab, op)
        assert rel_l2(ab[:, 0].cpu().numpy(), f[key]) < tol, key

    # rabi_coupling(A1, A2, dz=0.3, omega=1.3): pure rotation (zero nonlinear step)
    ab = torch.from_numpy(np.stack([A, B], axis=1).copy()).to(dev)
    P = params({0: [0, 0, 0, 0, np.inf, np.inf, 0], 7: [0, 0, 0, 0, np.inf, np.inf, 0],
                14: [np.cos(1.3 * 0.3), np.sin(1.3 * 0.3)]})
    op = OperatorData(prop=prop, params=P, scheme=0, rabi=True)
    engine.nonlinear(plan2, ab, op)
    assert rel_l2(ab[:, 0].cpu().numpy(), f["rabi1"]) < tol
    assert rel_l2(ab[:, 1].cpu().numpy(), f["rabi2"]) < tol

    # square_mod
    sq = torch.empty(A.shape, dtype=torch.float32 if dt == 0 else torch.float64, device=dev)
    engine.square_mod(torch.from_numpy(A).to(dev), sq)
    assert np.allclose(sq.cpu().numpy(), f["square_mod"], rtol=1e-6 if dt == 0 else 1e-15)
