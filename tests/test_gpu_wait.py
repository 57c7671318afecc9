"""Bounded waits give up, report and leave the context usable (no GPU fault).

nlse_wait_selftest waits on an mbarrier that nothing completes, with the
loop every wait of the passes uses, and a short limit; the device timeout
code must reach the status word, the wait must have lasted its limit, and
the next propagation must still match the oracle (complex128, 1e-12).
"""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import nlse_gb300 as ng  # noqa: E402
from nlse_gb300 import _lib  # noqa: E402
from oracle import nlse_oracle as orc  # noqa: E402
from tests import cases  # noqa: E402

DEV_WAIT_TIMEOUT = 1


def _stream():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_wait_gives_up_reports_and_the_context_stays_usable():
    lib = _lib.load()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    el = torch.zeros(1, dtype=torch.int64, device="cuda")
    limit = 20_000_000  # 20 ms
    _lib.check(lib.nlse_wait_selftest(st.data_ptr(), el.data_ptr(), limit, _stream()),
               "wait selftest")
    torch.cuda.synchronize()
    assert int(st.item()) == DEV_WAIT_TIMEOUT
    assert limit <= int(el.item()) < limit + 200_000_000
    p, o, E = cases.oracle_pair(ng.NLSE, orc.OracleNLSE, 64, dtype=np.complex128)
    got = p.out_field(E, 2e-3, verbose=False)
    ref, _ = o.out_field(E, 2e-3)
    assert cases.rel_l2(got, ref) <= 1e-12


@pytest.mark.parametrize("limit", [0, -5, 2_000_000_000])
def test_wait_limit_is_checked(limit):
    lib = _lib.load()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    el = torch.zeros(1, dtype=torch.int64, device="cuda")
    assert lib.nlse_wait_selftest(st.data_ptr(), el.data_ptr(), limit, _stream()) == -1
    assert int(st.item()) == 0
