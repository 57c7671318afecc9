"""The allocation-free power sum (nlse_power_noalloc) against nlse_power.

nlse_power_noalloc serves callers that cannot allocate device memory (its
scratch is a static array inside the library).  It must give the same FP64
sums as nlse_power with a caller workspace, on consecutive calls that reuse
the shared array, and refuse requests larger than that array.  This file
runs last (pytest collects it after the others) and also passes alone in a
fresh process.
"""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _lib():
    from nlse_gb300 import _build, _lib

    _build.build()
    return _lib.load(), _lib


def _sums_with_workspace(lib, A, dtype, nseg, seg):
    out = torch.empty(nseg, dtype=torch.float64, device=A.device)
    wsb = lib.nlse_power_workspace_size(nseg, seg)
    ws = torch.empty(max(1, wsb // 8), dtype=torch.float64, device=A.device)
    rc = lib.nlse_power(ct.c_void_p(A.data_ptr()), dtype, nseg, seg, ct.c_void_p(out.data_ptr()),
                        ct.c_void_p(ws.data_ptr()), wsb,
                        ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    return out


def _sums_noalloc(lib, A, dtype, nseg, seg):
    out = torch.empty(nseg, dtype=torch.float64, device=A.device)
    rc = lib.nlse_power_noalloc(ct.c_void_p(A.data_ptr()), dtype, nseg, seg,
                                ct.c_void_p(out.data_ptr()),
                                ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.nlse_last_error()
    return out


@pytest.mark.parametrize("tdtype,code", [(torch.complex64, 0), (torch.complex128, 1)])
def test_noalloc_power_matches_workspace_power_on_consecutive_calls(tdtype, code):
    lib, _ = _lib()
    torch.cuda.set_device(0)
    g = torch.Generator(device="cuda").manual_seed(7)
    # two different calls in a row: the second reuses (and must overwrite) the static array
    for nseg, seg in ((6, 256 * 256 + 17), (3, 2048 * 2048)):
        A = torch.randn(nseg * seg, dtype=tdtype, device="cuda", generator=g)
        ref = _sums_with_workspace(lib, A, code, nseg, seg)
        got = _sums_noalloc(lib, A, code, nseg, seg)
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(), rtol=1e-13, atol=0)


def test_noalloc_power_rejects_requests_beyond_its_array():
    lib, L = _lib()
    A = torch.zeros(16, dtype=torch.complex64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # 65 segments x 1024 chunks each exceed the 65,536 partial sums; no kernel runs
    rc = lib.nlse_power_noalloc(ct.c_void_p(A.data_ptr()), 0, 65, 1024 * 8192,
                                ct.c_void_p(out.data_ptr()), None)
    assert rc == L.ERR_ARG
    assert "static array holds 65536" in L.last_error()
