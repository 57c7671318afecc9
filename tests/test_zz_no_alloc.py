"""The allocation-free power sum (nlse_power_noalloc) against nlse_power.

nlse_power_noalloc serves callers that cannot allocate device memory (its
scratch is a static array inside the library).  It must give the same FP64
sums as nlse_power with a caller workspace, on consecutive calls that reuse
the shared array, up to the array's exact capacity, and refuse requests
larger than that array.  It must not allocate device memory once warmed up,
and a call captured into a CUDA graph after the first one must replay to the
same sums.  This file runs last (pytest collects it after the others) and
also passes alone in a fresh process.
"""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CAPACITY = 65536  # partial sums the static array holds
CHUNK = 8192      # elements per partial sum (at most 1024 partials per segment)


def _lib():
    from nlse_gb300 import _build, _lib

    _build.build()
    return _lib.load(), _lib


def _partials(nseg, seg):
    return nseg * min(1024, -(-seg // CHUNK))


def _sums_with_workspace(lib, A, dtype, nseg, seg):
    out = torch.empty(nseg, dtype=torch.float64, device=A.device)
    wsb = lib.nlse_power_workspace_size(nseg, seg)
    ws = torch.empty(max(1, wsb // 8), dtype=torch.float64, device=A.device)
    rc = lib.nlse_power(ct.c_void_p(A.data_ptr()), dtype, nseg, seg, ct.c_void_p(out.data_ptr()),
                        ct.c_void_p(ws.data_ptr()), wsb,
                        ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    return out


def _noalloc_into(lib, A, dtype, nseg, seg, out, stream=None):
    s = (stream or torch.cuda.current_stream()).cuda_stream
    rc = lib.nlse_power_noalloc(ct.c_void_p(A.data_ptr()), dtype, nseg, seg,
                                ct.c_void_p(out.data_ptr()), ct.c_void_p(s))
    assert rc == 0, lib.nlse_last_error()
    return out


def _sums_noalloc(lib, A, dtype, nseg, seg):
    out = torch.empty(nseg, dtype=torch.float64, device=A.device)
    return _noalloc_into(lib, A, dtype, nseg, seg, out)


def _fp64_sums(A, nseg):
    a = A.cpu().numpy().reshape(nseg, -1).astype(np.complex128)
    return (a.real ** 2 + a.imag ** 2).sum(axis=1)


def _host_rtol(tdtype):
    """Against exact FP64 squares: complex64 squares are formed in FP32 (the
    reference's own power of a complex64 field), then summed in FP64."""
    return 1e-7 if tdtype == torch.complex64 else 1e-12


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
        # and against an independent FP64 sum on the host
        np.testing.assert_allclose(got.cpu().numpy(), _fp64_sums(A, nseg), rtol=_host_rtol(tdtype),
                                   atol=0)


def test_noalloc_power_at_exact_capacity():
    """65,536 partials exactly: accepted, and the array's last element is written
    (the previous call filled it with other values)."""
    lib, _ = _lib()
    torch.cuda.set_device(0)
    nseg, seg = 32768, CHUNK + 1
    assert _partials(nseg, seg) == CAPACITY
    g = torch.Generator(device="cuda").manual_seed(11)
    A = torch.randn(nseg * seg, dtype=torch.complex64, device="cuda", generator=g)
    B = 3 * torch.randn(nseg * seg, dtype=torch.complex64, device="cuda", generator=g)
    _sums_noalloc(lib, B, 0, nseg, seg)  # leaves B's partials in every slot
    got = _sums_noalloc(lib, A, 0, nseg, seg)
    ref = _sums_with_workspace(lib, A, 0, nseg, seg)
    torch.cuda.synchronize()
    np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(), rtol=1e-13, atol=0)
    np.testing.assert_allclose(got[-4:].cpu().numpy(), _fp64_sums(A[-4 * seg:], 4),
                               rtol=_host_rtol(torch.complex64))


def test_noalloc_power_rejects_requests_beyond_its_array():
    """One partial over capacity is refused.  The buffer really holds the
    requested elements, so a broken size guard would give a wrong answer,
    not an out-of-bounds read."""
    lib, L = _lib()
    torch.cuda.set_device(0)
    nseg, seg = 32769, CHUNK + 1
    assert _partials(nseg, seg) == CAPACITY + 2
    A = torch.zeros(nseg * seg, dtype=torch.complex64, device="cuda")
    out = torch.zeros(nseg, dtype=torch.float64, device="cuda")
    rc = lib.nlse_power_noalloc(ct.c_void_p(A.data_ptr()), 0, nseg, seg,
                                ct.c_void_p(out.data_ptr()), None)
    assert rc == L.ERR_ARG
    assert "static array holds 65536" in L.last_error()
    del A
    torch.cuda.empty_cache()


def test_noalloc_power_allocates_nothing_and_replays_from_a_graph():
    lib, _ = _lib()
    torch.cuda.set_device(0)
    nseg, seg = 4, 1024 * 1024
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(nseg * seg, dtype=torch.complex64, device="cuda", generator=g)
    out = torch.zeros(nseg, dtype=torch.float64, device="cuda")
    _noalloc_into(lib, A, 0, nseg, seg, out)  # first call on the device: address lookup
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _noalloc_into(lib, A, 0, nseg, seg, out)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    ref = _fp64_sums(A, nseg)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=_host_rtol(torch.complex64))
    # captured on a side stream after the first call, then replayed
    side = torch.cuda.Stream()
    graph_out = torch.zeros(nseg, dtype=torch.float64, device="cuda")
    graph = torch.cuda.CUDAGraph()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        graph.capture_begin()
        _noalloc_into(lib, A, 0, nseg, seg, graph_out, stream=side)
        graph.capture_end()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    assert float(graph_out.abs().sum()) == 0.0  # capture does not run the kernels
    graph.replay()
    torch.cuda.synchronize()
    np.testing.assert_allclose(graph_out.cpu().numpy(), out.cpu().numpy(), rtol=0, atol=0)
