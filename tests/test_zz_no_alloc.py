"""The allocation-free batched entry point, xs_run_event_batched_static.

It serves callers that must not allocate device memory (a host thread driving
other GPU work, which cudaMalloc/cudaFree could stall; a program whose memory
manager owns the device budget).  Its scratch is a static device array, shared
by every call, so the test makes two calls in a row and checks each against
the allocating entry point, xs_run_event with the batched kernel, at the
tolerance the parity tests use (FAST: per-lookup macro_xs vectors within 1e-12
relative; EXACT: bit-identical), on a unionized and a hash-grid problem;
checks that a batch above the array's limit is refused; and checks that the
calls leave the device's free memory unchanged.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

import xsbench_gb300 as X
from conftest import golden_json, product_inputs

pytestmark = pytest.mark.gpu

MAX_LOOKUPS = 1 << 19


def rel_err(a, b):
    return float(np.max(np.max(np.abs(a - b), axis=1) / np.max(np.abs(b), axis=1)))


@pytest.fixture(scope="module", params=["tiny_unionized", "tiny_hash"])
def ctx(request):
    inp = product_inputs(request.param)
    with X.grid_init(inp) as p, X.Context(inp, p) as c:
        c.name = request.param
        yield c


@pytest.mark.parametrize("arith", ["fast", "exact"])
def test_static_matches_allocating_entry_on_two_calls(ctx, arith):
    import torch
    n = 150000
    ref_macro = np.empty((n, 5))
    ref_idx = np.empty(n, np.uint8)
    for first in (0, 50000):  # two calls in a row, each against the allocating path
        r = ctx.run_event(first=first, count=n, kernel="batched", arith=arith,
                          macro_out=ref_macro, max_idx_out=ref_idx)
        d_macro = torch.full((n, 5), float("nan"), dtype=torch.float64, device="cuda")
        d_idx = torch.full((n,), 255, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        L = X.lib()
        v = C.c_ulonglong()
        st = L.xs_run_event_batched_static(ctx._h, first, n, X.ARITH_EXACT if arith == "exact" else X.ARITH_FAST,
                                           1024, C.c_void_p(d_macro.data_ptr()),
                                           C.c_void_p(d_idx.data_ptr()), None, C.byref(v))
        assert st == 0, L.xs_last_error()
        assert v.value == r.verification
        m = d_macro.cpu().numpy()
        assert np.array_equal(d_idx.cpu().numpy(), ref_idx)
        if arith == "exact":
            assert np.array_equal(m, ref_macro)
        else:
            assert rel_err(m, ref_macro) <= 1e-12


def test_static_full_batch_in_chunks_gives_reference_hash(ctx):
    g = golden_json("full_" + ctx.name)
    total = 0
    for a in range(0, g["lookups"], MAX_LOOKUPS):
        n = min(MAX_LOOKUPS, g["lookups"] - a)
        total += ctx.run_event_batched_static(a, n)
    assert total == g["verification"]


def test_static_rejects_oversized_batches(ctx):
    L = X.lib()
    v = C.c_ulonglong()
    assert L.xs_run_event_batched_static(ctx._h, 0, MAX_LOOKUPS + 1, 0, 1024, None, None, None,
                                         C.byref(v)) == 1
    assert b"static scratch" in L.xs_last_error()
    assert L.xs_run_event_batched_static(ctx._h, 0, 1000, 0, 8192, None, None, None,
                                         C.byref(v)) == 1
    host = np.empty((1000, 5))
    assert L.xs_run_event_batched_static(ctx._h, 0, 1000, 0, 1024,
                                         host.ctypes.data_as(C.c_void_p), None, None,
                                         C.byref(v)) == 1
    # the Python wrapper refuses outputs the kernels would overrun or misread
    import torch
    with pytest.raises(ValueError):   # float32: half the bytes of (count, 5) doubles
        ctx.run_event_batched_static(0, 1000, macro_out=torch.empty((1000, 5), dtype=torch.float32,
                                                                    device="cuda"))
    with pytest.raises(ValueError):   # too short
        ctx.run_event_batched_static(0, 1000, macro_out=torch.empty((999, 5), dtype=torch.float64,
                                                                    device="cuda"))
    with pytest.raises(ValueError):
        ctx.run_event_batched_static(0, 1000, max_idx_out=torch.empty(999, dtype=torch.uint8,
                                                                      device="cuda"))
    with pytest.raises(ValueError):   # host memory
        ctx.run_event_batched_static(0, 1000, max_idx_out=np.empty(1000, np.uint8))
    # the entry point still works after the refusals
    assert ctx.run_event_batched_static(0, 1000) == ctx.run_event(count=1000).verification


def test_static_calls_allocate_no_device_memory(ctx):
    """Device memory in use (cudaMemGetInfo) and the context's own bytes are
    the same before and after static calls made back to back, with no
    allocating call between them; the calling thread's device is unchanged."""
    import torch
    n = 200000
    d_macro = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    d_idx = torch.empty(n, dtype=torch.uint8, device="cuda")
    ctx.run_event_batched_static(0, n, macro_out=d_macro, max_idx_out=d_idx)  # kernels loaded
    torch.cuda.synchronize()
    dev = torch.cuda.current_device()
    free0, _ = torch.cuda.mem_get_info()
    bytes0 = ctx.device_bytes
    sums = [ctx.run_event_batched_static(a, n, macro_out=d_macro, max_idx_out=d_idx)
            for a in (0, 100000, 0)]
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert ctx.device_bytes == bytes0
    assert torch.cuda.current_device() == dev
    assert sums[0] == sums[2]
