"""The allocation-free direction-set entry point, memd_directions_noalloc_f64.

It exists for callers that must not allocate device memory: a MATLAB MEX
function whose GPU buffers have to come from MATLAB's own allocator, a
real-time acquisition loop that cannot afford the device-wide synchronisation
cudaMalloc/cudaFree may cause, or an application that hands out all device
memory from one arena of its own.  Its scratch (the prime table) is a static
device array of 4096 entries shared by every call.

The GPU tests call it through the C ABI several times in a row, with
different tables, and check each result against the allocating entry point
memd_directions_f64, and check that the calls leave the device's free memory
unchanged.  This file is collected last so that a run stopping at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import memd_gb300 as mg


def _noalloc(C, K, primes, out_ptr):
    pr = None if primes is None else np.ascontiguousarray(primes, dtype=np.int32)
    return mg.lib().memd_directions_noalloc_f64(
        C, K, None if pr is None else pr.ctypes.data_as(ctypes.c_void_p), out_ptr, None)


@pytest.mark.gpu
def test_noalloc_directions_match_allocating_entry_on_two_calls():
    torch = pytest.importorskip("torch")
    # the standalone table first, then a MEX-style table that overwrites the
    # shared static array, then the standalone case again
    cases = [(32, 128, None), (6, 40, [2, 3, 5, 7, 11, 13]), (32, 128, None)]
    for C, K, primes in cases:
        out = torch.full((K, C), float("nan"), dtype=torch.float64, device="cuda")
        assert _noalloc(C, K, primes, out.data_ptr()) == mg.MEMD_OK, mg.last_error()
        torch.cuda.synchronize()
        ref = mg.directions(C, K, primes=primes, dtype="f64")
        diff = (out - ref).abs().max().item()
        assert diff <= 1e-15, (C, K, diff)
        # unit vectors, as the allocating entry point gives
        assert (out.norm(dim=1) - 1).abs().max().item() < 1e-14


@pytest.mark.gpu
def test_noalloc_directions_allocate_no_device_memory():
    torch = pytest.importorskip("torch")
    C, K = 16, 64
    outs = [torch.empty((K, C), dtype=torch.float64, device="cuda") for _ in range(2)]
    # one call first: it may load the library's kernels into the context
    assert _noalloc(C, K, None, outs[0].data_ptr()) == mg.MEMD_OK, mg.last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    held0 = torch.cuda.memory_allocated()
    for i in range(6):
        primes = None if i % 2 == 0 else [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53]
        assert _noalloc(C, K, primes, outs[i % 2].data_ptr()) == mg.MEMD_OK, mg.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    assert torch.cuda.memory_allocated() == held0
    ref = mg.directions(C, K, primes=[2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53], dtype="f64")
    assert (outs[1] - ref).abs().max().item() <= 1e-15


def test_noalloc_rejects_more_channels_than_the_static_table():
    # the size check runs before any CUDA call; the pointer is never touched
    rc = _noalloc(4097, 8, None, 16)
    assert rc == mg.MEMD_ERR_INVALID
    assert "4096" in mg.last_error()
