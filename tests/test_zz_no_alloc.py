"""The allocation-free per-history trace entry point, midsx_gpu_trace_deposits_noalloc.

Some callers cannot allocate device memory while they run: a service that reserves its
whole GPU memory budget at start-up and treats any later allocation as a failure, a host
application whose device memory is owned by its own pool allocator, or a latency-critical
loop that cannot afford the device-wide synchronisation of cudaFree.  For them the library
offers this one entry point, which uses a fixed scratch array compiled into its device code
instead of cudaMalloc.  This test calls it through the C ABI, twice in a row with different
inputs, and checks each result against the allocating entry point midsx_gpu_trace_deposits
on the same inputs; it also checks that a request above the fixed limit, or one asking for a
tracking mode whose set-up would allocate (macro cells), is refused, and that the device's
free memory (cudaMemGetInfo, read through torch) is the same before and after warm calls.
The free-memory reading is coarse - the driver hands out memory in pages, so a small
allocation can hide in a page already mapped - and backs up, not replaces, the code path:
the entry point calls no allocating routine.
"""
import ctypes as C

import numpy as np
import pytest

import midsx_gb300 as M
from midsx_gb300 import native as N
from midsx_gb300 import scenes

pytestmark = pytest.mark.gpu

LIMIT = 1 << 20  # histories per call that the fixed scratch holds


def call_noalloc(lib, tables, ph, src, cfg, out):
    return lib.midsx_gpu_trace_deposits_noalloc(tables.handle, ph.handle, src.handle, C.byref(cfg), N.dptr(out), None)


def test_noalloc_trace_equals_allocating_trace_twice_in_a_row():
    sc = scenes.water_cube(n=20, bins=10)
    tables, ph, src, _ = sc.build()
    lib = N.load()
    calls = [dict(n=60_000, seed=3, first=0, precision="fp64"),
             dict(n=25_000, seed=4, first=7_000, precision="mixed")]
    for c in calls:
        expect = M.trace_deposits(tables, ph, src, c["n"], seed=c["seed"], first=c["first"], precision=c["precision"])
        cfg = M.run_config(c["n"], c["seed"], c["first"], c["precision"])
        got = np.full(c["n"], -1.0)
        status = call_noalloc(lib, tables, ph, src, cfg, got)
        assert status == N.OK, lib.midsx_last_error()
        # same kernel on the same Philox streams: equal within the trace tolerance used by
        # the other parity tests (1e-9 relative)
        assert np.all(np.abs(got - expect) <= 1e-9 * np.maximum(1.0, np.abs(expect)))
        assert got.sum() > 0


def test_noalloc_trace_refuses_requests_above_its_limit():
    sc = scenes.water_cube(n=10, bins=10)
    tables, ph, src, _ = sc.build()
    lib = N.load()
    cfg = M.run_config(LIMIT + 1, seed=1)
    out = np.zeros(1)  # never written: the call is refused before any device work
    status = call_noalloc(lib, tables, ph, src, cfg, out)
    assert status == N.INVALID_ARG
    assert b"1048576" in lib.midsx_last_error()


def free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_trace_leaves_free_memory_unchanged_and_refuses_allocating_modes():
    sc = scenes.water_cube(n=64, bins=10)
    tables, ph, src, _ = sc.build()
    lib = N.load()
    n = 400_000
    out = np.zeros(n)
    cfg = M.run_config(n, seed=5, precision="mixed")
    assert call_noalloc(lib, tables, ph, src, cfg, out) == N.OK  # warm: the kernel's module is loaded
    before = free_bytes()
    for seed in (6, 7):
        cfg = M.run_config(n, seed=seed, precision="mixed")
        assert call_noalloc(lib, tables, ph, src, cfg, out) == N.OK, lib.midsx_last_error()
    assert free_bytes() == before
    # macro-cell tracking would build the phantom's cells with cudaMalloc: refused up front
    cfg = M.run_config(n, seed=8, precision="mixed", tracking="macro_cell")
    assert call_noalloc(lib, tables, ph, src, cfg, out) == N.INVALID_ARG
    assert b"reference tracking" in lib.midsx_last_error()
    assert free_bytes() == before
