"""gs3d_prefix_scan_noalloc: the prefix scan for callers that cannot let a
library allocate device memory (their GPU memory belongs to their own pool or
caching allocator, or their frame loop must not hit the implicit device
synchronisation of cudaMalloc/cudaFree).  Its scratch is a fixed array
inside the library shared by every call, so the test runs it several times in
a row on different inputs, through the C ABI, and compares each result with
the context-based gs3d_prefix_scan on the same counts and with a host
cumulative sum (integers: bit-exact).  A total of 2^32 or more must be
reported by gs3d_prefix_scan_noalloc_status, not returned as a silent wrong
result.

This file sorts last so that a failure here, under -x, comes after every
other test; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from gs3d import _lib
from gs3d.camera import camera_struct
from gs3d import scenes

pytestmark = pytest.mark.gpu


def context_scan(lib, counts):
    """Offsets from the existing entry point (gs3d_prefix_scan on a context)."""
    n = len(counts)
    ctx = C.c_void_p()
    assert lib.gs3d_create(C.byref(ctx), None) == 0
    try:
        z = np.zeros((n, 4), np.float32)
        p = z.ctypes.data_as(C.c_void_p)
        assert lib.gs3d_set_splats(ctx, n, p, p, p, p, None, 0, 0) == 0
        cam = camera_struct(scenes.small_camera(64, 64).getUniformData(64, 64))
        assert lib.gs3d_set_camera(ctx, C.byref(cam), 64, 64) == 0
        assert lib.gs3d_write_buffer(ctx, _lib.BUFFERS["splat_ref_counts"],
                                     counts.ctypes.data_as(C.c_void_p), counts.nbytes) == 0
        assert lib.gs3d_prefix_scan(ctx) == 0
        out = np.zeros(n + 1, np.uint32)
        assert lib.gs3d_read_buffer(ctx, _lib.BUFFERS["splat_ref_offsets"],
                                    out.ctypes.data_as(C.c_void_p), out.nbytes) == 0
        return out
    finally:
        lib.gs3d_destroy(ctx)


def host_scan(counts):
    """Exclusive prefix sum with the total appended, as u32 (no overflow here)."""
    inc = np.cumsum(counts, dtype=np.uint64)
    return np.concatenate(([0], inc)).astype(np.uint32)


def noalloc_scan(lib, torch, counts, stream):
    n = len(counts)
    d_counts = torch.from_numpy(counts.view(np.int32)).cuda()
    d_out = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
    rc = lib.gs3d_prefix_scan_noalloc(C.c_void_p(d_counts.data_ptr()),
                                      C.c_void_p(d_out.data_ptr()), n, C.c_void_p(stream))
    assert rc == 0, lib.gs3d_last_error(None)
    status = lib.gs3d_prefix_scan_noalloc_status(C.c_void_p(stream))
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint32), status


def test_noalloc_scan_matches_context_scan_twice(built_lib):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    rng = np.random.default_rng(7)
    stream = torch.cuda.current_stream().cuda_stream
    # several calls in a row: full look-back tiles, ragged tails, one count,
    # one count past a tile
    for n, hi in ((1_000_003, 40), (777_777, 7), (1, 1000), (2049, 3), (4096, 100)):
        counts = rng.integers(0, hi, n).astype(np.uint32)
        got, status = noalloc_scan(lib, torch, counts, stream)
        assert status == 0, lib.gs3d_last_error(None)
        assert np.array_equal(got, host_scan(counts))
        assert np.array_equal(got, context_scan(lib, counts))
        assert got[-1] == counts.astype(np.uint64).sum()


def test_noalloc_scan_reports_a_total_past_32_bits(built_lib):
    """2^21 counts of 4096 sum to 2^33: the offsets cannot be represented in
    u32, so the status call reports the capacity error (offsets[n] holds the
    0xffffffff sentinel); the next in-range call reports success again."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    counts = np.full(1 << 21, 4096, np.uint32)
    got, status = noalloc_scan(lib, torch, counts, stream)
    assert status == _lib.ERR_CAPACITY
    assert b"2^32" in lib.gs3d_last_error(None)
    assert got[-1] == 0xFFFFFFFF
    # offsets below the overflow are exact: the first 2^20 - 1 tiles' prefixes fit
    k = (1 << 20) - 4096
    assert np.array_equal(got[:k], host_scan(counts[:k])[:k])
    small = np.arange(5000, dtype=np.uint32) % 9
    got, status = noalloc_scan(lib, torch, small, stream)
    assert status == 0
    assert np.array_equal(got, host_scan(small))


def test_noalloc_scan_rejects_oversized_input(built_lib):
    lib = _lib.load()
    rc = lib.gs3d_prefix_scan_noalloc(C.c_void_p(16), C.c_void_p(16), (1 << 26) + 1, None)
    assert rc == _lib.ERR_INVALID_ARG
    assert b"exceeds the maximum" in lib.gs3d_last_error(None)
