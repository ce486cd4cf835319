"""gs3d_prefix_scan_noalloc: the prefix scan for callers that cannot let a
library allocate device memory (their GPU memory belongs to their own pool or
caching allocator, or their frame loop must not hit the implicit device
synchronisation of cudaMalloc/cudaFree).  Its scratch is a fixed array
inside the library shared by every call, so the test runs it twice in a row
on different inputs, through the C ABI, and compares each result with the
context-based gs3d_prefix_scan on the same counts (integers: bit-exact).

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


def test_noalloc_scan_matches_context_scan_twice(built_lib):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    rng = np.random.default_rng(7)
    stream = torch.cuda.current_stream().cuda_stream
    for n, hi in ((1_000_003, 40), (777_777, 7)):  # two calls in a row, different sizes
        counts = rng.integers(0, hi, n).astype(np.uint32)
        d_counts = torch.from_numpy(counts.view(np.int32)).cuda()
        d_out = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
        rc = lib.gs3d_prefix_scan_noalloc(C.c_void_p(d_counts.data_ptr()),
                                          C.c_void_p(d_out.data_ptr()), n, C.c_void_p(stream))
        assert rc == 0, lib.gs3d_last_error(None)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(np.uint32)
        expect = context_scan(lib, counts)
        assert np.array_equal(got, expect)
        assert got[-1] == counts.astype(np.uint64).sum()


def test_noalloc_scan_rejects_oversized_input(built_lib):
    lib = _lib.load()
    rc = lib.gs3d_prefix_scan_noalloc(C.c_void_p(16), C.c_void_p(16), (1 << 26) + 1, None)
    assert rc == _lib.ERR_INVALID_ARG
    assert b"exceeds the maximum" in lib.gs3d_last_error(None)
