"""C-ABI surface checks that need no GPU: the in-tree libgs3d.so loads and
exports every entry point include/gs3d.h declares, and its entry points
fail with status codes (no crash) when no device is present."""
import ctypes as C
import re
from pathlib import Path

import pytest

from conftest import ROOT, has_gpu

HEADER = ROOT / "include" / "gs3d.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^(?:int|const char\*|void)\s+\*?(gs3d_\w+)\s*\(", text, re.M)))


def test_header_declares_the_rebin_stages():
    names = declared_functions()
    for stage in ("gs3d_preprocess", "gs3d_prefix_scan", "gs3d_emit_tile_refs", "gs3d_radix_sort",
                  "gs3d_identify_tile_ranges", "gs3d_rasterize_tiles", "gs3d_rebin"):
        assert stage in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_the_header(built_lib):
    from gs3d import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES), \
        set(declared_functions()) - set(_lib.SIGNATURES)
    lib = _lib.load()
    assert lib.gs3d_abi_version() == 1


def test_null_arguments_are_rejected(built_lib):
    from gs3d import _lib
    lib = _lib.load()
    assert lib.gs3d_create(None, None) == _lib.ERR_INVALID_ARG
    assert lib.gs3d_destroy(None) == _lib.ERR_INVALID_ARG
    assert lib.gs3d_rebin(None, None, 1, 1) == _lib.ERR_INVALID_ARG
    assert lib.gs3d_synchronize(None) == _lib.ERR_INVALID_ARG
    assert lib.gs3d_prefix_scan_noalloc(None, None, 4, None) == _lib.ERR_INVALID_ARG
    assert lib.gs3d_set_tuning(None, None) == _lib.ERR_INVALID_ARG
    assert lib.gs3d_get_tuning(None, None) == _lib.ERR_INVALID_ARG
    assert lib.gs3d_autotune(None, None, 0, 0, None, 0, None) == _lib.ERR_INVALID_ARG
    assert b"null" in lib.gs3d_last_error(None)


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_noalloc_status_without_device_is_a_status_code(built_lib):
    from gs3d import _lib
    lib = _lib.load()
    assert lib.gs3d_prefix_scan_noalloc_status(None) == _lib.ERR_NO_DEVICE


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_create_without_device_reports_no_device(built_lib):
    from gs3d import _lib
    lib = _lib.load()
    ctx = C.c_void_p()
    assert lib.gs3d_create(C.byref(ctx), None) == _lib.ERR_NO_DEVICE
    assert not ctx.value


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_renderer_init_raises_without_device(built_lib):
    from gs3d import GaussianSplatRenderer, Gs3dError, Scene
    r = GaussianSplatRenderer(Scene())
    with pytest.raises(Gs3dError) as ei:
        r.init()
    assert ei.value.code == 7
