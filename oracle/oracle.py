"""ctypes bindings of liboracle.so (CPU restatement of the rebin path).

TEST INFRASTRUCTURE ONLY: what the tests compare the CUDA library with, and the
timed CPU baseline.  Every array crossing the boundary is a C-contiguous numpy array in
the reference's layout (vec4 f32 splat SoA, 64-byte ProjectedSplat,
interleaved u32 [hi, lo] keys).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build import build

PROJ_DTYPE = np.dtype([
    ("mean_px", "<f4", (2,)), ("depth", "<f4"), ("radius_px", "<f4"),
    ("conic", "<f4", (3,)), ("opacity", "<f4"),
    ("color", "<f4", (3,)), ("valid", "<u4"),
    ("tile_min", "<u4", (2,)), ("tile_max", "<u4", (2,)),
])
assert PROJ_DTYPE.itemsize == 64

_P = C.c_void_p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class Oracle:
    def __init__(self):
        lib = C.CDLL(str(build()))
        u32, i32, f64 = C.c_uint32, C.c_int, C.c_double
        lib.orc_camera_uniform.argtypes = [_P, _P, _P, f64, f64, f64, f64, f64, f64, _P]
        lib.orc_activate.argtypes = [u32] + [_P] * 9
        lib.orc_preprocess.argtypes = [u32, _P, _P, _P, _P, _P, _P, _P, _P, u32, _P, _P, i32]
        lib.orc_prefix_scan.argtypes = [u32, _P, _P]
        lib.orc_prefix_scan.restype = u32
        lib.orc_emit.argtypes = [u32, u32, _P, _P, _P, _P]
        lib.orc_radix_sort.argtypes = [u32, _P, _P, _P, _P, i32]
        lib.orc_identify.argtypes = [u32, _P, _P]
        lib.orc_rasterize.argtypes = [u32, u32, u32, u32, u32, u32, _P, _P, _P, _P, _P, i32]
        lib.orc_rebin.argtypes = ([u32, _P, u32, u32, u32, u32] + [_P] * 5 +
                                  [u32, _P, _P, _P, u32, _P, _P, _P, _P, _P, _P, _P, i32])
        lib.orc_rebin.restype = u32
        lib.orc_raster_pairs.argtypes = [u32, u32, u32, u32, u32, u32, _P, _P, _P, _P, i32]
        lib.orc_max_threads.restype = i32
        self.lib = lib

    def max_threads(self) -> int:
        return int(self.lib.orc_max_threads())

    # Camera.ts:69-79,172-191 with gl-matrix lookAt/perspective
    def camera_uniform(self, eye, target, up, fovy, aspect, near, far, width, height):
        out = np.zeros(72, np.float32)
        self.lib.orc_camera_uniform(_ptr(_c(eye, np.float32)), _ptr(_c(target, np.float32)),
                                    _ptr(_c(up, np.float32)), fovy, aspect, near, far,
                                    float(width), float(height), _ptr(out))
        return out

    # SceneWorker.ts:407-464
    def activate(self, xyz, f_dc, opacity, scale_log, rot):
        n = len(opacity)
        pos, col, sc, ro = (np.zeros((n, 4), np.float32) for _ in range(4))
        self.lib.orc_activate(n, _ptr(_c(xyz, np.float64)), _ptr(_c(f_dc, np.float64)),
                              _ptr(_c(opacity, np.float64)), _ptr(_c(scale_log, np.float64)),
                              _ptr(_c(rot, np.float64)), _ptr(pos), _ptr(col), _ptr(sc), _ptr(ro))
        return pos, col, sc, ro

    def preprocess(self, cam, tile_count, inv_tile, pos, scale, rot, color, sh=None,
                   sh_degree=0, threads=0):
        n = len(pos)
        proj = np.zeros(n, PROJ_DTYPE)
        counts = np.zeros(n, np.uint32)
        shc = None if (sh is None or sh_degree == 0) else _c(sh, np.float32)
        self.lib.orc_preprocess(n, _ptr(_c(cam, np.float32)), _ptr(_c(tile_count, np.uint32)),
                                _ptr(_c(inv_tile, np.float32)), _ptr(_c(pos, np.float32)),
                                _ptr(_c(scale, np.float32)), _ptr(_c(rot, np.float32)),
                                _ptr(_c(color, np.float32)), _ptr(shc),
                                sh_degree if shc is not None else 0, _ptr(proj), _ptr(counts),
                                threads)
        return proj, counts

    def prefix_scan(self, counts):
        counts = _c(counts, np.uint32)
        off = np.zeros(len(counts) + 1, np.uint32)
        total = self.lib.orc_prefix_scan(len(counts), _ptr(counts), _ptr(off))
        return off, int(total)

    def emit(self, tiles_x, proj, offsets, total):
        keys = np.zeros((total, 2), np.uint32)
        vals = np.zeros(total, np.uint32)
        self.lib.orc_emit(len(proj), tiles_x, _ptr(np.ascontiguousarray(proj)),
                          _ptr(_c(offsets, np.uint32)), _ptr(keys), _ptr(vals))
        return keys, vals

    def radix_sort(self, keys, vals, threads=0):
        keys = np.array(keys, np.uint32, order="C", copy=True)
        vals = np.array(vals, np.uint32, order="C", copy=True)
        tk, tv = np.empty_like(keys), np.empty_like(vals)
        self.lib.orc_radix_sort(len(vals), _ptr(keys), _ptr(vals), _ptr(tk), _ptr(tv), threads)
        return keys, vals

    def identify(self, keys, num_tiles):
        off = np.zeros(num_tiles + 1, np.uint32)
        keys = _c(keys, np.uint32)
        self.lib.orc_identify(len(keys), _ptr(keys), _ptr(off))
        return off

    def rasterize(self, width, height, tile_w, tile_h, proj, tile_offsets, vals, threads=0):
        tx, ty = -(-width // tile_w), -(-height // tile_h)
        img = np.zeros((height, width, 4), np.float32)
        costs = np.zeros(tx * ty, np.uint32)
        self.lib.orc_rasterize(width, height, tile_w, tile_h, tx, ty,
                               _ptr(np.ascontiguousarray(proj)), _ptr(_c(tile_offsets, np.uint32)),
                               _ptr(_c(vals, np.uint32)), _ptr(img), _ptr(costs), threads)
        return img, costs

    def raster_pairs(self, width, height, tile_w, tile_h, proj, tile_offsets, vals, threads=0):
        """(pixel, splat) pairs of the reference raster loop: iterated, exp
        evaluated, blended."""
        tx, ty = -(-width // tile_w), -(-height // tile_h)
        out = np.zeros(3, np.uint64)
        self.lib.orc_raster_pairs(width, height, tile_w, tile_h, tx, ty,
                                  _ptr(np.ascontiguousarray(proj)),
                                  _ptr(_c(tile_offsets, np.uint32)), _ptr(_c(vals, np.uint32)),
                                  _ptr(out), threads)
        return {"iterated": int(out[0]), "evaluated": int(out[1]), "blended": int(out[2])}

    def rebin(self, cam, width, height, tile_w, tile_h, pos, scale, rot, color, sh=None,
              sh_degree=0, threads=0, key_capacity=None):
        """Whole path; returns a dict of every intermediate named buffer."""
        n = len(pos)
        tx, ty = -(-width // tile_w), -(-height // tile_h)
        if key_capacity is None:
            _, counts = self.preprocess(cam, (tx, ty), (np.float32(1.0 / tile_w),
                                        np.float32(1.0 / tile_h)), pos, scale, rot, color,
                                        sh, sh_degree, threads)
            key_capacity = int(counts.astype(np.uint64).sum())
        proj = np.zeros(n, PROJ_DTYPE)
        counts = np.zeros(n, np.uint32)
        off = np.zeros(n + 1, np.uint32)
        cap = max(1, key_capacity)
        keys = np.zeros((cap, 2), np.uint32)
        vals = np.zeros(cap, np.uint32)
        tk, tv = np.zeros_like(keys), np.zeros_like(vals)
        toff = np.zeros(tx * ty + 1, np.uint32)
        img = np.zeros((height, width, 4), np.float32)
        costs = np.zeros(tx * ty, np.uint32)
        shc = None if (sh is None or sh_degree == 0) else _c(sh, np.float32)
        r = self.lib.orc_rebin(n, _ptr(_c(cam, np.float32)), width, height, tile_w, tile_h,
                               _ptr(_c(pos, np.float32)), _ptr(_c(scale, np.float32)),
                               _ptr(_c(rot, np.float32)), _ptr(_c(color, np.float32)),
                               _ptr(shc), sh_degree if shc is not None else 0, _ptr(proj),
                               _ptr(counts), _ptr(off), cap, _ptr(keys), _ptr(vals), _ptr(tk),
                               _ptr(tv), _ptr(toff), _ptr(img), _ptr(costs), threads)
        if r == 0xFFFFFFFF:
            raise OverflowError("key capacity exceeded")
        return dict(projected_splats=proj, splat_ref_counts=counts, splat_ref_offsets=off,
                    ref_counter=int(r), sort_keys_a=keys[:r], sort_values_a=vals[:r],
                    tile_offsets=toff, image=img, tile_costs=costs, tiles=(tx, ty))
