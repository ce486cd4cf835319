"""Host mirror of the reference renderer's plug-in surface over libgs3d.

`GaussianSplatRenderer` keeps the method names and argument meaning of
src/renderers/GaussianSplatRenderer.ts (init, render, rebin, setTileSize,
setAlwaysRebin, getTileCount, getTileSize, readTileCounts) and `SceneSyncer`
those of src/SceneSyncer.ts (setSplatData).  A WebGPU command encoder and
swapchain texture do not exist here: `render` takes a `RenderFrameInfo` that
carries the viewport size, the camera and its version counter, and the splat
target is a headless rgba16float device buffer (readImage copies it out).

Errors: the reference throws on configuration bugs and surfaces WebGPU
validation errors asynchronously; here every library failure raises
`Gs3dError` carrying the C status code and the library's message.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import Config_t, Gs3dError
from .camera import Camera, camera_struct
from .scenes import GaussianSplatData

PROJ_DTYPE = np.dtype([
    ("mean_px", "<f4", (2,)), ("depth", "<f4"), ("radius_px", "<f4"),
    ("conic", "<f4", (3,)), ("opacity", "<f4"),
    ("color", "<f4", (3,)), ("valid", "<u4"),
    ("tile_min", "<u4", (2,)), ("tile_max", "<u4", (2,)),
])


@dataclass
class Scene:
    """src/Scene.ts: tile pixel size and the splat data."""
    tiles: list = field(default_factory=lambda: [16, 16])
    splats: GaussianSplatData | None = None


@dataclass
class RenderFrameInfo:
    """src/renderers/IRenderer.ts:1-8 without the WebGPU textures."""
    width: int
    height: int
    camera: Camera | np.ndarray  # a Camera or its 72-float uniform block
    cameraVersion: int = 0


def _check(lib, ctx, rc: int):
    if rc != _lib.OK:
        msg = lib.gs3d_last_error(ctx) if ctx else b"no context"
        raise Gs3dError(rc, (msg or b"").decode(errors="replace"))


class GaussianSplatRenderer:
    def __init__(self, scene: Scene, device: int = 0, stream: int | None = None):
        self.scene = scene
        self.device = device
        self.stream = stream
        self.ctx = None
        self.lib = None
        self.alwaysRebin = False
        self.lastSplatCount = -1
        self.lastViewport = (-1, -1)
        self.lastCameraVersion = -1
        self.tileCountX = self.tileCountY = 0
        self.tileSizeX, self.tileSizeY = scene.tiles
        self.viewport = (0, 0)

    # ---- lifetime (GaussianSplatRenderer.init, :331-471) -------------------
    def init(self, format: str = "rgba16float") -> None:
        if format != "rgba16float":
            raise ValueError("the splat target is rgba16float (GaussianSplatRenderer.ts:234)")
        self.lib = _lib.load()
        cfg = Config_t(self.device, int(self.scene.tiles[0]), int(self.scene.tiles[1]), 16,
                       self.stream, 0)
        ctx = C.c_void_p()
        rc = self.lib.gs3d_create(C.byref(ctx), C.byref(cfg))
        if rc != _lib.OK:
            raise Gs3dError(rc, "gs3d_create failed (no sm_103 device, or the library "
                                "was built for another architecture)")
        self.ctx = ctx
        self.tileSizeX, self.tileSizeY = self.setTileSize(*self.scene.tiles)

    def destroy(self) -> None:
        if self.ctx:
            self.lib.gs3d_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        if self.ctx is None:
            self.init()
        return self

    def __exit__(self, *exc):
        self.destroy()

    def _call(self, name, *args):
        _check(self.lib, self.ctx, getattr(self.lib, name)(self.ctx, *args))

    # ---- SceneSyncer.setSplatData (SceneSyncer.ts:25-38) -------------------
    def setSplatData(self, data: GaussianSplatData | None = None) -> None:
        data = data if data is not None else self.scene.splats
        if data is None:
            return
        self.scene.splats = data
        arrs = [np.ascontiguousarray(a, np.float32) for a in
                (data.positions, data.scales, data.rotations, data.colors)]
        for a in arrs:
            if a.shape != (data.splatCount, 4):
                raise ValueError("splat arrays must be (N, 4) float32")
        sh = None
        deg = int(data.sphericalHarmonicsDegree)
        if deg > 0:
            sh = np.ascontiguousarray(data.sphericalHarmonics, np.float32)
            k = 3 * ((deg + 1) ** 2 - 1)
            if sh.shape != (data.splatCount, k):
                raise ValueError(f"sphericalHarmonics must be (N, {k}) for degree {deg}")
        ptr = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
        self._call("gs3d_set_splats", data.splatCount, *(ptr(a) for a in arrs), ptr(sh), deg, 0)
        self.lastSplatCount = -1  # force a rebin

    # ---- knobs ---------------------------------------------------------------
    def setTileSize(self, x: int, y: int) -> tuple[int, int]:
        ox, oy = C.c_uint32(), C.c_uint32()
        self._call("gs3d_set_tile_size", int(x), int(y), C.byref(ox), C.byref(oy))
        if (ox.value, oy.value) != (self.tileSizeX, self.tileSizeY):
            self.lastViewport = (-1, -1)
        self.tileSizeX, self.tileSizeY = ox.value, oy.value
        self.scene.tiles = [ox.value, oy.value]
        return ox.value, oy.value

    def setStagewise(self, on: bool) -> None:
        """Selects the stage-wise rebin (the six reference stages in order)
        instead of the fused default; both give identical sorted keys,
        values, tile ranges and images."""
        self._flags = (getattr(self, "_flags", 0) & ~_lib.FLAG_STAGEWISE_REBIN) | \
            (_lib.FLAG_STAGEWISE_REBIN if on else 0)
        self._call("gs3d_set_flags", self._flags)

    def setCudaGraph(self, on: bool) -> None:
        """Runs fused rebins as a captured CUDA graph, replayed per batch layout."""
        self._flags = (getattr(self, "_flags", 0) & ~_lib.FLAG_CUDA_GRAPH) | \
            (_lib.FLAG_CUDA_GRAPH if on else 0)
        self._call("gs3d_set_flags", self._flags)

    def setSchedule(self, schedule: int) -> None:
        """Raster work order: _lib.SCHEDULE_ROW_MAJOR or SCHEDULE_KEY_COUNT."""
        self._call("gs3d_set_schedule", int(schedule))

    def setCostModel(self, path=None) -> bool:
        """Loads a cost-MLP checkpoint (default: the one trained for the 3M-splat
        1080p workload).  When its held-out error is within its bound and it
        ranks tiles better than the key count, it is installed and the learned
        schedule selected; otherwise the key-count schedule is selected.
        Once installed, the library measures the model's error against the
        costs every raster records and orders frames by key count while the
        running error exceeds the checkpoint's bound (getScheduleStatus).
        Returns whether the learned schedule is selected."""
        from pathlib import Path
        from . import learned
        path = Path(path) if path else Path(__file__).with_name("cost_mlp_c1.npz")
        params, mean, std, metrics, bound = learned.load(path)
        if not learned.gate(metrics, bound):
            self.setSchedule(_lib.SCHEDULE_KEY_COUNT)
            return False
        f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
        params, mean, std = f32(params), f32(mean), f32(std)
        self.setScheduleGate(bound)
        self._call("gs3d_set_cost_model", params.ctypes.data_as(C.c_void_p),
                   mean.ctypes.data_as(C.c_void_p), std.ctypes.data_as(C.c_void_p))
        self.setSchedule(_lib.SCHEDULE_LEARNED)
        return True

    def setScheduleGate(self, bound: float) -> None:
        """Bound on the learned schedule's running mean |log cost error|; above
        it the library orders frames by key count until the error recovers."""
        self._call("gs3d_set_schedule_gate", float(bound))

    def getScheduleStatus(self) -> dict:
        """Requested and active raster order, the gate's measured error and
        the number of tiles the last raster split (blocking)."""
        st = _lib.ScheduleStatus_t()
        self._call("gs3d_get_schedule_status", C.byref(st))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def setSplitAllTiles(self, on: bool) -> None:
        """Shades every tile as half-strip work items (testing the split; the
        image is unchanged)."""
        self._flags = (getattr(self, "_flags", 0) & ~_lib.FLAG_SPLIT_ALL_TILES) | \
            (_lib.FLAG_SPLIT_ALL_TILES if on else 0)
        self._call("gs3d_set_flags", self._flags)

    def setTuning(self, tile: int | tuple[int, int] = 16, digit_bits: int = 8,
                  raster_batch: int = 0) -> None:
        """Speed knobs that leave every image bit-identical: square (or
        (w, h)) tile size (up to 1024 pixels, or 2048 with a width that divides
        by 8 and a height by 16), widest tile-id radix digit (4, 6, 8 or 11
        bits), splats staged per raster batch (0 = one per tile pixel, at most
        1024)."""
        tw, th = (tile, tile) if isinstance(tile, int) else tile
        t = _lib.Tuning_t(int(tw), int(th), int(digit_bits), int(raster_batch))
        self._call("gs3d_set_tuning", C.byref(t))
        # the tuning may hold tiles above setTileSize's 1024-pixel clamp
        if (int(tw), int(th)) != (self.tileSizeX, self.tileSizeY):
            self.lastViewport = (-1, -1)
        self.tileSizeX, self.tileSizeY = int(tw), int(th)
        self.scene.tiles = [int(tw), int(th)]

    def getTuning(self) -> dict:
        t = _lib.Tuning_t()
        self._call("gs3d_get_tuning", C.byref(t))
        return {"tile": (t.tile_w, t.tile_h), "digit_bits": t.digit_bits,
                "raster_batch": t.raster_batch}

    def autotune(self, views, reps: int = 3) -> list[dict]:
        """Times the batched rebin of views ((scene, camera_uniform, w, h)
        tuples) under every candidate tuning, applies the fastest and returns
        the measurements, fastest first."""
        views = list(views)
        arr = (_lib.View_t * len(views))()
        for i, (scene, u, w, h) in enumerate(views):
            arr[i].camera = camera_struct(u)
            arr[i].scene = int(scene)
            arr[i].width = int(w)
            arr[i].height = int(h)
        out = (_lib.TuneResult_t * 64)()
        n = C.c_uint32()
        self._call("gs3d_autotune", C.cast(arr, C.c_void_p), len(views), int(reps), out, 64,
                   C.byref(n))
        best = self.getTuning()
        self.tileSizeX, self.tileSizeY = best["tile"]
        self.scene.tiles = list(best["tile"])
        self.lastViewport = (-1, -1)
        res = [{"tile": (r.tuning.tile_w, r.tuning.tile_h), "digit_bits": r.tuning.digit_bits,
                "raster_batch": r.tuning.raster_batch, "ms_per_view": float(r.ms_per_view),
                "tile_passes": int(r.tile_passes), "refs": int(r.refs)}
               for r in out[:n.value]]
        return sorted(res, key=lambda r: r["ms_per_view"])

    def setAlwaysRebin(self, on: bool) -> None:
        self.alwaysRebin = bool(on)

    def getTileCount(self) -> tuple[int, int]:
        return self.tileCountX, self.tileCountY

    def getTileSize(self) -> tuple[int, int]:
        return self.tileSizeX, self.tileSizeY

    # ---- frame ---------------------------------------------------------------
    @staticmethod
    def _uniform(camera, width, height) -> np.ndarray:
        if isinstance(camera, Camera):
            return camera.getUniformData(width, height)
        return np.ascontiguousarray(camera, np.float32)

    def render(self, frame: RenderFrameInfo) -> bool:
        """GaussianSplatRenderer.render (:1033-1098) up to the composite pass:
        re-runs the rebin only when the camera, splat count or viewport
        changed (or always-rebin is on).  Returns whether it rebinned."""
        if self.scene.splats is None:
            return False
        n = self.scene.splats.splatCount
        w, h = max(1, int(frame.width)), max(1, int(frame.height))
        self.tileCountX = -(-w // self.tileSizeX)
        self.tileCountY = -(-h // self.tileSizeY)
        count_changed = n != self.lastSplatCount
        self.lastSplatCount = n
        viewport_changed = (w, h) != self.lastViewport
        self.lastViewport = (w, h)
        moved = frame.cameraVersion != self.lastCameraVersion
        self.lastCameraVersion = frame.cameraVersion
        if self.alwaysRebin or moved or count_changed or viewport_changed:
            self.rebin(n, self.tileCountX, self.tileCountY, w, h,
                       self._uniform(frame.camera, w, h))
            return True
        return False

    def rebin(self, splatCount, tilesX, tilesY, viewportWidth, viewportHeight,
              camera_uniform: np.ndarray, check: bool = True) -> None:
        """rebin (:1104-1266): all six stages.  On a key-capacity overflow the
        library grows its buffers and the rebin is issued again, so the
        result is never truncated."""
        cam = camera_struct(camera_uniform)
        self.viewport = (viewportWidth, viewportHeight)
        self.tileCountX, self.tileCountY = tilesX, tilesY
        for _ in range(3):
            self._call("gs3d_rebin", C.byref(cam), viewportWidth, viewportHeight)
            if not check:
                return
            rc = self.lib.gs3d_synchronize(self.ctx)
            if rc == _lib.ERR_CAPACITY:
                continue
            _check(self.lib, self.ctx, rc)
            return
        _check(self.lib, self.ctx, rc)

    def loadPly(self, source, newScene: bool = False) -> tuple[int, dict]:
        """SceneLoader.startLoadSplats + SceneWorker.parseGaussianSplatPly
        (SceneLoader.ts:75-88, SceneWorker.ts:146-550): parses the PLY at
        `source` (a path or bytes) and decodes it on the device into the
        scene (scene 0, like setSplatData, or a new scene for batched views).
        Returns (scene id, header info with position bounds)."""
        from . import ply
        if isinstance(source, (bytes, bytearray, memoryview)):
            data = np.frombuffer(source, np.uint8)
        else:
            data = np.fromfile(source, np.uint8)
        info = _lib.PlyInfo_t()
        out = C.c_uint32()
        self._call("gs3d_load_ply", data.ctypes.data_as(C.c_void_p), data.nbytes,
                   _lib.PLY_NEW_SCENE if newScene else 0, C.byref(out), C.byref(info))
        d = ply.info_dict(info)
        if not newScene or self.scene.splats is None:
            self.scene.splats = DeviceSplats(d["splat_count"], d["sh_degree"])
            self.lastSplatCount = -1  # force a rebin
        return int(out.value), d

    # ---- batched rendering (extension) -----------------------------------------
    def addScene(self, data: GaussianSplatData) -> int:
        """Makes another scene resident; returns its id for batched views."""
        arrs = [np.ascontiguousarray(a, np.float32) for a in
                (data.positions, data.scales, data.rotations, data.colors)]
        deg = int(data.sphericalHarmonicsDegree)
        sh = np.ascontiguousarray(data.sphericalHarmonics, np.float32) if deg > 0 else None
        ptr = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
        out = C.c_uint32()
        self._call("gs3d_add_scene", data.splatCount, *(ptr(a) for a in arrs), ptr(sh), deg, 0,
                   C.byref(out))
        if self.scene.splats is None:
            self.scene.splats = data
        return int(out.value)

    def rebinBatch(self, views, check: bool = True) -> None:
        """views: iterable of (scene_id, camera_uniform_72, width, height)."""
        views = list(views)
        arr = (_lib.View_t * len(views))()
        for i, (scene, u, w, h) in enumerate(views):
            arr[i].camera = camera_struct(u)
            arr[i].scene = int(scene)
            arr[i].width = int(w)
            arr[i].height = int(h)
        self._batch = len(views)
        for _ in range(3):
            self._call("gs3d_rebin_batch", C.cast(arr, C.c_void_p), len(views))
            if not check:
                return
            rc = self.lib.gs3d_synchronize(self.ctx)
            if rc == _lib.ERR_CAPACITY:
                continue
            _check(self.lib, self.ctx, rc)
            return
        _check(self.lib, self.ctx, rc)

    def viewInfo(self, v: int) -> _lib.ViewInfo_t:
        info = _lib.ViewInfo_t()
        self._call("gs3d_get_view_info", int(v), C.byref(info))
        return info

    def readViewImage(self, v: int) -> np.ndarray:
        info = self.viewInfo(v)
        n = (info.pixel_offset + info.width * info.height) * 4
        flat = np.zeros(n, np.float16)
        self._call("gs3d_read_buffer", _lib.BUFFERS["splat_target"],
                   flat.ctypes.data_as(C.c_void_p), flat.nbytes)
        return flat[info.pixel_offset * 4:].reshape(info.height, info.width, 4)

    def readViewRefs(self, v: int):
        """(keys, values, tile counts) of view v in single-view terms: tile ids
        relative to the view, values as scene splat ids."""
        info = self.viewInfo(v)
        t0, t1 = info.tile_base, info.tile_base + info.tiles_x * info.tiles_y
        total = self._total_tiles()
        off = np.zeros(total + 1, np.uint32)
        self._call("gs3d_read_buffer", _lib.BUFFERS["tile_offsets"],
                   off.ctypes.data_as(C.c_void_p), off.nbytes)
        o = off.astype(np.int64)
        all_counts = np.maximum(o[1:] - o[:-1], 0)  # exact: trailing tiles hold no refs
        a = int(all_counts[:t0].sum())
        b = a + int(all_counts[t0:t1].sum())
        k = np.zeros((b - a, 2), np.uint32)
        vals = np.zeros(b - a, np.uint32)
        self._call("gs3d_read_buffer_range", _lib.BUFFERS["sort_keys_a"], 8 * a,
                   k.ctypes.data_as(C.c_void_p), k.nbytes)
        self._call("gs3d_read_buffer_range", _lib.BUFFERS["sort_values_a"], 4 * a,
                   vals.ctypes.data_as(C.c_void_p), vals.nbytes)
        k[:, 0] -= t0
        return k, vals - info.splat_base, all_counts[t0:t1]

    def _total_tiles(self) -> int:
        last = self.viewInfo(self._batch - 1)
        return last.tile_base + last.tiles_x * last.tiles_y

    # ---- individual stages (for stage-wise parity) --------------------------
    def setCamera(self, camera_uniform, width, height) -> None:
        cam = camera_struct(camera_uniform)
        self._call("gs3d_set_camera", C.byref(cam), int(width), int(height))
        self.viewport = (int(width), int(height))
        self.tileCountX = -(-int(width) // self.tileSizeX)
        self.tileCountY = -(-int(height) // self.tileSizeY)

    def preprocess(self):
        self._call("gs3d_preprocess")

    def prefixScan(self):
        self._call("gs3d_prefix_scan")

    def emitTileRefs(self):
        self._call("gs3d_emit_tile_refs")

    def radixSort(self):
        self._call("gs3d_radix_sort")

    def identifyTileRanges(self):
        self._call("gs3d_identify_tile_ranges")

    def rasterizeTiles(self):
        self._call("gs3d_rasterize_tiles")

    def synchronize(self) -> None:
        self._call("gs3d_synchronize")

    # ---- buffers ---------------------------------------------------------------
    def refCount(self) -> int:
        v = C.c_uint32()
        self._call("gs3d_ref_count", C.byref(v))
        return int(v.value)

    def bufferInfo(self, name: str) -> tuple[int, int]:
        p, b = C.c_void_p(), C.c_size_t()
        self._call("gs3d_buffer_info", _lib.BUFFERS[name], C.byref(p), C.byref(b))
        return int(p.value or 0), int(b.value)

    def readBuffer(self, name: str, count: int | None = None) -> np.ndarray:
        """Copies a named buffer out in the reference's layout."""
        n = self.scene.splats.splatCount if self.scene.splats else 0
        tiles = self.tileCountX * self.tileCountY
        w, h = self.viewport
        if name in ("sort_keys_a", "sort_values_a", "sort_keys_b", "sort_values_b"):
            count = self.refCount() if count is None else count
        deg = self.scene.splats.sphericalHarmonicsDegree if self.scene.splats else 0
        shapes = {
            "splat_positions": (np.float32, (n, 4)), "splat_scales": (np.float32, (n, 4)),
            "splat_rotations": (np.float32, (n, 4)), "splat_colors": (np.float32, (n, 4)),
            "splat_sh_rest": (np.float32, (n, 3 * ((deg + 1) ** 2 - 1))),
            "projected_splats": (PROJ_DTYPE, (n,)),
            "splat_ref_counts": (np.uint32, (n,)),
            "splat_ref_offsets": (np.uint32, (n + 1,)),
            "ref_counter": (np.uint32, (1,)),
            "sort_keys_a": (np.uint32, (count, 2)), "sort_keys_b": (np.uint32, (count, 2)),
            "sort_values_a": (np.uint32, (count,)), "sort_values_b": (np.uint32, (count,)),
            "tile_offsets": (np.uint32, (tiles + 1,)),
            "splat_target": (np.float16, (h, w, 4)),
            "tile_costs": (np.uint32, (tiles,)),
        }
        dtype, shape = shapes[name]
        out = np.zeros(shape, dtype)
        self._call("gs3d_read_buffer", _lib.BUFFERS[name], out.ctypes.data_as(C.c_void_p),
                   out.nbytes)
        return out

    def writeBuffer(self, name: str, data: np.ndarray) -> None:
        data = np.ascontiguousarray(data)
        self._call("gs3d_write_buffer", _lib.BUFFERS[name], data.ctypes.data_as(C.c_void_p),
                   data.nbytes)

    def readImage(self) -> np.ndarray:
        return self.readBuffer("splat_target")

    def composite(self, view: int = 0, heatmap: bool = False, background=(0.0, 0.0, 0.0, 1.0),
                  debugRef: int = 256) -> np.ndarray:
        """The composite pass (and, with heatmap, the splats-per-tile overlay
        pass before it) rendered headless over a premultiplied background:
        (H, W, 4) uint8 RGBA."""
        info = self.viewInfo(view)
        out = np.zeros((info.height, info.width, 4), np.uint8)
        bg = np.ascontiguousarray(background, np.float32)
        self._call("gs3d_composite", int(view),
                   _lib.COMPOSITE_TILE_HEATMAP if heatmap else _lib.COMPOSITE_SPLATS,
                   int(debugRef), bg.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p),
                   out.nbytes, 0)
        return out

    def saveComposite(self, path, **kw) -> np.ndarray:
        """composite() written to a PNG file."""
        from .image import write_png
        img = self.composite(**kw)
        write_png(path, img)
        return img

    def readTileCounts(self) -> np.ndarray:
        """readTileCounts (:1278-1310): max(0, off[t+1] - off[t]) per tile."""
        tiles = self.tileCountX * self.tileCountY
        out = np.zeros(tiles, np.uint32)
        self._call("gs3d_read_tile_counts", out.ctypes.data_as(C.c_void_p), tiles)
        return out


class DeviceSplats:
    """A scene whose splat arrays live only on the device (loadPly)."""

    def __init__(self, count: int, sh_degree: int):
        self.splatCount = int(count)
        self.sphericalHarmonicsDegree = int(sh_degree)


class SceneSyncer:
    """src/SceneSyncer.ts: pushes the scene's splat SoA into the renderer."""

    def __init__(self, scene: Scene, renderer: GaussianSplatRenderer):
        self.scene = scene
        self.renderer = renderer

    def setSplatData(self) -> None:
        if self.scene.splats is None:
            return
        self.renderer.setSplatData(self.scene.splats)
