"""GPU parity of every rebin stage against the CPU oracle, through the C ABI.

Tolerances (from the path's specification):
  * scan offsets, ref counts, emitted keys/values, sorted order and
    tile_offsets: bit-exact given the same projected splats;
  * projected means, conics and colours: <= 1e-5 relative (the library's
    preprocess is in fact compared bit for bit as well);
  * images: <= 2/255 max-abs per channel.
"""
import math

import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Gs3dError, Scene, scenes
from gs3d import _lib

pytestmark = pytest.mark.gpu

IMG_TOL = 2.0 / 255.0
REL_TOL = 1e-5


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


def oracle_frame(oracle, data, uniform, w, h, tw, th):
    return oracle.rebin(uniform, w, h, tw, th, data.positions, data.scales, data.rotations,
                        data.colors, data.sphericalHarmonics, data.sphericalHarmonicsDegree)


def gpu_frame(r, data, uniform, w, h, tw=16, th=16):
    r.setTileSize(tw, th)
    r.setSplatData(data)
    tx, ty = -(-w // tw), -(-h // th)
    r.rebin(data.splatCount, tx, ty, w, h, uniform)
    R = r.refCount()
    return dict(
        projected_splats=r.readBuffer("projected_splats"),
        splat_ref_counts=r.readBuffer("splat_ref_counts"),
        splat_ref_offsets=r.readBuffer("splat_ref_offsets"),
        ref_counter=R,
        sort_keys_a=r.readBuffer("sort_keys_a", R),
        sort_values_a=r.readBuffer("sort_values_a", R),
        tile_offsets=r.readBuffer("tile_offsets"),
        image=r.readImage().astype(np.float32),
        tile_costs=r.readBuffer("tile_costs"),
    )


def assert_projected_match(g, o):
    assert np.array_equal(g["valid"], o["valid"])
    v = o["valid"] == 1
    for f in ("tile_min", "tile_max"):
        assert np.array_equal(g[f][v], o[f][v]), f
    for f in ("mean_px", "depth", "radius_px", "conic", "opacity", "color"):
        a, b = g[f][v].astype(np.float64), o[f][v].astype(np.float64)
        err = np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
        err = np.where(np.abs(a - b) <= 1e-30, 0.0, err)
        assert err.max(initial=0.0) <= REL_TOL, (f, err.max())


def assert_frame_match(g, o, exact_preprocess=True):
    assert_projected_match(g["projected_splats"], o["projected_splats"])
    if exact_preprocess:
        assert g["projected_splats"].tobytes() == o["projected_splats"].tobytes()
    assert np.array_equal(g["splat_ref_counts"], o["splat_ref_counts"])
    assert np.array_equal(g["splat_ref_offsets"], o["splat_ref_offsets"])
    assert g["ref_counter"] == o["ref_counter"]
    assert np.array_equal(g["sort_keys_a"], o["sort_keys_a"])
    assert np.array_equal(g["sort_values_a"], o["sort_values_a"])
    assert np.array_equal(g["tile_offsets"], o["tile_offsets"])
    diff = np.abs(g["image"] - o["image"])
    assert diff.max(initial=0.0) <= IMG_TOL, diff.max()
    # tile costs depend on the exp() rounding at the 1/255 and 1e-4 cut-offs
    gc, oc = g["tile_costs"].astype(np.int64), o["tile_costs"].astype(np.int64)
    assert np.mean(gc == oc) >= 0.98
    assert np.abs(gc - oc).sum() <= 0.01 * max(1, oc.sum())


def test_small_scene_end_to_end(renderer, oracle):
    """The small benchmark scene: 100k splats, SH 0, 1280x720, 16x16 tiles."""
    data = scenes.scene_small(100_000, seed=0)
    u = scenes.small_camera().getUniformData(1280, 720)
    o = oracle_frame(oracle, data, u, 1280, 720, 16, 16)
    g = gpu_frame(renderer, data, u, 1280, 720)
    assert o["ref_counter"] > 100_000
    assert_frame_match(g, o)


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_sh_colour_degrees(renderer, oracle, deg):
    data = scenes.scene_clusters(30_000, seed=deg, sh_degree=deg)
    u = scenes.camera_at(scenes.orbit_eyes(4, radius=12.0)[deg], 800, 600).getUniformData(800, 600)
    o = oracle_frame(oracle, data, u, 800, 600, 16, 16)
    g = gpu_frame(renderer, data, u, 800, 600)
    assert_frame_match(g, o)


@pytest.mark.parametrize("w,h,tw,th", [(1000, 563, 16, 16), (640, 360, 8, 8), (1024, 600, 32, 32),
                                       (333, 217, 12, 20), (17, 9, 16, 16)])
def test_ragged_viewports_and_tile_sizes(renderer, oracle, w, h, tw, th):
    data = scenes.scene_small(40_000, seed=5)
    u = scenes.small_camera(w, h).getUniformData(w, h)
    o = oracle_frame(oracle, data, u, w, h, tw, th)
    g = gpu_frame(renderer, data, u, w, h, tw, th)
    assert_frame_match(g, o)
    renderer.setTileSize(16, 16)


def test_empty_scene(renderer):
    z = np.zeros((0, 4), np.float32)
    data = scenes.GaussianSplatData(z, z, z, z, None, 0, 0)
    u = scenes.small_camera(320, 200).getUniformData(320, 200)
    g = gpu_frame(renderer, data, u, 320, 200)
    assert g["ref_counter"] == 0
    assert not g["tile_offsets"].any() and not g["image"].any()


def test_everything_culled(renderer):
    data = scenes.scene_small(10_000, seed=1)
    u = scenes.camera_at((0, 0, 30), 320, 200, target=(0, 0, 60)).getUniformData(320, 200)
    g = gpu_frame(renderer, data, u, 320, 200)
    assert g["ref_counter"] == 0 and not g["projected_splats"]["valid"].any()
    assert not g["image"].any()


def test_stagewise_from_oracle_projection(renderer, oracle):
    """Keys, sort and tile ranges bit-exact given the SAME projected splats:
    the oracle's ProjectedSplat buffer is fed into the GPU stages."""
    data = scenes.scene_clusters(50_000, seed=9, sh_degree=0)
    w, h = 960, 540
    u = scenes.camera_at((0.0, 2.0, 11.0), w, h).getUniformData(w, h)
    o = oracle_frame(oracle, data, u, w, h, 16, 16)
    r = renderer
    r.setTileSize(16, 16)
    r.setSplatData(data)
    r.setCamera(u, w, h)
    r.writeBuffer("projected_splats", o["projected_splats"])
    r.writeBuffer("splat_ref_counts", o["splat_ref_counts"])
    r.prefixScan()
    assert np.array_equal(r.readBuffer("splat_ref_offsets"), o["splat_ref_offsets"])
    r.emitTileRefs()
    R = r.refCount()
    assert R == o["ref_counter"]
    keys_e, vals_e = oracle.emit(r.getTileCount()[0], o["projected_splats"],
                                 o["splat_ref_offsets"], R)
    assert np.array_equal(r.readBuffer("sort_keys_a", R), keys_e)
    assert np.array_equal(r.readBuffer("sort_values_a", R), vals_e)
    r.radixSort()
    assert np.array_equal(r.readBuffer("sort_keys_a", R), o["sort_keys_a"])
    assert np.array_equal(r.readBuffer("sort_values_a", R), o["sort_values_a"])
    r.identifyTileRanges()
    assert np.array_equal(r.readBuffer("tile_offsets"), o["tile_offsets"])
    r.rasterizeTiles()
    diff = np.abs(r.readImage().astype(np.float32) - o["image"])
    assert diff.max() <= IMG_TOL
    counts = r.readTileCounts()
    off = o["tile_offsets"].astype(np.int64)
    assert np.array_equal(counts, np.maximum(off[1:] - off[:-1], 0))


@pytest.mark.parametrize("tiles_w,tiles_h,R", [(256, 256, 2_000_000), (3, 1, 300_000),
                                               (1, 1, 70_000), (120, 68, 4097)])
def test_radix_sort_random_keys(renderer, oracle, tiles_w, tiles_h, R):
    """Sort stage alone on random keys with heavy ties (all 2^k pass counts)."""
    rng = np.random.default_rng(R)
    data = scenes.scene_small(max(200_000, R // 8), seed=2)
    r = renderer
    r.setTileSize(16, 16)
    r.setSplatData(data)
    w, h = tiles_w * 16, tiles_h * 16
    r.setCamera(scenes.small_camera(w, h).getUniformData(w, h), w, h)
    keys = np.empty((R, 2), np.uint32)
    keys[:, 0] = rng.integers(0, tiles_w * tiles_h, R)
    keys[:, 1] = rng.integers(0, 1 << 31, R)
    keys[::3, 1] = np.float32(rng.uniform(1, 2)).view(np.uint32)  # ties
    vals = rng.permutation(R).astype(np.uint32)
    r.writeBuffer("sort_keys_a", keys)
    r.writeBuffer("sort_values_a", vals)
    r.writeBuffer("ref_counter", np.array([R], np.uint32))
    r.radixSort()
    order = np.lexsort((np.arange(R), keys[:, 1], keys[:, 0]))
    assert np.array_equal(r.readBuffer("sort_keys_a", R), keys[order])
    assert np.array_equal(r.readBuffer("sort_values_a", R), vals[order])


def test_capacity_overflow_grows_and_reruns(oracle, built_lib):
    """Key capacity starts at N refs (max_tiles_per_splat = 1): the first
    rebin overflows, is reported, the buffers grow, and the re-issued rebin
    matches the oracle - never a truncated result."""
    import ctypes as C
    from gs3d.camera import camera_struct
    data = scenes.scene_small(30_000, seed=4)
    w, h = 640, 480
    u = scenes.small_camera(w, h).getUniformData(w, h)
    lib = _lib.load()
    ctx = C.c_void_p()
    cfg = _lib.Config_t(0, 16, 16, 1, None, 0)
    assert lib.gs3d_create(C.byref(ctx), C.byref(cfg)) == 0
    try:
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        assert lib.gs3d_set_splats(ctx, data.splatCount, ptr(data.positions), ptr(data.scales),
                                   ptr(data.rotations), ptr(data.colors), None, 0, 0) == 0
        cam = camera_struct(u)
        assert lib.gs3d_rebin(ctx, C.byref(cam), w, h) == 0
        assert lib.gs3d_synchronize(ctx) == _lib.ERR_CAPACITY
        assert b"re-run" in lib.gs3d_last_error(ctx)
        assert lib.gs3d_rebin(ctx, C.byref(cam), w, h) == 0
        assert lib.gs3d_synchronize(ctx) == 0
        o = oracle_frame(oracle, data, u, w, h, 16, 16)
        R = C.c_uint32()
        assert lib.gs3d_ref_count(ctx, C.byref(R)) == 0 and R.value == o["ref_counter"]
        vals = np.zeros(R.value, np.uint32)
        assert lib.gs3d_read_buffer(ctx, 10, ptr(vals), vals.nbytes) == 0
        assert np.array_equal(vals, o["sort_values_a"])
    finally:
        lib.gs3d_destroy(ctx)


def test_change_gated_render(renderer):
    """render() re-bins only when the camera version, splat count or viewport
    changes (GaussianSplatRenderer.ts:1062-1073) or always-rebin is on."""
    from gs3d import RenderFrameInfo
    data = scenes.scene_small(5_000, seed=8)
    renderer.setTileSize(16, 16)
    renderer.setSplatData(data)
    cam = scenes.small_camera(320, 240)
    f = RenderFrameInfo(320, 240, cam, cam.version)
    assert renderer.render(f) is True
    assert renderer.render(f) is False
    cam.setPosition((0.0, 1.0, 6.0))
    assert renderer.render(RenderFrameInfo(320, 240, cam, cam.version)) is True
    renderer.setAlwaysRebin(True)
    assert renderer.render(RenderFrameInfo(320, 240, cam, cam.version)) is True
    renderer.setAlwaysRebin(False)


def test_errors_are_status_codes(renderer):
    _, nbytes = renderer.bufferInfo("tile_offsets")
    with pytest.raises(Gs3dError) as ei:
        renderer.writeBuffer("tile_offsets", np.zeros(nbytes // 4 + 1, np.uint32))
    assert ei.value.code == _lib.ERR_INVALID_ARG
    with pytest.raises(Gs3dError) as ei:
        renderer._call("gs3d_set_splats", 1, None, None, None, None, None, 0, 0)
    assert ei.value.code == _lib.ERR_INVALID_ARG
