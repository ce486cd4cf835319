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


def gpu_frame(r, data, uniform, w, h, tw=16, th=16, stagewise=False):
    r.setTileSize(tw, th)
    r.setSplatData(data)
    r.setStagewise(stagewise)
    tx, ty = -(-w // tw), -(-h // th)
    r.rebin(data.splatCount, tx, ty, w, h, uniform)
    r.setStagewise(False)
    R = r.refCount()
    return dict(
        projected_splats=r.readBuffer("projected_splats"),
        splat_ref_counts=r.readBuffer("splat_ref_counts"),
        splat_ref_offsets=r.readBuffer("splat_ref_offsets") if stagewise else None,
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
    if g["splat_ref_offsets"] is not None:  # stage-wise path: reference splat order
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


@pytest.mark.parametrize("stagewise", [False, True])
def test_small_scene_end_to_end(renderer, oracle, stagewise):
    """The small benchmark scene: 100k splats, SH 0, 1280x720, 16x16 tiles,
    through the fused rebin and through the six reference stages."""
    data = scenes.scene_small(100_000, seed=0)
    u = scenes.small_camera().getUniformData(1280, 720)
    o = oracle_frame(oracle, data, u, 1280, 720, 16, 16)
    g = gpu_frame(renderer, data, u, 1280, 720, stagewise=stagewise)
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
                                       (333, 217, 12, 20), (17, 9, 16, 16), (4000, 40, 4, 4),
                                       # 1024-pixel tiles shaded by one, two or four strip CTAs
                                       (1000, 563, 128, 8), (900, 500, 64, 16), (700, 450, 16, 64)])
@pytest.mark.parametrize("stagewise", [False, True])
def test_ragged_viewports_and_tile_sizes(renderer, oracle, w, h, tw, th, stagewise):
    data = scenes.scene_small(40_000, seed=5)
    u = scenes.small_camera(w, h).getUniformData(w, h)
    o = oracle_frame(oracle, data, u, w, h, tw, th)
    g = gpu_frame(renderer, data, u, w, h, tw, th, stagewise=stagewise)
    assert_frame_match(g, o)
    renderer.setTileSize(16, 16)


@pytest.mark.parametrize("stagewise", [False, True])
def test_empty_scene(renderer, stagewise):
    z = np.zeros((0, 4), np.float32)
    data = scenes.GaussianSplatData(z, z, z, z, None, 0, 0)
    u = scenes.small_camera(320, 200).getUniformData(320, 200)
    g = gpu_frame(renderer, data, u, 320, 200, stagewise=stagewise)
    assert g["ref_counter"] == 0
    assert not g["tile_offsets"].any() and not g["image"].any()


@pytest.mark.parametrize("stagewise", [False, True])
def test_everything_culled(renderer, stagewise):
    data = scenes.scene_small(10_000, seed=1)
    u = scenes.camera_at((0, 0, 30), 320, 200, target=(0, 0, 60)).getUniformData(320, 200)
    g = gpu_frame(renderer, data, u, 320, 200, stagewise=stagewise)
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


def test_fused_equals_stagewise_at_full_size(renderer):
    """The 3M-splat SH-3 1080p workload: the fused rebin and the six-stage
    rebin give bit-identical sorted keys, values, tile ranges and images, and
    the result satisfies the size-independent properties of a correct sort."""
    data = scenes.scene_clusters(3_000_000, seed=0, sh_degree=3)
    w, h = 1920, 1080
    u = scenes.camera_at(scenes.orbit_eyes(64)[5], w, h).getUniformData(w, h)
    out = []
    for sw in (False, True):
        renderer.setTileSize(16, 16)
        renderer.setSplatData(data)
        renderer.setStagewise(sw)
        renderer.rebin(data.splatCount, 120, 68, w, h, u)
        R = renderer.refCount()
        out.append((R, renderer.readBuffer("sort_keys_a", R), renderer.readBuffer("sort_values_a", R),
                    renderer.readBuffer("tile_offsets"), renderer.readImage(),
                    renderer.readBuffer("splat_ref_counts"), renderer.readBuffer("projected_splats")))
    renderer.setStagewise(False)
    (R, k, v, t, img, cnt, proj), (R2, k2, v2, t2, img2, _, _) = out
    assert R == R2 and R == int(cnt.astype(np.int64).sum()) and R > 10_000_000
    assert np.array_equal(k, k2) and np.array_equal(v, v2)
    assert np.array_equal(t, t2) and np.array_equal(img.view(np.uint16), img2.view(np.uint16))
    # sortedness: (tile, depth bits, splat id) strictly increasing
    key64 = (k[:, 0].astype(np.uint64) << np.uint64(32)) | k[:, 1].astype(np.uint64)
    d = np.diff(key64.astype(np.float64))  # exactness not needed for the sign test below
    same = key64[1:] == key64[:-1]
    assert np.all((key64[1:] > key64[:-1]) | (same & (v[1:] > v[:-1])))
    # every ref names a valid splat whose depth bits and tile rectangle match
    assert np.all(proj["valid"][v] == 1)
    assert np.array_equal(k[:, 1], (-proj["depth"][v]).view(np.uint32))
    tx, ty = k[:, 0] % 120, k[:, 0] // 120
    assert np.all((proj["tile_min"][v, 0] <= tx) & (tx <= proj["tile_max"][v, 0]))
    assert np.all((proj["tile_min"][v, 1] <= ty) & (ty <= proj["tile_max"][v, 1]))
    # per-splat ref multiplicity equals its count
    assert np.array_equal(np.bincount(v, minlength=len(cnt)), cnt)
    del d
