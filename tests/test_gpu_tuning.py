"""Tuning knobs (tile size, tile-id digit width, raster batch depth) and the
autotuner: every tuning renders the bit-identical image, and under any
tuning the keys, values and tile ranges equal the oracle's for that tile
grid."""
import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Gs3dError, Scene, scenes
from gs3d import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


def _views(n, sizes):
    eyes = scenes.orbit_eyes(n, radius=10.0, jitter_deg=15.0, seed=3)
    return [(0, scenes.camera_at(eyes[i], w, h).getUniformData(w, h), w, h)
            for i, (w, h) in enumerate(sizes)]


def _images(r, views):
    return [r.readViewImage(v) for v in range(len(views))]


def test_every_tuning_renders_the_same_image(renderer):
    data = scenes.scene_clusters(150_000, seed=7, sh_degree=1)
    renderer.setSplatData(data)
    views = _views(3, [(640, 360), (1280, 720), (333, 217)])
    renderer.setTuning(16, 8, 0)
    renderer.rebinBatch(views)
    want = _images(renderer, views)
    for tile in (8, 16, 32, (32, 64), (64, 32)):
        for digit in (4, 6, 8, 11):
            for batch in (0, 64, 512):
                renderer.setTuning(tile, digit, batch)
                renderer.rebinBatch(views)
                got = _images(renderer, views)
                for v in range(len(views)):
                    assert np.array_equal(got[v].view(np.uint16), want[v].view(np.uint16)), \
                        (tile, digit, batch, v)
    renderer.setTuning(16, 8, 0)


@pytest.mark.parametrize("tile,digit,batch", [(8, 6, 128), (32, 6, 512), (16, 6, 64),
                                              (16, 4, 256), (8, 4, 0), (8, 11, 256),
                                              (16, 11, 0), (32, 11, 512)])
def test_tuned_keys_match_the_oracle(renderer, oracle, tile, digit, batch):
    """Single-view fused rebin under a non-default tuning: sorted keys,
    values and tile_offsets bit-exact with the oracle's for that tile grid."""
    data = scenes.scene_small(60_000, seed=11)
    w, h = 1000, 563
    u = scenes.small_camera(w, h).getUniformData(w, h)
    o = oracle.rebin(u, w, h, tile, tile, data.positions, data.scales, data.rotations,
                     data.colors, data.sphericalHarmonics, data.sphericalHarmonicsDegree)
    renderer.setSplatData(data)
    renderer.setTuning(tile, digit, batch)
    renderer.rebin(data.splatCount, -(-w // tile), -(-h // tile), w, h, u)
    R = renderer.refCount()
    assert R == o["ref_counter"]
    assert np.array_equal(renderer.readBuffer("sort_keys_a", R), o["sort_keys_a"])
    assert np.array_equal(renderer.readBuffer("sort_values_a", R), o["sort_values_a"])
    assert np.array_equal(renderer.readBuffer("tile_offsets"), o["tile_offsets"])
    img = renderer.readImage().astype(np.float32)
    assert np.abs(img - o["image"]).max() <= 2.0 / 255.0
    # tile costs (32x32 tiles are shaded by four strip CTAs whose costs
    # combine by maximum); exp() rounding at the cut-offs moves a few
    gc = renderer.readBuffer("tile_costs").astype(np.int64)
    oc = o["tile_costs"].astype(np.int64)
    assert np.mean(gc == oc) >= 0.98
    assert np.abs(gc - oc).sum() <= 0.01 * max(1, oc.sum())
    renderer.setTuning(16, 8, 0)


@pytest.mark.parametrize("tw,th,digit,batch", [(32, 64, 8, 256), (64, 32, 8, 0),
                                                (128, 16, 6, 512), (32, 64, 11, 128)])
def test_wide_tiles_match_the_oracle(renderer, oracle, tw, th, digit, batch):
    """2048-pixel tiles (tuning API only: shaded by the two-pixel raster as
    row strips of at most 512 threads): keys, values and tile ranges
    bit-exact with the oracle's for that grid, the image within tolerance,
    tile costs as the oracle counts them."""
    data = scenes.scene_small(60_000, seed=11)
    w, h = 1000, 563
    u = scenes.small_camera(w, h).getUniformData(w, h)
    o = oracle.rebin(u, w, h, tw, th, data.positions, data.scales, data.rotations,
                     data.colors, data.sphericalHarmonics, data.sphericalHarmonicsDegree)
    renderer.setSplatData(data)
    renderer.setTuning((tw, th), digit, batch)
    try:
        renderer.rebin(data.splatCount, -(-w // tw), -(-h // th), w, h, u)
        R = renderer.refCount()
        assert R == o["ref_counter"]
        assert np.array_equal(renderer.readBuffer("sort_keys_a", R), o["sort_keys_a"])
        assert np.array_equal(renderer.readBuffer("sort_values_a", R), o["sort_values_a"])
        assert np.array_equal(renderer.readBuffer("tile_offsets"), o["tile_offsets"])
        img = renderer.readImage().astype(np.float32)
        assert np.abs(img - o["image"]).max() <= 2.0 / 255.0
        gc = renderer.readBuffer("tile_costs").astype(np.int64)
        oc = o["tile_costs"].astype(np.int64)
        assert np.mean(gc == oc) >= 0.98
        assert np.abs(gc - oc).sum() <= 0.01 * max(1, oc.sum())
        # the stage-wise rebin's one-pixel raster cannot shade them
        renderer.setStagewise(True)
        with pytest.raises(Gs3dError) as ei:
            renderer.rebin(data.splatCount, -(-w // tw), -(-h // th), w, h, u)
        assert ei.value.code == _lib.ERR_INVALID_ARG
    finally:
        renderer.setStagewise(False)
        renderer.setTuning(16, 8, 0)


@pytest.mark.parametrize("w,h", [(2048, 300), (2400, 300), (300, 2100)])
def test_tile_grids_wider_than_256_match_the_oracle(renderer, oracle, w, h):
    """Grids of more than 256 tiles on an axis keep the emit's tile
    rectangles in the projected records instead of one-word rectangles
    (2048 px at 8 px tiles is the largest one-word grid); keys, values and
    ranges stay bit-exact, alone and batched with a view whose grid fits
    the one-word form."""
    tile = 8
    data = scenes.scene_small(60_000, seed=13)
    u = scenes.small_camera(w, h).getUniformData(w, h)
    o = oracle.rebin(u, w, h, tile, tile, data.positions, data.scales, data.rotations,
                     data.colors, data.sphericalHarmonics, data.sphericalHarmonicsDegree)
    renderer.setSplatData(data)
    renderer.setTuning(tile, 8, 0)
    renderer.rebin(data.splatCount, -(-w // tile), -(-h // tile), w, h, u)
    R = renderer.refCount()
    assert R == o["ref_counter"]
    assert np.array_equal(renderer.readBuffer("sort_keys_a", R), o["sort_keys_a"])
    assert np.array_equal(renderer.readBuffer("sort_values_a", R), o["sort_values_a"])
    assert np.array_equal(renderer.readBuffer("tile_offsets"), o["tile_offsets"])
    img = renderer.readImage()
    small = scenes.small_camera(640, 360).getUniformData(640, 360)
    renderer.rebinBatch([(0, small, 640, 360), (0, u, w, h)])
    assert np.array_equal(renderer.readViewImage(1).view(np.uint16), img.view(np.uint16))
    renderer.rebinBatch([(0, small, 640, 360)])
    alone = renderer.readViewImage(0)
    renderer.rebinBatch([(0, small, 640, 360), (0, u, w, h)])
    assert np.array_equal(renderer.readViewImage(0).view(np.uint16), alone.view(np.uint16))
    renderer.setTuning(16, 8, 0)


def test_autotune_applies_the_fastest_candidate(renderer):
    data = scenes.scene_clusters(200_000, seed=2, sh_degree=0)
    renderer.setSplatData(data)
    views = _views(2, [(1280, 720), (960, 540)])
    renderer.setTuning(16, 8, 0)
    renderer.rebinBatch(views)
    want = _images(renderer, views)
    res = renderer.autotune(views, reps=2)
    assert len(res) == 5 * 3 * 3
    assert all(r["ms_per_view"] > 0 for r in res)
    best = renderer.getTuning()
    assert (best["tile"], best["digit_bits"], best["raster_batch"]) == \
        (res[0]["tile"], res[0]["digit_bits"], res[0]["raster_batch"])
    # fewer refs with larger tiles; the 6-bit digit never needs fewer passes
    by = {(r["tile"][0], r["digit_bits"], r["raster_batch"]): r for r in res}
    assert by[(32, 8, 256)]["refs"] < by[(16, 8, 256)]["refs"] < by[(8, 8, 256)]["refs"]
    assert by[(16, 4, 256)]["tile_passes"] >= by[(16, 8, 256)]["tile_passes"] >= \
        by[(16, 11, 256)]["tile_passes"]
    renderer.rebinBatch(views)
    got = _images(renderer, views)
    for v in range(len(views)):
        assert np.array_equal(got[v].view(np.uint16), want[v].view(np.uint16))
    renderer.setTuning(16, 8, 0)


def test_bad_tunings_are_rejected(renderer):
    for bad in [(16, 7, 0), (16, 12, 0), (16, 8, 48), (16, 8, 2048), (64, 8, 0),
                ((64, 24), 8, 0), ((60, 32), 8, 0), ((128, 32), 8, 0)]:
        with pytest.raises(Gs3dError) as ei:
            renderer.setTuning(*bad)
        assert ei.value.code == _lib.ERR_INVALID_ARG
    renderer.setTuning(16, 8, 0)
