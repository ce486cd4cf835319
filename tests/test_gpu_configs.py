"""The batched and stress configurations at their full sizes, checked by
size-independent properties: every view of a mixed batch equals its
one-view rebin bit for bit (refs and image), the sorted keys keep the
(view, tile, depth) order, and the work order never changes an image.

  * batched: 4 scenes of 0.5M, 1M, 3M and 6M splats (cluster distribution,
    seeds 1-4, SH 3), 32 views per batch at sizes drawn from 640x360 ...
    3840x2160, random poses at radius 8-16, autotuned;
  * skewed stress: 10M splats (16 dense clusters + uniform background,
    heavy-tailed scales, SH 3) at 3840x2160, 8 close-up and 8 wide views,
    rendered in the largest batches whose refs fit one rebin's u32 indices.
"""
import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Gs3dError, Scene, _lib, scenes

pytestmark = pytest.mark.gpu

SIZES = [(640, 360), (1280, 720), (1920, 1080), (2560, 1440), (3840, 2160)]


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


def check_view_against_single(r, views, v):
    """View v of the current batch == the same view rendered alone."""
    k, vals, counts = r.readViewRefs(v)
    img = r.readViewImage(v).copy()
    # (tile, depth bits, splat) strictly ordered within the view
    key = (k[:, 0].astype(np.uint64) << np.uint64(32)) | k[:, 1].astype(np.uint64)
    assert np.all(key[1:] >= key[:-1])
    tie = key[1:] == key[:-1]
    assert np.all(vals[1:][tie] > vals[:-1][tie])
    batch = list(views)
    r.rebinBatch([batch[v]])
    k1, vals1, counts1 = r.readViewRefs(0)
    np.testing.assert_array_equal(k1, k)
    np.testing.assert_array_equal(vals1, vals)
    np.testing.assert_array_equal(counts1, counts)
    np.testing.assert_array_equal(r.readViewImage(0).view(np.uint16), img.view(np.uint16))
    r.rebinBatch(batch)


def test_batched_config_full_size(renderer):
    r = renderer
    ids = []
    for i, (n, seed) in enumerate(((500_000, 1), (1_000_000, 2), (3_000_000, 3),
                                   (6_000_000, 4))):
        data = scenes.scene_clusters(n, seed=seed, sh_degree=3)
        if i == 0:
            r.setSplatData(data)
            ids.append(0)
        else:
            ids.append(r.addScene(data))
    rng = np.random.default_rng(11)
    eyes = scenes.random_eyes(32, 8.0, 16.0, seed=11)
    views = []
    for i in range(32):
        w, h = SIZES[int(rng.integers(len(SIZES)))]
        views.append((ids[i % 4], scenes.camera_at(eyes[i], w, h).getUniformData(w, h), w, h))
    res = r.autotune(views, reps=1)
    assert res and res[0] == min(res, key=lambda x: x["ms_per_view"])
    best = r.getTuning()
    assert (best["tile"], best["digit_bits"], best["raster_batch"]) == \
        (res[0]["tile"], res[0]["digit_bits"], res[0]["raster_batch"])
    r.rebinBatch(views)
    # global tile ids: every view's grid follows the previous views' grids, so
    # the view is folded into the key's high bits
    base = 0
    for v in range(len(views)):
        info = r.viewInfo(v)
        assert info.tile_base == base
        base += info.tiles_x * info.tiles_y
    assert r.viewInfo(31).tile_base > 31 * min(r.viewInfo(v).tiles_x * r.viewInfo(v).tiles_y
                                               for v in range(31))
    # one view of each scene, including the 4K ones
    picks = {}
    for v, (sid, _, w, h) in enumerate(views):
        if sid not in picks or w > views[picks[sid]][2]:
            picks[sid] = v
    for v in sorted(picks.values()):
        check_view_against_single(r, views, v)
    r.setTuning(16, 8, 0)


def render_in_batches(r, views):
    """Renders views in the largest batches (halving when the refs exceed one
    rebin's limit); yields each rendered batch's view indices."""
    pending = [list(range(len(views)))]
    while pending:
        idx = pending.pop(0)
        try:
            r.rebinBatch([views[i] for i in idx])
        except Gs3dError as e:
            if e.code != _lib.ERR_CAPACITY or len(idx) == 1:
                raise
            h = len(idx) // 2
            pending[:0] = [idx[:h], idx[h:]]
            continue
        yield idx


def test_skewed_stress_full_size(renderer):
    r = renderer
    data = scenes.scene_skewed(10_000_000, seed=0, sh_degree=3)
    r.setSplatData(data)
    r.setTuning(32, 8, 512)
    W, H = 3840, 2160
    # close-ups inside the radius-20 background, near the radius-8 clusters:
    # about 1.1e9 refs for one 4K view at 32x32 tiles
    close = scenes.random_eyes(8, 3.0, 5.0, seed=21)
    wide = scenes.random_eyes(8, 28.0, 34.0, seed=22)
    views = [(0, scenes.camera_at(e, W, H).getUniformData(W, H), W, H)
             for e in np.concatenate([close, wide])]
    nz, batches = [], 0
    for idx in render_in_batches(r, views):
        batches += 1
        batch = [views[i] for i in idx]
        for j in range(len(idx)):
            _, _, counts = r.readViewRefs(j)
            nz.append(counts[counts > 0])
        for want in (0, 15):  # a close-up and a wide view
            if want in idx:
                j = idx.index(want)
                check_view_against_single(r, batch, j)
                # the raster order leaves the image unchanged
                img = r.readViewImage(j).copy()
                for sched in (_lib.SCHEDULE_KEY_COUNT, _lib.SCHEDULE_ROW_MAJOR):
                    r.setSchedule(sched)
                    r.rebinBatch(batch)
                    np.testing.assert_array_equal(r.readViewImage(j).view(np.uint16),
                                                  img.view(np.uint16))
                r.setSchedule(_lib.SCHEDULE_ROW_MAJOR)
    nz = np.concatenate(nz)
    # heavy-tailed footprints: a few large splats cover every tile, so the
    # non-empty tiles' key counts span about three orders of magnitude
    # (1411 .. 1,477,709 at 32x32, 1369 .. 931,826 at 16x16 on these poses)
    assert nz.max() / nz.min() >= 1e2
    print(f"skewed stress, 32x32 tiles: {batches} batches, "
          f"per-tile key counts {nz.min()}..{nz.max()}")
    # the same at the reference's 16x16 tiles (one close-up, one wide view)
    r.setTuning(16, 8, 0)
    nz16 = []
    for v in (0, 15):
        r.rebinBatch([views[v]])
        _, _, counts = r.readViewRefs(0)
        nz16.append(counts[counts > 0])
    nz16 = np.concatenate(nz16)
    print(f"16x16 tiles: per-tile key counts {nz16.min()}..{nz16.max()}")
    assert nz16.max() / nz16.min() >= 1e2
