"""Batched rebin (many views, several scenes, uneven sizes, one launch
sequence) and raster schedules: every view's sorted keys, values, tile counts
and image are bit-identical to a single-view rebin of that view, and the
image does not depend on the raster work order."""
import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Scene, scenes
from gs3d import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


def single(r, data, u, w, h):
    r.setSplatData(data)
    r.rebin(data.splatCount, -(-w // 16), -(-h // 16), w, h, u)
    R = r.refCount()
    off = r.readBuffer("tile_offsets").astype(np.int64)
    return (r.readBuffer("sort_keys_a", R), r.readBuffer("sort_values_a", R),
            np.maximum(off[1:] - off[:-1], 0), r.readImage())


def test_batch_matches_single_views(renderer, oracle):
    r = renderer
    r.setTileSize(16, 16)
    a = scenes.scene_clusters(60_000, seed=1, sh_degree=3)
    b = scenes.scene_small(40_000, seed=2)
    r.setSplatData(a)            # scene 0
    sb = r.addScene(b)           # scene 1
    eyes = scenes.random_eyes(5, 8.0, 16.0, seed=3)
    sizes = [(640, 360), (1280, 720), (333, 217), (960, 540), (200, 640)]
    views = []
    for i, (eye, (w, h)) in enumerate(zip(eyes, sizes)):
        sc = 0 if i % 2 == 0 else sb
        views.append((sc, scenes.camera_at(eye, w, h).getUniformData(w, h), w, h))
    r.rebinBatch(views)
    got = [(r.readViewRefs(v), r.readViewImage(v)) for v in range(len(views))]
    for v, (sc, u, w, h) in enumerate(views):
        data = a if sc == 0 else b
        (k, val, cnt), img = got[v]
        k1, v1, c1, img1 = single(r, data, u, w, h)
        assert np.array_equal(k, k1) and np.array_equal(val, v1), v
        assert np.array_equal(cnt, c1), v
        assert np.array_equal(img.view(np.uint16), img1.view(np.uint16)), v
        if v == 2:  # and one view against the oracle
            o = oracle.rebin(u, w, h, 16, 16, data.positions, data.scales, data.rotations,
                             data.colors, data.sphericalHarmonics, data.sphericalHarmonicsDegree)
            assert np.array_equal(k, o["sort_keys_a"]) and np.array_equal(val, o["sort_values_a"])
            assert np.abs(img.astype(np.float32) - o["image"]).max() <= 2 / 255


@pytest.mark.parametrize("schedule", [_lib.SCHEDULE_KEY_COUNT])
def test_schedule_leaves_image_unchanged(renderer, schedule):
    r = renderer
    data = scenes.scene_clusters(200_000, seed=4, sh_degree=0)
    w, h = 1280, 720
    u = scenes.camera_at((1.0, 2.0, 9.0), w, h).getUniformData(w, h)
    r.setSchedule(_lib.SCHEDULE_ROW_MAJOR)
    _, _, _, img0 = single(r, data, u, w, h)
    c0 = r.readBuffer("tile_costs")
    r.setSchedule(schedule)
    _, _, _, img1 = single(r, data, u, w, h)
    c1 = r.readBuffer("tile_costs")
    r.setSchedule(_lib.SCHEDULE_ROW_MAJOR)
    assert np.array_equal(img0.view(np.uint16), img1.view(np.uint16))
    assert np.array_equal(c0, c1)


def test_cuda_graph_replay_matches_eager(renderer):
    """Graph mode: first call captures, later calls replay with new cameras;
    every replay equals the eager batched rebin bit for bit."""
    r = renderer
    r.setTileSize(16, 16)
    a = scenes.scene_clusters(80_000, seed=8, sh_degree=2)
    r.setSplatData(a)
    sizes = [(640, 360), (1280, 720), (480, 480)]
    outs = {}
    for graph in (False, True):
        r.setCudaGraph(graph)
        for rep in range(3):
            eyes = scenes.random_eyes(3, 8.0, 14.0, seed=20 + rep)
            views = [(0, scenes.camera_at(e, w, h).getUniformData(w, h), w, h)
                     for e, (w, h) in zip(eyes, sizes)]
            r.rebinBatch(views)
            outs[(graph, rep)] = [(r.readViewRefs(v), r.readViewImage(v)) for v in range(3)]
    r.setCudaGraph(False)
    for rep in range(3):
        for v in range(3):
            (k0, v0, c0), i0 = outs[(False, rep)][v]
            (k1, v1, c1), i1 = outs[(True, rep)][v]
            assert np.array_equal(k0, k1) and np.array_equal(v0, v1) and np.array_equal(c0, c1)
            assert np.array_equal(i0.view(np.uint16), i1.view(np.uint16))
