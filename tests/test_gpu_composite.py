"""gs3d_composite (headless composite and tile heat map) against the oracle,
bit for bit, on single-view and batched frames."""
import ctypes as C

import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Scene, _lib, scenes
from gs3d.image import read_png
from oracle import composite_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


def _oracle_for(r, v, heatmap, ref, bg):
    info = r.viewInfo(v)
    img = r.readViewImage(v)
    T = info.tiles_x * info.tiles_y
    full = np.zeros(info.tile_base + T + 1, np.uint32)
    r._call("gs3d_read_buffer", _lib.BUFFERS["tile_offsets"],
            full.ctypes.data_as(C.c_void_p), full.nbytes)
    off = full[info.tile_base:info.tile_base + T + 1]
    tw, th = r.getTileSize()
    return composite_oracle.composite(img, off, tw, th, info.tiles_x, info.tiles_y,
                                      heatmap, ref, bg)


@pytest.mark.parametrize("heatmap", [False, True])
@pytest.mark.parametrize("bg", [(0.0, 0.0, 0.0, 1.0), (0.1, 0.2, 0.3, 1.0), (0, 0, 0, 0)])
def test_single_view_matches_oracle(renderer, heatmap, bg):
    data = scenes.scene_clusters(120_000, seed=3, sh_degree=2)
    renderer.setSplatData(data)
    cam = scenes.camera_at(scenes.orbit_eyes(3, radius=9.0)[2], 1000, 563)
    renderer.rebin(data.splatCount, 63, 36, 1000, 563, cam.getUniformData(1000, 563))
    got = renderer.composite(0, heatmap=heatmap, background=bg, debugRef=300)
    want = _oracle_for(renderer, 0, heatmap, 300, bg)
    np.testing.assert_array_equal(got, want)


def test_batched_views_and_png(renderer, tmp_path):
    data = scenes.scene_clusters(100_000, seed=8, sh_degree=1)
    renderer.setSplatData(data)
    eyes = scenes.orbit_eyes(3, radius=10.0, seed=1)
    sizes = [(640, 360), (333, 217), (800, 450)]
    views = [(0, scenes.camera_at(eyes[i], w, h).getUniformData(w, h), w, h)
             for i, (w, h) in enumerate(sizes)]
    renderer.rebinBatch(views)
    for v in range(3):
        for heatmap in (False, True):
            got = renderer.composite(v, heatmap=heatmap, background=(0.05, 0.05, 0.05, 1.0))
            want = _oracle_for(renderer, v, heatmap, 256, (0.05, 0.05, 0.05, 1.0))
            np.testing.assert_array_equal(got, want)
    path = tmp_path / "view1_heatmap.png"
    img = renderer.saveComposite(path, view=1, heatmap=True)
    np.testing.assert_array_equal(read_png(path), img)
