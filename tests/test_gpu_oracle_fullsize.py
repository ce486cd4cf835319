"""The configurations the benchmark numbers are quoted on, diffed element by
element against the CPU oracle at their full sizes:

  * the headline scene (3M splats, SH 3, 1920x1080, orbit poses): two poses
    through the single-view fused rebin at the reference's 16x16 tiles, and
    two views of the headline 8-view batch at the autotuned 32x32 tiles,
    8-bit digits, 256-splat raster batches, learned raster order, replayed
    as a CUDA graph;
  * the batched configuration's largest scene: a 3840x2160 view of the
    6M-splat scene, batched with a 1280x720 view of the 0.5M-splat scene;
  * the skewed stress configuration: a wide 3840x2160 view of the 10M-splat
    scene (about 2.5e8 refs at 32x32 tiles).

Every view must give the oracle's ProjectedSplat records byte for byte,
its ref counts, sorted keys and values and tile ranges bit for bit, and an
image within 2/255 (rasterize_tiles.wgsl:44-110 and emit_tile_refs.wgsl:57-79
through the oracle).  Views of a batch are read in single-view terms (tile
ids relative to the view, values as scene splat ids, the view's tile ranges
rebuilt with identify's trailing-zero convention)."""
import ctypes as C

import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Scene, _lib, learned, scenes
from oracle import PROJ_DTYPE
from test_gpu_parity import assert_frame_match, gpu_frame, oracle_frame

pytestmark = pytest.mark.gpu

W1, H1 = 1920, 1080
W4, H4 = 3840, 2160


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


@pytest.fixture(scope="module")
def c1():
    return scenes.scene_clusters(3_000_000, seed=0, sh_degree=3)


def c1_uniform(pose):
    eyes = scenes.orbit_eyes(64, radius=12.0, jitter_deg=20.0, seed=0)
    return scenes.camera_at(eyes[pose], W1, H1).getUniformData(W1, H1)


def read_range(r, name, offset_bytes, dtype, count):
    out = np.zeros(count, dtype)
    r._call("gs3d_read_buffer_range", _lib.BUFFERS[name], offset_bytes,
            out.ctypes.data_as(C.c_void_p), out.nbytes)
    return out


def tile_offsets_from_counts(counts):
    """tile_offsets as identify writes them for one view (cleared to 0, then
    the prefix up to one past the last populated tile; later tiles stay 0)."""
    counts = counts.astype(np.int64)
    prefix = np.concatenate(([0], np.cumsum(counts)))
    out = np.zeros(len(counts) + 1, np.uint32)
    nz = np.nonzero(counts)[0]
    if len(nz):
        last = int(nz[-1])
        out[:last + 2] = prefix[:last + 2]
    return out


def batch_view_frame(r, v):
    """View v of the current batch in the single-view terms of oracle.rebin."""
    info = r.viewInfo(v)
    n, t = info.splat_count, info.tiles_x * info.tiles_y
    keys, vals, tcounts = r.readViewRefs(v)
    return dict(
        projected_splats=read_range(r, "projected_splats", 64 * info.splat_base, PROJ_DTYPE, n),
        splat_ref_counts=read_range(r, "splat_ref_counts", 4 * info.splat_base, np.uint32, n),
        splat_ref_offsets=None,
        ref_counter=len(vals),
        sort_keys_a=keys,
        sort_values_a=vals,
        tile_offsets=tile_offsets_from_counts(tcounts),
        image=r.readViewImage(v).astype(np.float32),
        tile_costs=read_range(r, "tile_costs", 4 * info.tile_base, np.uint32, t),
    )


@pytest.mark.parametrize("pose", [0, 37])
def test_c1_single_view_16x16_matches_oracle(renderer, oracle, c1, pose):
    u = c1_uniform(pose)
    o = oracle_frame(oracle, c1, u, W1, H1, 16, 16)
    g = gpu_frame(renderer, c1, u, W1, H1, 16, 16)
    assert o["ref_counter"] > 10_000_000
    assert_frame_match(g, o)


@pytest.mark.parametrize("tw,th,batch,order", [(32, 32, 256, "learned"),
                                                (64, 32, 512, "key_count")])
def test_c1_headline_batch_matches_oracle(renderer, oracle, c1, tw, th, batch, order):
    """The bench's first 8-view batch at an autotuned tuning (64x32 tiles with
    512-splat batches, the autotuner's pick on this workload, in key-count
    order; 32x32 with 256-splat batches in the learned order), CUDA-graph
    replay: views 0 and 5 against the oracle for that tile grid."""
    r = renderer
    r.setSplatData(c1)
    r.setTuning((tw, th), 8, batch)
    path = learned.checkpoint_for(tw, th)
    if order == "learned" and path is not None:
        r.setCostModel(path)
    else:
        r.setSchedule(_lib.SCHEDULE_KEY_COUNT)
    r.setCudaGraph(True)
    try:
        views = [(0, c1_uniform(i), W1, H1) for i in range(8)]
        r.rebinBatch(views)  # eager + capture
        r.rebinBatch(views)  # replay
        for v in (0, 5):
            o = oracle_frame(oracle, c1, views[v][1], W1, H1, tw, th)
            assert_frame_match(batch_view_frame(r, v), o)
    finally:
        r.setCudaGraph(False)
        r.setSchedule(_lib.SCHEDULE_ROW_MAJOR)
        r.setTuning(16, 8, 0)


def test_c2_4k_view_of_6m_scene_matches_oracle(renderer, oracle):
    r = renderer
    big = scenes.scene_clusters(6_000_000, seed=4, sh_degree=3)
    small = scenes.scene_clusters(500_000, seed=1, sh_degree=3)
    r.setSplatData(big)
    sid = r.addScene(small)
    eyes = scenes.random_eyes(32, 8.0, 16.0, seed=11)
    u_big = scenes.camera_at(eyes[3], W4, H4).getUniformData(W4, H4)
    u_small = scenes.camera_at(eyes[0], 1280, 720).getUniformData(1280, 720)
    r.setTuning(32, 8, 256)
    try:
        r.rebinBatch([(0, u_big, W4, H4), (sid, u_small, 1280, 720)])
        o = oracle_frame(oracle, big, u_big, W4, H4, 32, 32)
        assert o["ref_counter"] > 10_000_000
        assert_frame_match(batch_view_frame(r, 0), o)
        o = oracle_frame(oracle, small, u_small, 1280, 720, 32, 32)
        assert_frame_match(batch_view_frame(r, 1), o)
    finally:
        r.setTuning(16, 8, 0)


def test_c4_wide_view_matches_oracle(renderer, oracle):
    r = renderer
    data = scenes.scene_skewed(10_000_000, seed=0, sh_degree=3)
    r.setSplatData(data)
    wide = scenes.random_eyes(8, 28.0, 34.0, seed=22)
    u = scenes.camera_at(wide[7], W4, H4).getUniformData(W4, H4)
    r.setTuning(32, 8, 512)
    try:
        r.rebinBatch([(0, u, W4, H4)])
        o = oracle_frame(oracle, data, u, W4, H4, 32, 32)
        assert o["ref_counter"] > 100_000_000
        assert_frame_match(batch_view_frame(r, 0), o)
    finally:
        r.setTuning(16, 8, 0)
