"""Degenerate splats through the CUDA path: non-finite positions, zero and
huge scales, zero quaternions, splats at the eye, fully transparent and
fully opaque ones.  The rebin must finish without a device error, and the
fused path (depth digits sorted per splat, refs emitted in depth order)
must give the six reference stages' keys, values, tile ranges and image bit
for bit, also when non-finite depths produce sort keys equal to the culled
splats' all-ones key."""
import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Scene, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


def _degenerate_scene():
    base = scenes.scene_small(20_000, seed=3)
    pos, col = base.positions.copy(), base.colors.copy()
    scl, rot = base.scales.copy(), base.rotations.copy()
    pos[0:50, :3] = np.nan
    pos[50:100, 0] = np.inf
    pos[100:120, 1] = -np.inf
    scl[120:170, :3] = 0.0
    scl[170:220, :3] = 1e-30
    scl[220:230, :3] = 50.0
    rot[230:280] = 0.0
    col[280:320, 3] = 0.0
    col[320:360, 3] = 1.0
    pos[360:380, :3] = (0.0, 0.0, 6.0)  # the camera position of small_camera
    scl[380:400, 0] = np.nan
    return scenes.GaussianSplatData(pos, col, scl, rot, None, 0, base.splatCount)


def _frame(r, data, u, w, h, stagewise):
    r.setTileSize(16, 16)
    r.setSplatData(data)
    r.setStagewise(stagewise)
    r.rebin(data.splatCount, -(-w // 16), -(-h // 16), w, h, u)
    r.setStagewise(False)
    R = r.refCount()
    return dict(R=R, keys=r.readBuffer("sort_keys_a", R), vals=r.readBuffer("sort_values_a", R),
                toff=r.readBuffer("tile_offsets"), img=r.readImage())


@pytest.mark.parametrize("w,h", [(640, 360), (333, 217)])
def test_degenerate_splats_fused_equals_stagewise(renderer, w, h):
    data = _degenerate_scene()
    u = scenes.small_camera(w, h).getUniformData(w, h)
    f = _frame(renderer, data, u, w, h, stagewise=False)
    s = _frame(renderer, data, u, w, h, stagewise=True)
    assert f["R"] == s["R"] > 0
    assert np.array_equal(f["keys"], s["keys"])
    assert np.array_equal(f["vals"], s["vals"])
    assert np.array_equal(f["toff"], s["toff"])
    assert np.array_equal(f["img"].view(np.uint16), s["img"].view(np.uint16))
    # strict (tile, depth bits, splat id) order
    k = f["keys"].astype(np.uint64)
    order = (k[:, 0] << np.uint64(32)) | k[:, 1]
    assert np.all((order[1:] > order[:-1]) |
                  ((order[1:] == order[:-1]) & (f["vals"][1:] > f["vals"][:-1])))
    assert np.isfinite(f["img"].astype(np.float32)).all()


def _same_bits_or_both_nan(a, b):
    """Element-wise: equal f32 bit patterns, or both NaN (a NaN's payload
    bits are the platform's: canonical on the GPU, propagated from the input
    on the host)."""
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    fa, fb = a.view(np.float32), b.view(np.float32)
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(fa) & np.isnan(fb))


def _nan_keys_as_one(keys):
    """Sort keys with every NaN depth-key word (bits(-depth) of a NaN depth)
    replaced by 0xffffffff, the GPU's bits for it."""
    k = keys.copy()
    k[np.isnan(k[:, 1].view(np.float32)), 1] = 0xFFFFFFFF
    return k


@pytest.mark.parametrize("w,h", [(640, 360), (333, 217)])
def test_degenerate_splats_match_oracle(renderer, oracle, w, h):
    """The same degenerate scene against the oracle, whose semantics for
    non-finite values are defined (f32 -> u32 conversions saturate and send
    NaN to 0; min/max keep the non-NaN operand): records equal field by
    field up to NaN payloads, counts and tile ranges bit-exact, sorted keys
    and values bit-exact once every NaN depth key carries one bit pattern (the
    host's NaN payloads can differ between splats; the oracle's refs are
    re-sorted stably after that substitution), image within 2/255."""
    data = _degenerate_scene()
    u = scenes.small_camera(w, h).getUniformData(w, h)
    o = oracle.rebin(u, w, h, 16, 16, data.positions, data.scales, data.rotations, data.colors)
    f = _frame(renderer, data, u, w, h, stagewise=False)
    proj = renderer.readBuffer("projected_splats")
    counts = renderer.readBuffer("splat_ref_counts")
    gp = proj.view(np.uint32).reshape(len(proj), 16)
    op = o["projected_splats"].view(np.uint32).reshape(len(proj), 16)
    assert np.all(_same_bits_or_both_nan(gp, op))
    assert np.array_equal(counts, o["splat_ref_counts"])
    assert f["R"] == o["ref_counter"] > 0
    ok, ov = _nan_keys_as_one(o["sort_keys_a"]), o["sort_values_a"]
    order = np.lexsort((ov, ok[:, 1], ok[:, 0]))  # (tile, depth bits, splat id)
    assert np.array_equal(_nan_keys_as_one(f["keys"]), ok[order])
    assert np.array_equal(f["vals"], ov[order])
    assert np.array_equal(f["toff"], o["tile_offsets"])
    diff = np.abs(f["img"].astype(np.float32) - o["image"])
    assert diff.max() <= 2.0 / 255.0
