"""PLY ingest on the device (gs3d_load_ply) against the oracle's restatement
of the reference loader: the decoded, activated splat arrays, the bounds, the
errors, and the image rendered from a loaded scene."""
import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Gs3dError, Scene, ply, scenes
from oracle import ply_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


def ulps(a, b):
    """f32 ulp distance, elementwise."""
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7fffffff), ia)
    ib = np.where(ib < 0, -(ib & 0x7fffffff), ib)
    return np.abs(ia - ib)


def check_loaded(r, o):
    """Positions and SH bit-exact; transcendental activations (exp, sigmoid,
    hypot, computed in f64 on the device and in the host libm) within one f32
    ulp."""
    n = o["info"]["splat_count"]
    assert r.scene.splats.splatCount == n
    np.testing.assert_array_equal(r.readBuffer("splat_positions"), o["positions"])
    for name in ("scales", "rotations", "colors"):
        got = r.readBuffer("splat_" + name)
        assert ulps(got, o[name]).max(initial=0) <= 1, name
    deg = o["info"]["sh_degree"]
    want_sh = ply_oracle.sh_block(o["f_rest"], deg)
    if want_sh is not None:
        np.testing.assert_array_equal(r.readBuffer("splat_sh_rest"), want_sh)


@pytest.mark.parametrize("fmt", ["binary_little_endian", "binary_big_endian", "ascii"])
@pytest.mark.parametrize("variant", ["plain", "normals", "types", "elements", "f_rest48"])
def test_load_matches_oracle(renderer, oracle, fmt, variant):
    raw = scenes.raw_clusters(5000, seed=3, sh_degree=3)
    kw = {}
    if variant == "normals":
        kw = dict(normals=True, comments=["exported"])
    elif variant == "types":
        kw = dict(types={"x": "double", "opacity": "short", "f_dc_1": "int8", "rot_0": "uchar",
                         "scale_2": "double", "f_rest_7": "double"})
    elif variant == "elements":
        kw = dict(elements_before=[("camera", [("fx", "float", np.ones(2)),
                                               ("k", "uchar", np.arange(2))])],
                  elements_after=[("extra", [("v", "int", np.arange(7))])])
    elif variant == "f_rest48":
        kw = dict(f_rest_count=48)
    data = ply.write_ply(raw, fmt, **kw)
    o = ply_oracle.load(data, oracle)
    scene, info = renderer.loadPly(data)
    assert scene == 0
    assert {k: info[k] for k in o["info"]} == o["info"]
    assert list(info["bounds_min"]) == o["bounds"][0].tolist()
    assert list(info["bounds_max"]) == o["bounds"][1].tolist()
    check_loaded(renderer, o)


def test_loaded_scene_renders_like_set_splats(renderer, oracle, tmp_path):
    raw = scenes.raw_clusters(80_000, seed=6, sh_degree=3)
    path = tmp_path / "scene.ply"
    path.write_bytes(ply.write_ply(raw, "binary_little_endian", normals=True))
    o = ply_oracle.load(path.read_bytes(), oracle)
    cam = scenes.camera_at(scenes.orbit_eyes(2, radius=11.0)[1], 960, 540)
    u = cam.getUniformData(960, 540)
    renderer.loadPly(str(path))
    renderer.rebin(o["info"]["splat_count"], 60, 34, 960, 540, u)
    img_ply = renderer.readImage()
    data = scenes.GaussianSplatData(o["positions"], o["colors"], o["scales"], o["rotations"],
                                    ply_oracle.sh_block(o["f_rest"], 3), 3,
                                    o["info"]["splat_count"])
    renderer.setSplatData(data)
    renderer.rebin(data.splatCount, 60, 34, 960, 540, u)
    img_set = renderer.readImage()
    diff = np.abs(img_ply.astype(np.float32) - img_set.astype(np.float32))
    assert diff.max() <= 2.0 / 255.0


def test_new_scene_target_batches(renderer, oracle):
    a = scenes.scene_clusters(40_000, seed=1, sh_degree=1)
    renderer.setSplatData(a)
    data = ply.write_ply(scenes.raw_small(30_000, seed=2), "binary_big_endian")
    sid, info = renderer.loadPly(data, newScene=True)
    assert sid >= 1 and info["splat_count"] == 30_000
    eye = scenes.orbit_eyes(1, radius=6.0)[0]
    views = [(0, scenes.camera_at(eye, 640, 360).getUniformData(640, 360), 640, 360),
             (sid, scenes.small_camera(800, 450).getUniformData(800, 450), 800, 450)]
    renderer.rebinBatch(views)
    img = renderer.readViewImage(1).astype(np.float32)
    assert img[..., 3].max() > 0.5  # the loaded scene is visible in view 1


@pytest.mark.parametrize("case,message", [
    ("nan", "Invalid Gaussian Splat PLY row: missing 'opacity'"),
    ("short_ascii", "Unexpected end of ASCII PLY body"),
    ("bad_token", "Invalid ASCII PLY value 'abc'"),
    ("inf_token", "Invalid ASCII PLY value 'inf'"),
])
def test_body_errors_match_oracle(renderer, oracle, case, message):
    raw = scenes.raw_small(16, seed=4)
    if case == "nan":
        raw["opacity"] = raw["opacity"].copy()
        raw["opacity"][5] = np.nan
        data = ply.write_ply(raw, "binary_little_endian")
    else:
        data = ply.write_ply(raw, "ascii")
        lines = data.split(b"\n")
        last = len(lines) - 2
        toks = lines[last].split()
        if case == "short_ascii":
            toks = toks[:-2]
        else:
            toks[3] = b"abc" if case == "bad_token" else b"inf"
        lines[last] = b" ".join(toks)
        data = b"\n".join(lines)
    with pytest.raises(ply_oracle.PlyError) as want:
        ply_oracle.load(data, oracle)
    assert str(want.value) == message
    with pytest.raises(Gs3dError) as got:
        renderer.loadPly(data)
    assert got.value.message == message


def test_full_size_scene_round_trip(renderer):
    """The 3M-splat SH3 benchmark scene as a binary PLY: every decoded array
    equals the in-memory scene's (same float32 raw values, same activation)."""
    raw = scenes.raw_clusters(3_000_000, seed=0, sh_degree=3)
    d = scenes.activate(**raw)
    renderer.loadPly(ply.write_ply(raw, "binary_little_endian", normals=True))
    np.testing.assert_array_equal(renderer.readBuffer("splat_positions"), d.positions)
    for name, ref in (("scales", d.scales), ("rotations", d.rotations), ("colors", d.colors)):
        assert ulps(renderer.readBuffer("splat_" + name), ref).max() <= 1, name
    np.testing.assert_array_equal(renderer.readBuffer("splat_sh_rest"), d.sphericalHarmonics)
