"""Known-answer tests pinning the CPU oracle to the reference's WGSL text.

The reference ships no tests or golden data, and its WGSL cannot run here, so
each expectation below is derived by hand from the cited shader lines.
"""
import math
import struct

import numpy as np
import pytest

from oracle import PROJ_DTYPE


def f32bits(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def simple_camera(oracle, w=64, h=64, eye=(0.0, 0.0, 5.0), fovy=math.pi / 2, near=0.1, far=100.0):
    return oracle.camera_uniform(eye, (0, 0, 0), (0, 1, 0), fovy, w / h, near, far, w, h)


def one_splat(pos, scale, rot=(1, 0, 0, 0), rgba=(0.2, 0.4, 0.6, 0.8)):
    p = np.array([[*pos, 1.0]], np.float32)
    s = np.array([[*scale, 0.0]], np.float32)
    r = np.array([rot], np.float32)
    c = np.array([rgba], np.float32)
    return p, s, r, c


def test_camera_lookat_perspective_no(oracle):
    # gl-matrix lookAt from (0,0,5) to the origin is a pure translation
    u = simple_camera(oracle)
    view = u[0:16].reshape(4, 4)  # rows = columns of the matrix
    assert np.allclose(view[:3, :3], np.eye(3))
    assert view[3, 2] == -5.0
    proj = u[16:32]
    assert proj[0] == 1.0 and proj[5] == 1.0 and proj[11] == -1.0
    assert proj[10] == np.float32(100.1 / -99.9)         # (far+near)/(near-far)
    assert proj[14] == np.float32(2 * 100 * 0.1 / -99.9)  # 2 far near / (near-far)
    assert list(u[64:72]) == [0, 0, 5, 1, 64, 64, 1, 0]


def test_preprocess_axis_aligned_centre_splat(oracle):
    """preprocess_splats.wgsl:89-171 for a splat at the image centre, R = I."""
    cam = simple_camera(oracle)
    p, s, r, c = one_splat((0, 0, 0), (0.5, 0.25, 0.1))
    proj, counts = oracle.preprocess(cam, (4, 4), (1 / 16, 1 / 16), p, s, r, c)
    rec = proj[0]
    assert rec["valid"] == 1
    assert tuple(rec["mean_px"]) == (32.0, 32.0)       # (ndc*.5+.5)*W, (1-(ndc*.5+.5))*H
    assert rec["depth"] == -5.0
    # fx = fy = 32, J = diag(6.4, -6.4): a = 6.4^2 sx^2 + .3, c = 6.4^2 sy^2 + .3, b = 0
    a = 6.4 ** 2 * 0.25 + 0.3
    cc = 6.4 ** 2 * 0.0625 + 0.3
    det = a * cc
    np.testing.assert_allclose(rec["conic"], [cc / det, 0.0, a / det], rtol=1e-6, atol=1e-9)
    assert rec["radius_px"] == math.ceil(3 * math.sqrt(a))  # lambda = a when b = 0
    assert rec["radius_px"] == 10.0
    # px rect [22, 42] -> tiles [1, 2] x [1, 2]
    assert tuple(rec["tile_min"]) == (1, 1) and tuple(rec["tile_max"]) == (2, 2)
    assert counts[0] == 4
    assert tuple(rec["color"]) == pytest.approx((0.2, 0.4, 0.6))
    assert rec["opacity"] == np.float32(0.8)


@pytest.mark.parametrize("pos,why", [
    ((0.0, 0.0, 10.0), "behind the camera: clip.w <= 0 (:92)"),
    ((10.0, 0.0, 0.0), "centre outside ndc x (:95)"),
    ((0.0, -9.0, 0.0), "centre outside ndc y (:96)"),
    ((0.0, 0.0, 4.85), "view z = -0.15: ndc z < 0 with the [-1,1] projection (:97)"),
])
def test_preprocess_culls(oracle, pos, why):
    cam = simple_camera(oracle)
    proj, counts = oracle.preprocess(cam, (4, 4), (1 / 16, 1 / 16), *one_splat(pos, (0.1,) * 3))
    assert proj[0]["valid"] == 0, why
    assert counts[0] == 0


def test_preprocess_near_range_kept_beyond_ndc_zero(oracle):
    cam = simple_camera(oracle)
    proj, counts = oracle.preprocess(cam, (4, 4), (1 / 16, 1 / 16),
                                     *one_splat((0.0, 0.0, 4.75), (0.01,) * 3))
    assert proj[0]["valid"] == 1 and counts[0] >= 1   # view z = -0.25 -> ndc z > 0


def test_preprocess_clamps_rect_to_viewport(oracle):
    """A huge splat covers every tile; rect clamped to tile_count - 1 (:157-164)."""
    cam = simple_camera(oracle, w=70, h=40)
    proj, counts = oracle.preprocess(cam, (5, 3), (1 / 16, 1 / 16), *one_splat((0, 0, 0), (3.0,) * 3))
    rec = proj[0]
    assert tuple(rec["tile_min"]) == (0, 0) and tuple(rec["tile_max"]) == (4, 2)
    assert counts[0] == 15


def test_prefix_scan_sentinel(oracle):
    off, total = oracle.prefix_scan(np.array([3, 0, 2, 5], np.uint32))
    assert list(off) == [0, 3, 3, 5, 10] and total == 10   # prefix_scan_blocks.wgsl:41-42
    off, total = oracle.prefix_scan(np.zeros(0, np.uint32))
    assert list(off) == [0] and total == 0


def test_emit_row_major_and_depth_bits(oracle):
    proj = np.zeros(3, PROJ_DTYPE)
    proj[0]["valid"], proj[0]["depth"] = 1, -2.0
    proj[0]["tile_min"], proj[0]["tile_max"] = (1, 0), (2, 1)
    proj[2]["valid"], proj[2]["depth"] = 1, -1.0
    proj[2]["tile_min"], proj[2]["tile_max"] = (0, 3), (0, 3)
    offsets = np.array([0, 4, 4, 5], np.uint32)
    keys, vals = oracle.emit(4, proj, offsets, 5)
    assert [tuple(k) for k in keys] == [(1, f32bits(2.0)), (2, f32bits(2.0)), (5, f32bits(2.0)),
                                        (6, f32bits(2.0)), (12, f32bits(1.0))]
    assert list(vals) == [0, 0, 0, 0, 2]


def test_radix_sort_stable_lexicographic(oracle):
    a, b = f32bits(1.0), f32bits(2.0)
    keys = np.array([(5, a), (1, b), (5, a), (1, a)], np.uint32)
    vals = np.array([0, 1, 2, 3], np.uint32)
    sk, sv = oracle.radix_sort(keys, vals)
    assert [tuple(k) for k in sk] == [(1, a), (1, b), (5, a), (5, a)]
    assert list(sv) == [3, 1, 0, 2]          # equal keys keep emit order


def test_radix_sort_matches_numpy_lexsort(oracle):
    rng = np.random.default_rng(3)
    r = 50_000
    keys = np.stack([rng.integers(0, 300, r), rng.integers(0, 1 << 31, r)], 1).astype(np.uint32)
    keys[::7, 1] = keys[::7, 1] & 0xFF   # many ties
    vals = np.arange(r, dtype=np.uint32)
    sk, sv = oracle.radix_sort(keys, vals, threads=4)
    order = np.lexsort((vals, keys[:, 1], keys[:, 0]))
    assert np.array_equal(sv, vals[order]) and np.array_equal(sk, keys[order])


def test_identify_gaps_and_trailing_zeros(oracle):
    keys = np.array([[1, 0], [1, 0], [3, 0], [3, 0], [3, 0], [4, 0]], np.uint32)
    off = oracle.identify(keys, 7)
    # identify_tile_ranges.wgsl:38-51; tiles after the last populated one stay 0
    assert list(off) == [0, 0, 2, 2, 5, 6, 0, 0]
    counts = [max(0, int(off[t + 1]) - int(off[t])) for t in range(7)]
    assert counts == [0, 2, 0, 3, 1, 0, 0]


def test_identify_empty(oracle):
    assert list(oracle.identify(np.zeros((0, 2), np.uint32), 3)) == [0, 0, 0, 0]


def _raster_one(oracle, splats, w=16, h=16):
    proj = np.zeros(len(splats), PROJ_DTYPE)
    for i, (mx, my, r, conic, op, col) in enumerate(splats):
        proj[i]["mean_px"] = (mx, my)
        proj[i]["radius_px"] = r
        proj[i]["conic"] = conic
        proj[i]["opacity"] = op
        proj[i]["color"] = col
        proj[i]["valid"] = 1
    toff = np.array([0, len(splats)], np.uint32)
    vals = np.arange(len(splats), dtype=np.uint32)
    return oracle.rasterize(w, h, 16, 16, proj, toff, vals)


def test_raster_single_splat_centre_and_cutoff(oracle):
    img, costs = _raster_one(oracle, [(8.5, 8.5, 100.0, (1.0, 0.0, 1.0), 0.9, (1.0, 0.5, 0.25))])
    # centre pixel (8, 8): power = 0, alpha = 0.9 (rasterize_tiles.wgsl:89-96)
    np.testing.assert_allclose(img[8, 8], [0.9, 0.45, 0.225, 0.9], rtol=1e-6)
    # pixel (0, 0): d^2 = 72, alpha = .9 exp(-36) < 1/255 -> skipped
    assert np.all(img[0, 0] == 0.0)
    assert costs[0] == 1


def test_raster_radius_cull(oracle):
    img, _ = _raster_one(oracle, [(8.5, 8.5, 0.5, (1e-6, 0.0, 1e-6), 0.9, (1, 1, 1))])
    assert img[8, 8, 3] > 0.89 and np.all(img[8, 9] == 0.0)   # |d|^2 = 1 > r^2 (:85)


def test_raster_early_termination_and_cost(oracle):
    # two near-opaque splats drive T below 1e-4 at the centre: the third is never blended
    spl = [(8.5, 8.5, 100.0, (1.0, 0.0, 1.0), 0.99, (1.0, 0.0, 0.0))] * 2 + \
          [(8.5, 8.5, 100.0, (1.0, 0.0, 1.0), 0.99, (0.0, 0.0, 1.0))]
    img, costs = _raster_one(oracle, spl)
    t = np.float32(1) - np.float32(0.99)
    assert np.float32(t * t) < np.float32(1e-4)
    assert img[8, 8, 2] == 0.0           # blue splat after termination never blends
    assert costs[0] == 3                 # but other pixels of the tile iterate all three


def _pairs_one(oracle, splats):
    proj = np.zeros(len(splats), PROJ_DTYPE)
    for i, (mx, my, r, conic, op, col) in enumerate(splats):
        proj[i]["mean_px"] = (mx, my)
        proj[i]["radius_px"] = r
        proj[i]["conic"] = conic
        proj[i]["opacity"] = op
        proj[i]["color"] = col
        proj[i]["valid"] = 1
    toff = np.array([0, len(splats)], np.uint32)
    return oracle.raster_pairs(16, 16, 16, 16, proj, toff, np.arange(len(splats), dtype=np.uint32))


def test_raster_pair_counts(oracle):
    # one splat of radius 0.5: every pixel iterates it, only the centre pixel
    # is inside the radius (|d|^2 = 0; all others >= 1 > 0.25) and blends it
    assert _pairs_one(oracle, [(8.5, 8.5, 0.5, (1e-6, 0.0, 1e-6), 0.9, (1, 1, 1))]) == \
        {"iterated": 256, "evaluated": 1, "blended": 1}
    # three near-opaque unit-conic splats at the centre: every pixel is inside
    # the radius with power <= 0; alpha >= 1/255 where |d|^2 <= 10 (37 pixels);
    # the centre pixel terminates at the second splat, the others walk all 3
    spl = [(8.5, 8.5, 100.0, (1.0, 0.0, 1.0), 0.99, (1.0, 0.0, 0.0))] * 3
    assert _pairs_one(oracle, spl) == \
        {"iterated": 255 * 3 + 2, "evaluated": 255 * 3 + 2, "blended": 36 * 3 + 2}


def test_activations_match_loader(oracle):
    from gs3d.scenes import activate
    rng = np.random.default_rng(0)
    n = 1000
    xyz, fdc = rng.normal(0, 2, (n, 3)), rng.normal(0, 3, (n, 3))
    op, sl, rot = rng.normal(0, 3, n), rng.normal(-4, 1, (n, 3)), rng.normal(0, 1, (n, 4))
    rot[0] = 0.0                                     # zero-length quaternion: left as is
    p1 = activate(xyz, fdc, op, sl, rot)
    p2 = oracle.activate(xyz, fdc, op, sl, rot)
    for a, b in zip((p1.positions, p1.colors, p1.scales, p1.rotations), p2):
        np.testing.assert_array_max_ulp(a, b, maxulp=1)
    assert p1.colors.max() <= 1.0 and p1.colors.min() >= 0.0


def test_camera_module_matches_oracle(oracle):
    from gs3d.scenes import camera_at, orbit_eyes
    for eye in orbit_eyes(8):
        cam = camera_at(eye, 1920, 1080)
        u1 = cam.getUniformData(1920, 1080)
        u2 = oracle.camera_uniform(cam.position, cam.target, cam.up, cam.fov, cam.aspect,
                                   cam.near, cam.far, 1920, 1080)
        # both compute in float64 and round once; near-zero entries may differ
        # by the last bits of a double cancellation
        np.testing.assert_allclose(u1[:32], u2[:32], rtol=2e-7, atol=1e-6)
        np.testing.assert_array_equal(u1[64:], u2[64:])


def test_mlp_oracle_gradient_matches_finite_differences():
    """The float64 cost-MLP oracle that checks the GPU training kernels."""
    from oracle import mlp_oracle
    from gs3d import learned
    rng = np.random.default_rng(2)
    p = learned.init_params(4, 0.3).astype(np.float64)
    x, t = rng.normal(0, 1, (40, 16)), rng.normal(1, 1, 40)
    g = mlp_oracle.grad(p, x, t)
    loss = lambda q: np.mean((mlp_oracle.forward(q, x)[0] - t) ** 2)  # noqa: E731
    for i in rng.choice(len(p), 60, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (loss(p + e) - loss(p - e)) / 2e-6
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(g[i]))


def test_learned_gate():
    from gs3d import learned
    good = {"mlp_mae_log": 0.2, "keycount_mae_log": 0.4, "mlp_spearman": 0.9,
            "keycount_spearman": 0.8}
    assert learned.gate(good)
    assert not learned.gate({**good, "mlp_mae_log": 0.9})       # error above the bound
    assert not learned.gate({**good, "mlp_spearman": 0.7})      # ranks worse than key count
    assert abs(learned.spearman(np.arange(10.0), np.arange(10.0) ** 2) - 1.0) < 1e-12
