"""PLY ingest, host side (no GPU): the oracle's restatement of the reference
loader pinned by known answers, and gs3d_ply_inspect (the library's header
parser and layout) against it: same header facts, same errors."""
import numpy as np
import pytest

from gs3d import Gs3dError, ply, scenes
from oracle import ply_oracle

KAT = b"""ply
format ascii 1.0
comment known answers
element vertex 2
property float x
property float y
property float z
property float f_dc_0
property float f_dc_1
property float f_dc_2
property float opacity
property float scale_0
property float scale_1
property float scale_2
property float rot_0
property float rot_1
property float rot_2
property float rot_3
end_header
1 -2 3 0 0 0 0 0 0 0 2 0 0 0
0.5 0.25 -1 -10 10 0 100 -1 1 0.5 0 0 0 0
"""


def test_oracle_known_answers(oracle):
    o = ply_oracle.load(KAT, oracle)
    assert o["info"] == {"splat_count": 2, "header_bytes": KAT.index(b"end_header") + 11,
                         "format": 0, "f_rest_count": 0, "sh_degree": 0, "vertex_stride": 0}
    np.testing.assert_array_equal(o["positions"], [[1, -2, 3, 1], [0.5, 0.25, -1, 1]])
    # clamp01(0.5 + C0 * f_dc), clamp01(sigmoid(opacity))
    assert o["colors"][0].tolist() == [0.5, 0.5, 0.5, 0.5]
    c0 = 0.28209479177387814
    assert o["colors"][1].tolist() == [0.0, 1.0, 0.5, np.float32(1.0 / (1.0 + np.exp(-100.0)))]
    assert o["colors"][1, 0] == np.float32(max(0.0, 0.5 - 10 * c0))
    np.testing.assert_array_equal(o["scales"][0], [1, 1, 1, 0])
    assert o["scales"][1].tolist() == [np.float32(np.exp(-1.0)), np.float32(np.exp(1.0)),
                                       np.float32(np.exp(0.5)), 0.0]
    # rotation / hypot; a zero quaternion stays zero (invLength 1)
    assert o["rotations"][0].tolist() == [1, 0, 0, 0]
    assert o["rotations"][1].tolist() == [0, 0, 0, 0]
    assert o["bounds"][0].tolist() == [0.5, -2, -1] and o["bounds"][1].tolist() == [1, 0.25, 3]


@pytest.mark.parametrize("count,deg", [(0, 0), (8, 0), (9, 1), (23, 1), (24, 2), (44, 2),
                                       (45, 3), (48, 3)])
def test_sh_degree_inference(count, deg):
    assert ply_oracle.infer_degree(count) == deg
    raw = scenes.raw_clusters(4, seed=0, sh_degree=3)
    b = ply.write_ply(raw, "binary_little_endian", f_rest_count=count)
    info = ply.inspect(b)
    assert (info["f_rest_count"], info["sh_degree"]) == (count, deg)


def _variants():
    raw = scenes.raw_clusters(64, seed=5, sh_degree=2)
    before = [("camera", [("fx", "float", np.ones(3)), ("id", "uchar", np.arange(3))])]
    after = [("face", [("flag", "int", np.arange(5))])]
    mixed = {"x": "double", "y": "double", "z": "double", "opacity": "short", "f_dc_0": "uchar",
             "f_dc_1": "int8", "f_dc_2": "ushort", "rot_3": "int", "scale_0": "uint"}
    for fmt in ("ascii", "binary_little_endian", "binary_big_endian"):
        yield fmt, ply.write_ply(raw, fmt)
        yield fmt + "+normals+comments", ply.write_ply(raw, fmt, normals=True,
                                                      comments=["a", "b c"])
        yield fmt + "+elements", ply.write_ply(raw, fmt, elements_before=before,
                                               elements_after=after)
        yield fmt + "+types", ply.write_ply(raw, fmt, types=mixed)
        ncol = len(ply.vertex_columns(raw))
        yield fmt + "+order", ply.write_ply(raw, fmt, order=list(range(ncol))[::-1])
    yield "crlf", ply.write_ply(raw, "ascii").replace(b"\n", b"\r\n")
    yield "obj_info", ply.write_ply(raw, "binary_little_endian").replace(
        b"format binary_little_endian 1.0\n", b"format binary_little_endian 1.0\nobj_info x y\n")


@pytest.mark.parametrize("name,data", list(_variants()), ids=[n for n, _ in _variants()])
def test_inspect_matches_oracle(name, data, oracle):
    o = ply_oracle.load(data, oracle)
    info = ply.inspect(data)
    assert {k: info[k] for k in o["info"]} == o["info"]


def _errors():
    raw = scenes.raw_small(8, seed=0)
    good = ply.write_ply(raw, "binary_little_endian")
    head = good[:good.index(b"end_header")]
    yield "no end_header", head
    yield "no magic", good.replace(b"ply\n", b"plx\n", 1)
    yield "no format", good.replace(b"format binary_little_endian 1.0\n", b"")
    yield "bad format", good.replace(b"binary_little_endian", b"binary_middle_endian")
    yield "no vertex", good.replace(b"element vertex", b"element points")
    yield "missing rot_3", good.replace(b"property float rot_3", b"property float rot_9")
    yield "list", good.replace(b"property float x\n",
                               b"property list uchar int idx\nproperty float x\n")
    yield "count", good.replace(b"element vertex 8", b"element vertex -8")
    yield "fractional count", good.replace(b"element vertex 8", b"element vertex 7.5")
    yield "property first", good.replace(b"element vertex 8\n", b"").replace(
        b"end_header", b"element vertex 8\nend_header")
    yield "scalar type", good.replace(b"property float opacity", b"property half opacity")
    yield "truncated", good[:-7]


@pytest.mark.parametrize("name,data", list(_errors()), ids=[n for n, _ in _errors()])
def test_inspect_errors_match_oracle(name, data, oracle):
    with pytest.raises(ply_oracle.PlyError) as want:
        ply_oracle.load(data, oracle)
    with pytest.raises(Gs3dError) as got:
        ply.inspect(data)
    assert got.value.code == 1
    assert got.value.message == str(want.value)


def test_writer_round_trips_raw_values(oracle):
    raw = scenes.raw_clusters(32, seed=9, sh_degree=3)
    for fmt in ("binary_little_endian", "binary_big_endian", "ascii"):
        o = ply_oracle.load(ply.write_ply(raw, fmt), oracle)
        np.testing.assert_array_equal(o["positions"][:, :3], raw["xyz"])
        np.testing.assert_array_equal(o["f_rest"], raw["f_rest"])
