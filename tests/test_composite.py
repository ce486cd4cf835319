"""Headless composite (host side): the composite oracle pinned by known
answers, and the PNG writer."""
import numpy as np

from gs3d.image import png_bytes, read_png
from oracle import composite_oracle


def test_over_blend_known_answers():
    img = np.zeros((1, 3, 4), np.float16)
    img[0, 0] = (0.5, 0.0, 0.0, 0.5)   # half-covered red over blue
    img[0, 1] = (0.0, 0.0, 0.0, 0.0)   # empty: the background shows
    img[0, 2] = (0.2, 0.4, 0.6, 1.0)   # opaque
    out = composite_oracle.composite(img, [0, 0], 16, 16, 1, 1, background=(0, 0, 1, 1))
    assert out[0, 0].tolist() == [128, 0, 128, 255]
    assert out[0, 1].tolist() == [0, 0, 255, 255]
    assert out[0, 2].tolist() == [51, 102, 153, 255]


def test_heatmap_known_answers():
    img = np.zeros((2, 4, 4), np.float16)  # 2x2-pixel tiles, 2 tiles
    off = np.array([0, 0, 256], np.uint32)  # tile 0: 0 keys, tile 1: 256 keys
    out = composite_oracle.composite(img, off, 2, 2, 2, 1, heatmap=True, debug_ref=256,
                                     background=(0, 0, 0, 0))
    # tint green (few) / red (many) at 40% through an rgba16float target
    g = np.float16(np.float32(0.4)).astype(np.float32)
    v = int(np.rint(g * np.float32(255)))
    assert out[0, 0].tolist() == [0, v, 0, v]
    assert out[0, 3].tolist() == [v, 0, 0, v]
    # trailing zeros of tile_offsets (hi < lo) count as empty
    out2 = composite_oracle.composite(img, np.array([0, 5, 0], np.uint32), 2, 2, 2, 1,
                                      heatmap=True, debug_ref=10, background=(0, 0, 0, 0))
    assert out2[0, 3].tolist() == [0, v, 0, v]


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (17, 31, 4), dtype=np.uint8)
    data = png_bytes(img)
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    np.testing.assert_array_equal(read_png(data), img)
