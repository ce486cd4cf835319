"""Minimal PNG writer for headless frames (8-bit RGBA, no dependencies
beyond zlib)."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def png_bytes(rgba: np.ndarray) -> bytes:
    """(H, W, 4) uint8 -> PNG file bytes (colour type 6, no interlace)."""
    img = np.ascontiguousarray(rgba, np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("expected an (H, W, 4) uint8 array")
    h, w, _ = img.shape
    raw = np.zeros((h, 1 + 4 * w), np.uint8)  # filter byte 0 per row
    raw[:, 1:] = img.reshape(h, 4 * w)

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + \
            struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)) + chunk(b"IEND", b""))


def write_png(path, rgba: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(png_bytes(rgba))


def read_png(path_or_bytes) -> np.ndarray:
    """Reads back what png_bytes writes (8-bit RGBA, filter 0 rows)."""
    data = path_or_bytes if isinstance(path_or_bytes, bytes) else open(path_or_bytes, "rb").read()
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    return raw[:, 1:].reshape(h, w, 4).copy()
