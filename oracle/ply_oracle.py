"""CPU restatement of the reference's Gaussian-splat PLY loader
(src/workers/SceneWorker.ts:146-550), which the tests compare
gs3d_ply_inspect and gs3d_load_ply with.  TEST INFRASTRUCTURE ONLY.

Follows the reference step by step: the header is read from the first MB up
to end_header (parsePlyHeader, :149-253), the 14 required vertex properties
are checked (:255-272), every element's rows are read in order with the
typed readers (:274-336, :508-549) and each vertex row is activated in
float64 and stored as float32 (writeGaussianSplat, :378-464): positions,
colors = clamp01(0.5 + C0 f_dc) and clamp01(sigmoid(opacity)), scales =
exp, rotations / hypot.  f_rest values are kept raw in f_rest index order,
and the SH degree is inferred from their count (:501-506).

Where the reference is ill-defined on valid files the restatement follows
the PLY format, as the library does: the header ends at the one LF (or CRLF)
after end_header (the reference also skips any further CR/LF bytes, i.e. the
first bytes of a binary body that happen to be 0x0A or 0x0D).
"""
from __future__ import annotations

import math
import re

import numpy as np

_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2",
          "int16": "i2", "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4",
          "uint": "u4", "uint32": "u4", "float": "f4", "float32": "f4", "double": "f8",
          "float64": "f8"}
REQUIRED = ["x", "y", "z", "opacity", "scale_0", "scale_1", "scale_2",
            "rot_0", "rot_1", "rot_2", "rot_3", "f_dc_0", "f_dc_1", "f_dc_2"]
FORMATS = {"ascii": 0, "binary_little_endian": 1, "binary_big_endian": 2}


class PlyError(ValueError):
    pass


def parse_header(data: bytes) -> dict:
    """parsePlyHeader (SceneWorker.ts:149-253)."""
    prefix = data[:1 << 20]
    at = prefix.find(b"end_header")
    if at < 0:
        raise PlyError("Invalid PLY: missing end_header")
    hb = at + len(b"end_header")
    if hb < len(data) and data[hb:hb + 1] == b"\r":
        hb += 1
    if hb < len(data) and data[hb:hb + 1] == b"\n":
        hb += 1
    text = data[:at + len(b"end_header")].decode("utf-8", errors="replace")
    lines = [ln.strip() for ln in re.split(r"\r?\n", text)]
    lines = [ln for ln in lines if ln]
    if not lines or lines[0] != "ply":
        raise PlyError("Invalid PLY: file must start with `ply`")
    fmt = None
    elements = []
    cur = None
    for line in lines[1:]:
        if line == "end_header":
            break
        if line.startswith("comment ") or line.startswith("obj_info "):
            continue
        tok = line.split()
        if tok[0] == "format":
            fmt = tok[1] if len(tok) > 1 else ""
            continue
        if tok[0] == "element":
            name = tok[1] if len(tok) > 1 else ""
            try:
                count = float(tok[2]) if len(tok) > 2 else math.nan
            except ValueError:
                count = math.nan
            if not math.isfinite(count) or count < 0 or count != int(count):
                raise PlyError(f"Invalid PLY element count for '{name}'")
            cur = {"name": name, "count": int(count), "props": []}
            elements.append(cur)
            continue
        if tok[0] == "property":
            if cur is None:
                raise PlyError("Invalid PLY: property declared before element")
            if len(tok) > 1 and tok[1] == "list":
                raise PlyError("Unsupported PLY: list properties are not expected in "
                               "Gaussian Splat PLY files")
            cur["props"].append((tok[2] if len(tok) > 2 else "", tok[1] if len(tok) > 1 else ""))
    if not fmt:
        raise PlyError("Invalid PLY: missing format line")
    if fmt not in FORMATS:
        raise PlyError(f"Unsupported PLY format: {fmt}")
    vertex = next((e for e in elements if e["name"] == "vertex"), None)
    if vertex is None:
        raise PlyError("Invalid Gaussian Splat PLY: missing vertex element")
    names = {p for p, _ in vertex["props"]}
    for r in REQUIRED:  # validateGaussianSplatHeader (:255-272)
        if r not in names:
            raise PlyError(f"Invalid Gaussian Splat PLY: missing property '{r}'")
    return {"format": fmt, "elements": elements, "vertex": vertex, "header_bytes": hb}


def f_rest_names(vertex) -> list:
    """createGaussianPropertyLayout (:338-350): f_rest_<n>, by n, stable."""
    names = [p for p, _ in vertex["props"] if re.fullmatch(r"f_rest_\d+", p)]
    return sorted(names, key=lambda s: int(s[len("f_rest_"):]))


def infer_degree(count: int) -> int:
    return 3 if count >= 45 else 2 if count >= 24 else 1 if count >= 9 else 0


def read_vertex_rows(data: bytes, h: dict) -> dict:
    """All elements' rows in order; returns the vertex columns as float64."""
    fmt = h["format"]
    pos = h["header_bytes"]
    out = None
    if fmt == "ascii":
        tokens = data[pos:].decode("utf-8", errors="replace").split()
        ti = 0
        for e in h["elements"]:
            k = len(e["props"])
            need = e["count"] * k
            if ti + need > len(tokens):
                raise PlyError("Unexpected end of ASCII PLY body")
            chunk = tokens[ti:ti + need]
            ti += need
            vals = []
            for t in chunk:
                try:
                    v = float(t)
                except ValueError:
                    v = math.nan
                if not math.isfinite(v):
                    raise PlyError(f"Invalid ASCII PLY value '{t}'")
                vals.append(v)
            if e is h["vertex"]:
                arr = np.array(vals, np.float64).reshape(e["count"], k) if k else \
                    np.zeros((e["count"], 0))
                out = {p: arr[:, i] for i, (p, _) in enumerate(e["props"])}
        return out
    end = "<" if fmt == "binary_little_endian" else ">"
    for e in h["elements"]:
        for _, t in e["props"]:
            if t not in _TYPES:
                raise PlyError(f"Unsupported PLY scalar type: {t}")
        dt = np.dtype([(f"p{i}", end + _TYPES[t]) for i, (_, t) in enumerate(e["props"])])
        nbytes = dt.itemsize * e["count"]
        if pos + nbytes > len(data):
            raise PlyError("Invalid PLY: binary body shorter than its elements")
        rows = np.frombuffer(data, dt, count=e["count"], offset=pos) if e["count"] else \
            np.zeros(0, dt)
        pos += nbytes
        if e is h["vertex"]:
            out = {p: rows[f"p{i}"].astype(np.float64) for i, (p, _) in enumerate(e["props"])}
    return out


def load(data: bytes, oracle=None) -> dict:
    """parseGaussianSplatPly: header info, activated float32 splat arrays
    (the oracle library's orc_activate), raw f_rest and bounds."""
    h = parse_header(data)
    cols = read_vertex_rows(data, h)
    n = h["vertex"]["count"]
    for r in REQUIRED:  # required(): a finite number
        if n and not np.all(np.isfinite(cols[r])):
            raise PlyError(f"Invalid Gaussian Splat PLY row: missing '{r}'")
    xyz = np.stack([cols["x"], cols["y"], cols["z"]], 1)
    f_dc = np.stack([cols[f"f_dc_{c}"] for c in range(3)], 1)
    scale_log = np.stack([cols[f"scale_{c}"] for c in range(3)], 1)
    rot = np.stack([cols[f"rot_{c}"] for c in range(4)], 1)
    if oracle is None:
        from oracle import Oracle
        oracle = Oracle()
    pos, col, sc, ro = oracle.activate(xyz, f_dc, cols["opacity"], scale_log, rot)
    rest_names = f_rest_names(h["vertex"])
    rest = np.stack([cols[r] for r in rest_names], 1).astype(np.float32) if rest_names else None
    stride = 0
    if h["format"] != "ascii":
        stride = sum(np.dtype(_TYPES[t]).itemsize for _, t in h["vertex"]["props"])
    bounds = (xyz.min(0).astype(np.float32), xyz.max(0).astype(np.float32)) if n else None
    return {"info": {"splat_count": n, "header_bytes": h["header_bytes"],
                     "format": FORMATS[h["format"]], "f_rest_count": len(rest_names),
                     "sh_degree": infer_degree(len(rest_names)), "vertex_stride": stride},
            "positions": pos, "colors": col, "scales": sc, "rotations": ro, "f_rest": rest,
            "bounds": bounds}


def sh_block(f_rest, degree: int):
    """The SH coefficients the renderer uses: the first (d+1)^2 - 1 of each
    channel of the channel-major f_rest block (count divisible by 3)."""
    if f_rest is None or degree == 0 or f_rest.shape[1] % 3:
        return None
    per = f_rest.shape[1] // 3
    k = (degree + 1) ** 2 - 1
    return np.concatenate([f_rest[:, c * per:c * per + k] for c in range(3)], 1)
