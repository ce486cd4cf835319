"""Gaussian-splat PLY files: a writer for the 3DGS property layout and the
context-free header inspection of the library (gs3d_ply_inspect).  Loading
into a renderer is GaussianSplatRenderer.loadPly (device-side decode).

The writer produces what 3DGS trainers export: element vertex with x y z
[nx ny nz] f_dc_0..2 f_rest_0..K-1 opacity scale_0..2 rot_0..3 (rotation
w, x, y, z), values pre-activation (log scales, opacity logits)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

FORMATS = {"ascii": 0, "binary_little_endian": 1, "binary_big_endian": 2}
_NP = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
       "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
       "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


def vertex_columns(raw: dict, normals: bool = False, f_rest_count: int | None = None):
    """(name, values) columns of the 3DGS vertex layout from raw scene values
    (gs3d.scenes.raw_*)."""
    n = len(raw["opacity"])
    cols = [("x", raw["xyz"][:, 0]), ("y", raw["xyz"][:, 1]), ("z", raw["xyz"][:, 2])]
    if normals:
        cols += [(k, np.zeros(n, np.float32)) for k in ("nx", "ny", "nz")]
    cols += [(f"f_dc_{c}", raw["f_dc"][:, c]) for c in range(3)]
    rest = raw.get("f_rest")
    k = 0 if rest is None else rest.shape[1]
    if f_rest_count is not None:
        k = f_rest_count
    for i in range(k):
        cols.append((f"f_rest_{i}", rest[:, i] if rest is not None and i < rest.shape[1]
                     else np.zeros(n, np.float32)))
    cols.append(("opacity", raw["opacity"]))
    cols += [(f"scale_{c}", raw["scale_log"][:, c]) for c in range(3)]
    cols += [(f"rot_{c}", raw["rot"][:, c]) for c in range(4)]
    return cols


def _cast(vals, t: str) -> np.ndarray:
    """Values as PLY scalar type t (integers rounded and clipped to range)."""
    v = np.asarray(vals)
    dt = np.dtype(_NP[t])
    if dt.kind in "iu":
        info = np.iinfo(dt)
        v = np.clip(np.rint(np.nan_to_num(v.astype(np.float64))), info.min, info.max)
    return v.astype(dt)


def write_ply(raw: dict, fmt: str = "binary_little_endian", types: dict | None = None,
              comments=(), elements_before=(), elements_after=(), normals: bool = False,
              f_rest_count: int | None = None, order=None) -> bytes:
    """PLY bytes of a raw scene.  types maps property names to PLY scalar
    types (default float); elements_before / elements_after are
    (name, [(prop, type, values), ...]) elements around the vertex element;
    order permutes the vertex property columns."""
    types = types or {}
    cols = vertex_columns(raw, normals, f_rest_count)
    if order is not None:
        cols = [cols[i] for i in order]
    n = len(raw["opacity"])
    vertex = ("vertex", [(name, types.get(name, "float"), vals) for name, vals in cols])
    elements = list(elements_before) + [vertex] + list(elements_after)
    head = ["ply", f"format {fmt} 1.0"] + [f"comment {c}" for c in comments]
    for name, props in elements:
        count = n if name == "vertex" else len(props[0][2]) if props else 0
        head.append(f"element {name} {count}")
        head += [f"property {t} {p}" for p, t, _ in props]
    head.append("end_header")
    out = ("\n".join(head) + "\n").encode()
    for name, props in elements:
        count = n if name == "vertex" else len(props[0][2]) if props else 0
        if not props or count == 0:
            continue
        if fmt == "ascii":
            cols_txt = []
            for _, t, vals in props:
                v = np.asarray(vals)
                if _NP[t][0] == "f":  # shortest strings that round-trip the stored type
                    cols_txt.append([np.format_float_scientific(x, unique=True)
                                     if np.isfinite(x) else repr(float(x))
                                     for x in v.astype(_NP[t])])
                else:
                    cols_txt.append([str(int(x)) for x in _cast(v, t)])
            out += "".join(" ".join(row) + "\n" for row in zip(*cols_txt)).encode()
        else:
            end = "<" if fmt == "binary_little_endian" else ">"
            dt = np.dtype([(p, end + _NP[t]) for p, t, _ in props])
            arr = np.empty(count, dt)
            for p, t, vals in props:
                arr[p] = _cast(vals, t)
            out += arr.tobytes()
    return out


def inspect(data: bytes) -> dict:
    """Header of a Gaussian-splat PLY (gs3d_ply_inspect; no device needed)."""
    lib = _lib.load()
    info = _lib.PlyInfo_t()
    buf = np.frombuffer(data, np.uint8)
    rc = lib.gs3d_ply_inspect(buf.ctypes.data_as(C.c_void_p), buf.nbytes, C.byref(info))
    if rc != 0:
        raise _lib.Gs3dError(rc, lib.gs3d_last_error(None).decode())
    return info_dict(info)


def info_dict(info) -> dict:
    return {"splat_count": int(info.splat_count), "header_bytes": int(info.header_bytes),
            "format": int(info.format), "f_rest_count": int(info.f_rest_count),
            "sh_degree": int(info.sh_degree), "vertex_stride": int(info.vertex_stride),
            "bounds_min": tuple(info.bounds_min), "bounds_max": tuple(info.bounds_max)}
