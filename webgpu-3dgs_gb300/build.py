"""Builds libgs3d.so, the sm_103a CUDA library, in-tree (gs3d/libgs3d.so).

Every translation unit is compiled by nvcc for sm_103a only, in parallel, and
linked into one shared library with a static CUDA runtime.  preprocess.cu is
compiled with -fmad=false so its f32 arithmetic is one IEEE-rounded
operation per written operator, the property its bit-exact parity with the
CPU oracle relies on; the other stages use the default contraction.  Where
the raster must not contract (its reference-order form of d^T conic d) it
uses the scalar __fmul_rn / __fadd_rn intrinsics, which are never fused: a
paired FP32 multiply feeding a paired add is fused into a paired FMA on
sm_103a, with or without -fmad=false.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "gs3d"
BUILD_DIR = HERE / "_build"
LIB = OUT_DIR / "libgs3d.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-Xptxas", "-warn-spills"]
PER_FILE = {"preprocess.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD_DIR / (src.stem + ".o")
    # the flags live here, so a change of this file recompiles everything
    deps = [src] + sorted(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "gs3d.h",
                                                  Path(__file__).resolve()]
    if obj.exists() and obj.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *PER_FILE.get(src.name, []), "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    if force:
        for o in BUILD_DIR.glob("*.o"):
            o.unlink()
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs) and not force:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
