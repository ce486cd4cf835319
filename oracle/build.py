"""Build recipe for the CPU oracle (test infrastructure, never shipped).

Compiles gs_oracle.cpp with g++ -O3 -fopenmp -ffp-contract=off (no
fast-math, no -march) into oracle/_build/liboracle.so.  The reference itself
(TypeScript + WGSL) has no CPU code on this path that a C compiler could build,
so there is no oracle/_ref recipe.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"
FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
         "-fPIC", "-shared"]


def build(force: bool = False) -> Path:
    src = HERE / "gs_oracle.cpp"
    hdr = HERE / "gs_oracle.h"
    OUT.parent.mkdir(exist_ok=True)
    if (not force and OUT.exists()
            and OUT.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime)):
        return OUT
    cxx = shutil.which("g++") or "g++"
    tmp = OUT.with_suffix(".so.tmp")
    res = subprocess.run([cxx, *FLAGS, str(src), "-o", str(tmp)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
