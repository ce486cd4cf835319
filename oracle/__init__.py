"""CPU oracle of the webgpu-3dgs rebin path - TEST INFRASTRUCTURE ONLY.

Imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU baseline
legs, always as the reference the results are compared with or as the timed
CPU baseline, never by the library.
Parity status: unpinned against executable reference output (see
gs_oracle.cpp); pinned to the WGSL text by hand-derived known-answer tests.
"""
from .oracle import Oracle, PROJ_DTYPE  # noqa: F401
