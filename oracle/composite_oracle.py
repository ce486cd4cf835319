"""CPU restatement of the render passes after the rasterizer, which the tests
compare gs3d_composite with.  TEST INFRASTRUCTURE ONLY.

  * debug_tile_overlay.wgsl main_fs (src/shaders/render/debug_tile_overlay.wgsl
    :37-60): tile = min(px / tile_size, tile_count - 1); count = hi - lo
    guarded by hi >= lo; t = clamp(count / max(1, debug_ref), 0, 1);
    tint = (clamp(2t), clamp(2 - 2t), 0); out = tint * 0.4 + base * (1 - 0.4),
    alpha 0.4 + base.a * (1 - 0.4), stored to an rgba16float target;
  * composite_splats.wgsl with the premultiplied over blend
    (GaussianSplatRenderer.ts:938-945): out = src + dst * (1 - src.a);
  * unorm8 store: round-to-nearest-even(clamp01(x) * 255).
All in float32 without fused multiply-adds.
"""
from __future__ import annotations

import numpy as np

F = np.float32


def composite(image, tile_offsets, tile_w, tile_h, tiles_x, tiles_y, heatmap=False,
              debug_ref=256, background=(0.0, 0.0, 0.0, 1.0)) -> np.ndarray:
    """image: (H, W, 4) float16 premultiplied splat target of one view;
    tile_offsets: that view's T + 1 entries.  Returns (H, W, 4) uint8."""
    src = np.asarray(image, np.float16).astype(F)
    h, w, _ = src.shape
    if heatmap:
        py, px = np.mgrid[0:h, 0:w]
        tx = np.minimum(px // tile_w, tiles_x - 1)
        ty = np.minimum(py // tile_h, tiles_y - 1)
        t = (ty * tiles_x + tx).astype(np.int64)
        off = np.asarray(tile_offsets, np.uint32).astype(np.int64)
        lo, hi = off[t], off[t + 1]
        count = np.where(hi >= lo, hi - lo, 0).astype(F)
        tt = np.clip(count / F(max(1.0, float(debug_ref))), F(0), F(1)).astype(F)
        tint = np.stack([np.clip(tt * F(2), F(0), F(1)),
                         np.clip(F(2) - tt * F(2), F(0), F(1)),
                         np.zeros_like(tt)], -1).astype(F)
        ao = F(0.4)
        keep = F(1) - ao
        rgb = (tint * ao + src[..., :3] * keep).astype(F)
        a = (ao + src[..., 3] * keep).astype(F)
        src = np.concatenate([rgb, a[..., None]], -1).astype(np.float16).astype(F)
    bg = np.asarray(background, F)
    inv = (F(1) - src[..., 3:4]).astype(F)
    out = (src + bg * inv).astype(F)
    return np.rint(np.clip(out, F(0), F(1)) * F(255)).astype(np.uint8)
