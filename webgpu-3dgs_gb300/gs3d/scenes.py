"""Seeded synthetic scenes and camera poses of the benchmark workloads.

The reference's only sample scene is a missing large blob, and no public
dataset is mounted, so every workload is generated here with the shapes and
value distributions of the benchmark configurations.  Raw per-splat values are
drawn as float32 (what a 3DGS PLY stores), then activated exactly as the
reference's loader does (src/workers/SceneWorker.ts:407-464): in float64,
rounded to float32:

    rgb = clamp01(0.5 + C0 * f_dc), C0 = 0.28209479177387814
    a   = clamp01(sigmoid(opacity))
    s   = exp(scale_log)
    q   = rot / hypot(rot)  (w, x, y, z), unnormalised when the length is 0

f_rest coefficients are kept in PLY order (channel-major, 15 per channel at
degree 3), the order SceneWorker.ts:457-463 stores them in.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .camera import Camera

SH_C0 = 0.28209479177387814


@dataclass
class GaussianSplatData:
    """src/types/types.ts:14-22 (SoA of vec4 f32)."""
    positions: np.ndarray          # (N, 4) x, y, z, 1
    colors: np.ndarray             # (N, 4) r, g, b, a
    scales: np.ndarray             # (N, 4) sx, sy, sz, 0
    rotations: np.ndarray          # (N, 4) w, x, y, z
    sphericalHarmonics: np.ndarray | None  # (N, 3*((d+1)^2-1)) or None
    sphericalHarmonicsDegree: int
    splatCount: int


def activate(xyz, f_dc, opacity, scale_log, rot, f_rest=None, sh_degree=0) -> GaussianSplatData:
    n = len(opacity)
    xyz = np.asarray(xyz, np.float64)
    pos = np.empty((n, 4), np.float32)
    pos[:, :3] = xyz
    pos[:, 3] = 1.0
    col = np.empty((n, 4), np.float32)
    col[:, :3] = np.clip(0.5 + SH_C0 * np.asarray(f_dc, np.float64), 0.0, 1.0)
    col[:, 3] = np.clip(1.0 / (1.0 + np.exp(-np.asarray(opacity, np.float64))), 0.0, 1.0)
    sc = np.empty((n, 4), np.float32)
    sc[:, :3] = np.exp(np.asarray(scale_log, np.float64))
    sc[:, 3] = 0.0
    r = np.asarray(rot, np.float64)
    length = np.sqrt(np.sum(r * r, axis=1))
    inv = np.where(length > 0.0, 1.0 / np.where(length > 0.0, length, 1.0), 1.0)
    rots = (r * inv[:, None]).astype(np.float32)
    sh = None
    if sh_degree > 0 and f_rest is not None:
        sh = np.ascontiguousarray(f_rest, np.float32)
    return GaussianSplatData(pos, col, sc, rots, sh, sh_degree if sh is not None else 0, n)


def _normal(rng, size, mean=0.0, std=1.0):
    return (rng.standard_normal(size, dtype=np.float32) * np.float32(std)
            + np.float32(mean)).astype(np.float32)


def raw_small(n: int = 100_000, seed: int = 0) -> dict:
    """Raw (PLY) values of scene_small."""
    rng = np.random.default_rng(seed)
    xyz = _normal(rng, (n, 3), 0.0, 1.5)
    scale_log = _normal(rng, (n, 3), -4.5, 0.8)
    rot = _normal(rng, (n, 4))
    opacity = _normal(rng, n, 0.0, 1.5)
    f_dc = _normal(rng, (n, 3), 0.0, 0.5)
    return dict(xyz=xyz, f_dc=f_dc, opacity=opacity, scale_log=scale_log, rot=rot, f_rest=None,
                sh_degree=0)


def scene_small(n: int = 100_000, seed: int = 0) -> GaussianSplatData:
    """100k splats, SH degree 0: pos N(0, 1.5^2), scale exp(N(-4.5, 0.8^2)),
    rotation normalised N(0, 1)^4, opacity sigmoid(N(0, 1.5^2)), f_dc N(0, 0.5^2)."""
    return activate(**raw_small(n, seed))


def scene_clusters(n: int = 3_000_000, seed: int = 0, sh_degree: int = 3,
                   clusters: int = 64) -> GaussianSplatData:
    """Mixture of isotropic clusters (centres uniform in a radius-8 ball,
    sigma ~ U(0.2, 1.5)), scale exp(N(-4, 1)), rotation/opacity as the small
    scene, f_dc N(0, 0.5^2), f_rest N(0, 0.1^2)."""
    return activate(**raw_clusters(n, seed, sh_degree, clusters))


def raw_clusters(n: int = 3_000_000, seed: int = 0, sh_degree: int = 3,
                 clusters: int = 64) -> dict:
    """Raw (PLY) values of scene_clusters."""
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((clusters, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    centres = d * (8.0 * rng.random(clusters) ** (1.0 / 3.0))[:, None]
    sigma = rng.uniform(0.2, 1.5, clusters)
    which = rng.integers(0, clusters, n)
    xyz = (centres[which] + sigma[which, None] * rng.standard_normal((n, 3))).astype(np.float32)
    scale_log = _normal(rng, (n, 3), -4.0, 1.0)
    rot = _normal(rng, (n, 4))
    opacity = _normal(rng, n, 0.0, 1.5)
    f_dc = _normal(rng, (n, 3), 0.0, 0.5)
    k = 3 * ((sh_degree + 1) ** 2 - 1)
    f_rest = _normal(rng, (n, k), 0.0, 0.1) if k else None
    return dict(xyz=xyz, f_dc=f_dc, opacity=opacity, scale_log=scale_log, rot=rot, f_rest=f_rest,
                sh_degree=sh_degree)


def scene_skewed(n: int = 10_000_000, seed: int = 0, sh_degree: int = 3) -> GaussianSplatData:
    """16 very dense clusters (sigma ~ U(0.05, 0.3)) + 20% uniform background
    in a radius-20 ball, scale exp(N(-3.5, 1.5^2)), opacity sigmoid(N(1, 1.5^2))."""
    rng = np.random.default_rng(seed)
    n_bg = n // 5
    n_cl = n - n_bg
    d = rng.standard_normal((16, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    centres = d * (8.0 * rng.random(16) ** (1.0 / 3.0))[:, None]
    sigma = rng.uniform(0.05, 0.3, 16)
    which = rng.integers(0, 16, n_cl)
    cl = centres[which] + sigma[which, None] * rng.standard_normal((n_cl, 3))
    u = rng.standard_normal((n_bg, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    bg = u * (20.0 * rng.random(n_bg) ** (1.0 / 3.0))[:, None]
    xyz = np.concatenate([cl, bg]).astype(np.float32)
    scale_log = _normal(rng, (n, 3), -3.5, 1.5)
    rot = _normal(rng, (n, 4))
    opacity = _normal(rng, n, 1.0, 1.5)
    f_dc = _normal(rng, (n, 3), 0.0, 0.5)
    k = 3 * ((sh_degree + 1) ** 2 - 1)
    f_rest = _normal(rng, (n, k), 0.0, 0.1) if k else None
    return activate(xyz, f_dc, opacity, scale_log, rot, f_rest, sh_degree)


def scene_opacity_mix(n_opaque: int = 1_500_000, n_translucent: int = 400_000,
                      seed: int = 0) -> GaussianSplatData:
    """A frame of skewed tile costs, SH degree 0: 12 opaque clusters (centres
    in a radius-7 ball, sigma ~ U(0.3, 0.9), scale exp(N(-4.2, 0.6^2)),
    opacity sigmoid(N(4, 0.5^2)): many keys per tile, pixels terminate after
    a few dozen) beside 6 dense translucent ones (sigma ~ U(0.05, 0.15), scale
    exp(N(-3, 0.4^2)), opacity sigmoid(N(-5, 0.15^2)), alpha near the 1/255
    cut-off: no pixel terminates, every key of their tiles is iterated)."""
    rng = np.random.default_rng(seed + 3000)

    def clusters(n, k, smin, smax):
        d = rng.standard_normal((k, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        c = d * (7.0 * rng.random(k) ** (1.0 / 3.0))[:, None]
        sigma = rng.uniform(smin, smax, k)
        which = rng.integers(0, k, n)
        return c[which] + sigma[which, None] * rng.standard_normal((n, 3))

    n = n_opaque + n_translucent
    xyz = np.concatenate([clusters(n_opaque, 12, 0.3, 0.9),
                          clusters(n_translucent, 6, 0.05, 0.15)]).astype(np.float32)
    scale_log = np.concatenate([_normal(rng, (n_opaque, 3), -4.2, 0.6),
                                _normal(rng, (n_translucent, 3), -3.0, 0.4)])
    opacity = np.concatenate([_normal(rng, n_opaque, 4.0, 0.5),
                              _normal(rng, n_translucent, -5.0, 0.15)])
    rot = _normal(rng, (n, 4))
    f_dc = _normal(rng, (n, 3), 0.0, 0.5)
    return activate(xyz, f_dc, opacity, scale_log, rot, None, 0)


FOVY = math.radians(60.0)
NEAR = 0.2
FAR = 10000.0  # the reference's Viewport default far plane (src/Viewport.ts:58-66)


def camera_at(eye, width, height, target=(0.0, 0.0, 0.0), fovy=FOVY, near=NEAR,
              far=FAR) -> Camera:
    return Camera(eye, target, (0.0, 1.0, 0.0), fovy, width / height, near, far)


def small_camera(width=1280, height=720) -> Camera:
    """One pinhole camera at distance 6 looking at the origin."""
    return camera_at((0.0, 0.0, 6.0), width, height)


def orbit_eyes(count: int = 64, radius: float = 12.0, jitter_deg: float = 20.0,
               seed: int = 0) -> np.ndarray:
    """`count` poses evenly spaced in azimuth with uniform elevation jitter."""
    rng = np.random.default_rng(seed + 1000)
    az = 2.0 * math.pi * np.arange(count) / count
    el = np.radians(rng.uniform(-jitter_deg, jitter_deg, count))
    return np.stack([radius * np.cos(el) * np.sin(az), radius * np.sin(el),
                     radius * np.cos(el) * np.cos(az)], axis=1).astype(np.float32)


def random_eyes(count: int, rmin: float, rmax: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed + 2000)
    d = rng.standard_normal((count, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rng.uniform(rmin, rmax, count)
    return (d * r[:, None]).astype(np.float32)
