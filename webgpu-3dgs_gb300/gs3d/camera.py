"""Camera - the uniform-producing part of src/Camera.ts.

Restates Camera.updateView / setProjection / getUniformData
(src/Camera.ts:69-79,172-191), which call gl-matrix 3.4 (not vendored in the
reference; package-lock.json pins 3.4.4): mat4.lookAt, mat4.perspective (the
OpenGL "NO" convention, clip z in [-1, 1]) and mat4.invert.  gl-matrix
computes in float64 and stores into Float32Array outputs; this module does the
same with numpy.  Mouse-driven orbit/pan/zoom (Camera.ts:93-170) belongs to
the interactive UI and is not part of the rebin path.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from ._lib import Camera_t


def look_at(eye, target, up) -> np.ndarray:
    """mat4.lookAt: column-major 16 floats (computed in float64)."""
    e = np.asarray(eye, np.float64)
    t = np.asarray(target, np.float64)
    u = np.asarray(up, np.float64)
    if np.all(np.abs(e - t) < 1e-6):
        return np.eye(4, dtype=np.float64).reshape(-1)
    z = e - t
    z = z / math.sqrt(float(z @ z))
    x = np.array([u[1] * z[2] - u[2] * z[1], u[2] * z[0] - u[0] * z[2], u[0] * z[1] - u[1] * z[0]])
    n = math.sqrt(float(x @ x))
    x = x / n if n else np.zeros(3)
    y = np.array([z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]])
    n = math.sqrt(float(y @ y))
    y = y / n if n else np.zeros(3)
    return np.array([x[0], y[0], z[0], 0.0, x[1], y[1], z[1], 0.0, x[2], y[2], z[2], 0.0,
                     -(x @ e), -(y @ e), -(z @ e), 1.0])


def perspective(fovy, aspect, near, far) -> np.ndarray:
    """mat4.perspective (NO): column-major 16 floats (computed in float64)."""
    f = 1.0 / math.tan(fovy / 2.0)
    m = np.zeros(16)
    m[0] = f / aspect
    m[5] = f
    m[11] = -1.0
    if far is not None and math.isfinite(far):
        nf = 1.0 / (near - far)
        m[10] = (far + near) * nf
        m[14] = 2.0 * far * near * nf
    else:
        m[10] = -1.0
        m[14] = -2.0 * near
    return m


def _invert(m32: np.ndarray) -> np.ndarray:
    a = m32.astype(np.float64).reshape(4, 4).T  # row-major view of a column-major matrix
    try:
        inv = np.linalg.inv(a)
    except np.linalg.LinAlgError:
        return np.zeros(16, np.float32)
    return inv.T.reshape(-1).astype(np.float32)


class Camera:
    """Holds eye/target/up and projection parameters; produces the 72-float
    CameraUniforms block the preprocess stage reads."""

    def __init__(self, position, target, up, fov, aspect, near, far):
        self.position = np.asarray(position, np.float32).copy()  # gl-matrix vec3 = Float32Array
        self.target = np.asarray(target, np.float32).copy()
        self.up = np.asarray(up, np.float32).copy()
        self.fov = float(fov)
        self.aspect = float(aspect)
        self.near = float(near)
        self.far = float(far)
        self.version = 0
        self.updateView()
        self.setProjection()

    def updateView(self):
        self.viewMatrix = look_at(self.position, self.target, self.up).astype(np.float32)
        self.inverseViewMatrix = _invert(self.viewMatrix)
        self.version += 1

    def setProjection(self):
        self.projectionMatrix = perspective(self.fov, self.aspect, self.near,
                                            self.far).astype(np.float32)
        self.inverseProjectionMatrix = _invert(self.projectionMatrix)
        self.version += 1

    def setPosition(self, position):
        self.position = np.asarray(position, np.float32).copy()
        self.updateView()

    def setTarget(self, target):
        self.target = np.asarray(target, np.float32).copy()
        self.updateView()

    def getUniformData(self, width: float, height: float) -> np.ndarray:
        d = np.zeros(72, np.float32)
        d[0:16] = self.viewMatrix
        d[16:32] = self.projectionMatrix
        d[32:48] = self.inverseViewMatrix
        d[48:64] = self.inverseProjectionMatrix
        d[64:67] = self.position
        d[67] = 1.0
        d[68] = width
        d[69] = height
        d[70] = width / height
        d[71] = 0.0
        return d


def camera_struct(uniform72: np.ndarray) -> Camera_t:
    """Packs a 72-float uniform block into the C ABI's gs3d_camera."""
    u = np.ascontiguousarray(uniform72, np.float32)
    if u.shape != (72,):
        raise ValueError("camera uniform must hold 72 floats")
    c = Camera_t()
    ctypes.memmove(ctypes.addressof(c), u.tobytes(), 288)
    return c
