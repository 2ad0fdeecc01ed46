"""Host-side camera matching the reference's conventions.

Orbit pose, view matrix and perspective follow src/camera.ts:286-363
(cameraBasis, cameraBackVector, viewMatrixFromPose, perspective with WebGPU
depth [0,1]); the viewer's vertical flip follows src/realSmokeScene.ts:27-32
and composeFirstSmokeViewProjection (:239-241). JavaScript evaluates these in
double precision and stores each element into a Float32Array; the functions
below do the same (float64 arithmetic, float32 results).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

VIEWER_VERTICAL_FLIP = np.array([1, 0, 0, 0, 0, -1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1], dtype=np.float32)


def mul_mat4(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """src/math.ts mulMat4: column-major, double accumulation, f32 store."""
    a = np.asarray(a, dtype=np.float32).astype(np.float64)
    b = np.asarray(b, dtype=np.float32).astype(np.float64)
    out = np.zeros(16, dtype=np.float32)
    for i in range(4):
        for j in range(4):
            s = a[0 * 4 + i] * b[j * 4 + 0]
            s = s + a[1 * 4 + i] * b[j * 4 + 1]
            s = s + a[2 * 4 + i] * b[j * 4 + 2]
            s = s + a[3 * 4 + i] * b[j * 4 + 3]
            out[j * 4 + i] = np.float32(s)
    return out


def perspective(fov_y: float, aspect: float, near: float, far: float) -> np.ndarray:
    f = 1.0 / math.tan(fov_y / 2.0)
    range_inv = 1.0 / (near - far)
    return np.array([f / aspect, 0, 0, 0, 0, f, 0, 0, 0, 0, far * range_inv, -1, 0, 0, near * far * range_inv, 0],
                    dtype=np.float64).astype(np.float32)


@dataclass
class OrbitCamera:
    """Orbit camera state of src/camera.ts (createCamera defaults)."""

    azimuth: float = 0.0
    elevation: float = 0.3
    distance: float = 3.0
    target: tuple = (0.0, 0.0, 0.0)
    pan_offset: tuple = (0.0, 0.0, 0.0)
    fov_y: float = math.pi / 3.0
    near: float = 0.01
    far: float = 100.0
    extra: dict = field(default_factory=dict)

    def back(self):
        ce = math.cos(self.elevation)
        return (ce * math.sin(self.azimuth), math.sin(self.elevation), ce * math.cos(self.azimuth))

    def position(self):
        b = self.back()
        return tuple(self.target[i] + self.pan_offset[i] + b[i] * self.distance for i in range(3))

    def view_matrix(self) -> np.ndarray:
        eye = self.position()
        back = self.back()
        right = (math.cos(self.azimuth), 0.0, -math.sin(self.azimuth))
        up = (back[1] * right[2] - back[2] * right[1],
              back[2] * right[0] - back[0] * right[2],
              back[0] * right[1] - back[1] * right[0])
        fz = back
        return np.array([
            right[0], up[0], fz[0], 0,
            right[1], up[1], fz[1], 0,
            right[2], up[2], fz[2], 0,
            -(right[0] * eye[0] + right[1] * eye[1] + right[2] * eye[2]),
            -(up[0] * eye[0] + up[1] * eye[1] + up[2] * eye[2]),
            -(fz[0] * eye[0] + fz[1] * eye[1] + fz[2] * eye[2]),
            1,
        ], dtype=np.float64).astype(np.float32)

    def projection(self, width: int, height: int) -> np.ndarray:
        return perspective(self.fov_y, width / height, self.near, self.far)

    def frame(self, width: int, height: int) -> dict:
        view = self.view_matrix()
        proj = self.projection(width, height)
        vp = mul_mat4(VIEWER_VERTICAL_FLIP, mul_mat4(proj, view))
        return {
            "view": view,
            "proj": proj,
            "view_proj": vp,
            "camera_pos": np.array(self.position(), dtype=np.float32),
        }


def look_from(position, target=(0.0, 0.0, 0.0), **kw) -> OrbitCamera:
    """Orbit camera at `position` looking at `target` (azimuth/elevation form)."""
    d = np.asarray(position, dtype=np.float64) - np.asarray(target, dtype=np.float64)
    dist = float(np.linalg.norm(d))
    el = math.asin(d[1] / dist)
    az = math.atan2(d[0], d[2])
    return OrbitCamera(azimuth=az, elevation=el, distance=dist, target=tuple(map(float, target)), **kw)
