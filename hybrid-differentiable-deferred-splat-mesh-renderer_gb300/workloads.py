"""Seeded synthetic scenes for the compositor's benchmark configurations.

No public dataset is involved: every scene is drawn from numpy's PCG64 with a
fixed seed, in the shapes and value distributions of the configurations:
  plain50k     50k Gaussians, 800x600, means U[-2,2]^3, log-scales N(-3.5,0.5),
               quats normalise(N(0,1)^4), opacity sigmoid(N(0,1.5)), SH0 U[0,1],
               camera at (0,0,5) looking at the origin, fov 60 deg, seed 0.
  hot760k      760k Gaussians, 1920x1080: 70% on 6 seeded planes with N(0,0.01)
               normal jitter, 30% U[-3,3]^3; one log-scale axis N(-5,0.3), two
               N(-2.5,0.5) (axis seeded per splat); opacity sigmoid(N(1,1));
               SH0; camera chosen so that >= 20 tiles hold > 4096 entries.
  sh3_3m       3M Gaussians (hot760k means), SH3 (48 coefficients: DC U[0,1],
               higher bands N(0,0.05)), 3840x2160, 8-camera orbit at radius 6.
  train500k    500k Gaussians (hot760k distribution), SH1, 1024x1024.
Opacities fed to the compositor are activated (sigmoid) and clamped to [0,1].
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .camera import OrbitCamera, look_from
from .splats import SplatAttributes


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _sigmoid(x):
    return (1.0 / (1.0 + np.exp(-x))).astype(np.float32)


def _unit_quats(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def plain_scene(n: int = 50_000, seed: int = 0) -> SplatAttributes:
    rng = _rng(seed)
    pos = rng.uniform(-2.0, 2.0, (n, 3)).astype(np.float32)
    scl = rng.normal(-3.5, 0.5, (n, 3)).astype(np.float32)
    rot = _unit_quats(rng, n)
    opa = _sigmoid(rng.normal(0.0, 1.5, n))
    col = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    return SplatAttributes(positions=pos, scales=scl, rotations=rot, opacities=opa, colors=col)


def planes_means(rng, n: int) -> np.ndarray:
    """70% of means on 6 seeded planes (N(0,0.01) normal jitter), 30% U[-3,3]^3."""
    n_plane = int(round(n * 0.7))
    normals = rng.standard_normal((6, 3))
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    offsets = rng.uniform(-1.5, 1.5, 6)
    which = rng.integers(0, 6, n_plane)
    nrm = normals[which]
    helper = np.where(np.abs(nrm[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    t1 = np.cross(nrm, helper)
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(nrm, t1)
    uv = rng.uniform(-3.0, 3.0, (n_plane, 2))
    jit = rng.normal(0.0, 0.01, n_plane)
    p_plane = nrm * (offsets[which] + jit)[:, None] + t1 * uv[:, :1] + t2 * uv[:, 1:]
    p_free = rng.uniform(-3.0, 3.0, (n - n_plane, 3))
    pos = np.concatenate([p_plane, p_free], axis=0)
    perm = rng.permutation(n)
    return pos[perm].astype(np.float32)


def anisotropic_log_scales(rng, n: int) -> np.ndarray:
    scl = rng.normal(-2.5, 0.5, (n, 3))
    thin = rng.integers(0, 3, n)
    scl[np.arange(n), thin] = rng.normal(-5.0, 0.3, n)
    return scl.astype(np.float32)


def hot_scene(n: int = 760_000, seed: int = 2, sh_degree: int = 0) -> SplatAttributes:
    rng = _rng(seed)
    pos = planes_means(rng, n)
    scl = anisotropic_log_scales(rng, n)
    rot = _unit_quats(rng, n)
    opa = _sigmoid(rng.normal(1.0, 1.0, n))
    col = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    sh = None
    if sh_degree > 0:
        k = (sh_degree + 1) ** 2 - 1
        sh = rng.normal(0.0, 0.05, (n, 3 * k)).astype(np.float32)
    return SplatAttributes(positions=pos, scales=scl, rotations=rot, opacities=opa, colors=col, sh=sh,
                           sh_degree=sh_degree)


@dataclass
class Workload:
    name: str
    scene: SplatAttributes
    width: int
    height: int
    cameras: list

    def describe(self) -> dict:
        return {"workload": self.name, "splats": self.scene.count, "width": self.width, "height": self.height,
                "sh_degree": self.scene.sh_degree, "cameras": len(self.cameras)}


# Camera of the hot-tile stress scene: the first of hot_camera_candidates()
# (seed 7) with >= 20 tiles above 4096 entries. With this scale distribution
# every candidate qualifies: this pose gives about 40M (tile, splat) pairs
# and about 3,200 hot tiles. Recorded so every run renders the same frame.
HOT760K_CAMERA = dict(azimuth=3.927590651355011, elevation=0.47665656116349064, distance=6.766271296348564)


def plain50k() -> Workload:
    return Workload("plain50k_800x600", plain_scene(50_000, 0), 800, 600, [look_from((0.0, 0.0, 5.0))])


def hot760k() -> Workload:
    return Workload("hot760k_1920x1080", hot_scene(760_000, 2), 1920, 1080, [OrbitCamera(**HOT760K_CAMERA)])


def hot190k() -> Workload:
    """A quarter of the hot-tile workload (same distribution and camera), for
    profiler captures that must stay small (about 10M pairs)."""
    return Workload("hot190k_1920x1080", hot_scene(190_000, 2), 1920, 1080, [OrbitCamera(**HOT760K_CAMERA)])


def orbit_cameras(count: int, radius: float, elevation: float = 0.25) -> list:
    return [OrbitCamera(azimuth=2.0 * math.pi * i / count, elevation=elevation, distance=radius)
            for i in range(count)]


def sh3_3m() -> Workload:
    return Workload("sh3_3m_3840x2160", hot_scene(3_000_000, 3, sh_degree=3), 3840, 2160, orbit_cameras(8, 6.0))


def train500k() -> Workload:
    return Workload("train500k_1024x1024", hot_scene(500_000, 5, sh_degree=1), 1024, 1024,
                    [OrbitCamera(azimuth=0.4, elevation=0.2, distance=6.0)])


def hot_camera_candidates(seed: int = 7, count: int = 64) -> list:
    rng = _rng(seed)
    return [OrbitCamera(azimuth=float(rng.uniform(0, 2 * math.pi)), elevation=float(rng.uniform(-0.6, 0.6)),
                        distance=float(rng.uniform(2.5, 8.0))) for _ in range(count)]


WORKLOADS = {"plain50k": plain50k, "hot760k": hot760k, "hot190k": hot190k, "sh3_3m": sh3_3m,
             "train500k": train500k}
