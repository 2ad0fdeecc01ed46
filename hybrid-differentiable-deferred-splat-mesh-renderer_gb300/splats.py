"""Splat attribute packing and upload — the input contract of the compositor.

Mirrors src/splats.ts of the reference:
  - f32_to_f16_trunc        f32ToF16 (:431-442), truncating, no rounding
  - pack_material_buffer    packMaterialBuffer (:456-466), defaults 0.75 / 0.0
  - pack_normal_buffer      packNormalBuffer (:448-454)
  - pack_sh_data_buffer     packShDataBuffer (:471-500): dc3 | sh 3K | emissive3
  - upload_splat_attribute_buffers  uploadSplatAttributeBuffers (:376-428)
Opacities are clamped to [0, 1] as splatRenderer.loadScene does (:875-880).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def f32_to_f16_trunc(values) -> np.ndarray:
    """Bit-exact restatement of f32ToF16: underflow -> signed zero,
    overflow -> signed inf, mantissa truncated (vectorised)."""
    bits = np.asarray(values, dtype=np.float32).view(np.uint32).astype(np.int64)
    sign = (bits >> 16) & 0x8000
    exp = ((bits >> 23) & 0xFF) - 127 + 15
    frac = bits & 0x7FFFFF
    out = sign | (np.clip(exp, 0, 31) << 10) | (frac >> 13)
    out = np.where(exp <= 0, sign, out)
    out = np.where(exp >= 31, sign | 0x7C00, out)
    return out.astype(np.uint16)


def pack_material_buffer(count: int, roughness=None, metalness=None) -> np.ndarray:
    r = np.full(count, 0.75, np.float32) if roughness is None else np.asarray(roughness, np.float32)
    m = np.zeros(count, np.float32) if metalness is None else np.asarray(metalness, np.float32)
    return f32_to_f16_trunc(r).astype(np.uint32) | (f32_to_f16_trunc(m).astype(np.uint32) << 16)


def pack_normal_buffer(count: int, normals, detail_normals=None) -> np.ndarray:
    n = np.asarray(normals, np.float32).reshape(-1)
    if detail_normals is None:
        return n
    out = np.zeros(count * 6, np.float32)
    out[: count * 3] = n
    out[count * 3:] = np.asarray(detail_normals, np.float32).reshape(-1)
    return out


def sh_coefficient_count(degree: int) -> int:
    return (degree + 1) * (degree + 1) - 1


def pack_sh_data_buffer(dc_colors, sh=None, emissive=None) -> np.ndarray:
    dc = np.asarray(dc_colors, np.float32).reshape(-1, 3)
    n = dc.shape[0]
    sh_stride = 0 if sh is None else np.asarray(sh).reshape(n, -1).shape[1]
    out = np.zeros((n, 3 + sh_stride + 3), np.float32)
    out[:, :3] = dc
    if sh is not None:
        out[:, 3:3 + sh_stride] = np.asarray(sh, np.float32).reshape(n, -1)
    if emissive is not None:
        out[:, 3 + sh_stride:] = np.asarray(emissive, np.float32).reshape(n, 3)
    return out.reshape(-1)


@dataclass
class SplatAttributes:
    """Host splat attributes (src/splats.ts SplatAttributes :38-60)."""

    positions: np.ndarray          # (N,3) f32
    scales: np.ndarray             # (N,3) f32 log scales
    rotations: np.ndarray          # (N,4) f32 wxyz
    opacities: np.ndarray          # (N,) f32 activated
    colors: np.ndarray             # (N,3) f32 SH DC / RGB
    sh: np.ndarray | None = None   # (N, 3K) f32 'splat_coeff_rgb' layout
    sh_degree: int = 0
    normals: np.ndarray | None = None
    detail_normals: np.ndarray | None = None
    roughness: np.ndarray | None = None
    metalness: np.ndarray | None = None
    emissive: np.ndarray | None = None
    splat_scale: float = 1.0

    @property
    def count(self) -> int:
        return int(self.positions.shape[0])


@dataclass
class PackedSplats:
    """Host arrays in the device layout of SplatGpuBuffers (:70-83)."""

    count: int
    sh_degree: int
    positions: np.ndarray
    scales: np.ndarray
    rotations: np.ndarray
    opacities: np.ndarray
    material: np.ndarray
    normals: np.ndarray | None
    sh_data: np.ndarray


def pack_splat_attributes(attr: SplatAttributes) -> PackedSplats:
    n = attr.count
    normals = None
    if attr.normals is not None:
        normals = pack_normal_buffer(n, attr.normals, attr.detail_normals)
    return PackedSplats(
        count=n,
        sh_degree=attr.sh_degree,
        positions=np.ascontiguousarray(attr.positions, np.float32).reshape(-1),
        scales=np.ascontiguousarray(attr.scales, np.float32).reshape(-1),
        rotations=np.ascontiguousarray(attr.rotations, np.float32).reshape(-1),
        opacities=np.clip(np.asarray(attr.opacities, np.float32), 0.0, 1.0).astype(np.float32),
        material=pack_material_buffer(n, attr.roughness, attr.metalness),
        normals=normals,
        sh_data=pack_sh_data_buffer(attr.colors, attr.sh, attr.emissive),
    )


def upload_splat_attribute_buffers(packed: PackedSplats, sorted_indices: np.ndarray, device="cuda"):
    """Device copies (torch tensors) of the packed arrays plus sortedIndices."""
    import torch

    def t(x, dtype=None):
        arr = np.ascontiguousarray(x)
        if arr.dtype == np.uint32:
            arr = arr.view(np.int32)
        return torch.from_numpy(arr).to(device)

    return {
        "positions": t(packed.positions),
        "scales": t(packed.scales),
        "rotations": t(packed.rotations),
        "opacities": t(packed.opacities),
        "material": t(packed.material),
        "normals": None if packed.normals is None else t(packed.normals),
        "sh_data": t(packed.sh_data),
        "sorted_indices": t(np.asarray(sorted_indices, np.uint32)),
        "sh_degree": packed.sh_degree,
        "count": packed.count,
    }


def back_to_front_order(positions: np.ndarray, view: np.ndarray) -> np.ndarray:
    """sortedIndices as the reference produces them (gpuSortPrototype.ts:
    120-163): key = f32(-viewZ), descending, ties by ascending id."""
    p = np.asarray(positions, np.float32).reshape(-1, 3).astype(np.float64)
    v = np.asarray(view, np.float32).astype(np.float64)
    z = v[2] * p[:, 0] + v[6] * p[:, 1] + v[10] * p[:, 2] + v[14]
    keys = (-z).astype(np.float32)
    ids = np.arange(p.shape[0], dtype=np.int64)
    return np.lexsort((ids, -keys.astype(np.float64))).astype(np.uint32)
