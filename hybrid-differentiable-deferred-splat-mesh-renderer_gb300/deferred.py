"""The deferred frame tail over the compositor's G-buffer (C ABI hdsr_post_*).

Mirrors what src/splatRenderer.ts:1042-1139 encodes after the compositor:
screen-space normals, the bilateral normal filter, GTAO, bloom, material
curves, IBL and deferred lighting, each a CUDA kernel in libhdsr.so. Host-side
restatements beside them:
  mat4_inverse            mat4Inverse (splatRenderer.ts:148-168), double
                          arithmetic, f32 results, None when |det| < 1e-10
  light_direction         computeLightDirection (main.ts:257-281)
  f32_to_f16_ibl          ibl.ts f32ToF16 (:158-189): the environment upload's
                          rounding (ties away from zero, subnormals kept,
                          NaN -> 0x7C01)
  decode_radiance_hdr     decodeRadianceHDR (ibl.ts:192-276), parse_hdr_header
                          (:279-285)
  frame_params            the per-frame uniforms of each pass's encode()
The reference fetches its default environment (a 1k Poly Haven HDRI) over the
network; synthetic_environment() is a seeded stand-in of the same 2:1 shape.
"""
from __future__ import annotations

import ctypes
import math
import re

import numpy as np

from . import _lib
from .compositor import _DeviceView, _ptr, _stream_handle

# main.ts DEFAULT_SETTINGS :144-169
FIXED_LIGHT_AZIMUTH = 0.8
FIXED_LIGHT_ELEVATION = 0.6
LIGHT_MODES = ("camera", "fixed", "overhead", "rim")


def mat4_inverse(m) -> np.ndarray | None:
    a = [float(v) for v in np.asarray(m, np.float32).reshape(16)]
    a00, a01, a02, a03, a10, a11, a12, a13, a20, a21, a22, a23, a30, a31, a32, a33 = a
    b00 = a00 * a11 - a01 * a10; b01 = a00 * a12 - a02 * a10; b02 = a00 * a13 - a03 * a10
    b03 = a01 * a12 - a02 * a11; b04 = a01 * a13 - a03 * a11; b05 = a02 * a13 - a03 * a12
    b06 = a20 * a31 - a21 * a30; b07 = a20 * a32 - a22 * a30; b08 = a20 * a33 - a23 * a30
    b09 = a21 * a32 - a22 * a31; b10 = a21 * a33 - a23 * a31; b11 = a22 * a33 - a23 * a32
    det = b00 * b11 - b01 * b10 + b02 * b09 + b03 * b08 - b04 * b07 + b05 * b06
    if abs(det) < 1e-10:
        return None
    det = 1 / det
    o = [(a11 * b11 - a12 * b10 + a13 * b09) * det, (a02 * b10 - a01 * b11 - a03 * b09) * det,
         (a31 * b05 - a32 * b04 + a33 * b03) * det, (a22 * b04 - a21 * b05 - a23 * b03) * det,
         (a12 * b08 - a10 * b11 - a13 * b07) * det, (a00 * b11 - a02 * b08 + a03 * b07) * det,
         (a32 * b02 - a30 * b05 - a33 * b01) * det, (a20 * b05 - a22 * b02 + a23 * b01) * det,
         (a10 * b10 - a11 * b08 + a13 * b06) * det, (a01 * b08 - a00 * b10 - a03 * b06) * det,
         (a30 * b04 - a31 * b02 + a33 * b00) * det, (a21 * b02 - a20 * b04 - a23 * b00) * det,
         (a11 * b07 - a10 * b09 - a12 * b06) * det, (a00 * b09 - a01 * b07 + a02 * b06) * det,
         (a31 * b01 - a30 * b03 - a32 * b00) * det, (a20 * b03 - a21 * b01 + a22 * b00) * det]
    return np.array(o, np.float64).astype(np.float32)


def light_direction(mode: str, camera_pos, target=(0.0, 0.0, 0.0), fixed_azimuth: float = FIXED_LIGHT_AZIMUTH,
                    fixed_elevation: float = FIXED_LIGHT_ELEVATION) -> tuple:
    cam = [float(v) for v in np.asarray(camera_pos, np.float32).reshape(3)]
    if mode == "camera":
        lx, ly, lz = target[0] - cam[0], target[1] - cam[1], target[2] - cam[2]
        n = math.sqrt(lx * lx + ly * ly + lz * lz) or 1
        return lx / n, ly / n, lz / n
    if mode == "overhead":
        return 0.0, -1.0, 0.0
    if mode == "rim":
        lx, ly, lz = cam[0], -0.5, cam[2]
        n = math.sqrt(lx * lx + ly * ly + lz * lz) or 1
        return lx / n, ly / n, lz / n
    ce = math.cos(fixed_elevation)
    return math.cos(fixed_azimuth) * ce, -math.sin(fixed_elevation), math.sin(fixed_azimuth) * ce


def f32_to_f16_ibl(values) -> np.ndarray:
    bits = np.asarray(values, np.float32).view(np.uint32).astype(np.int64)
    sign = (bits >> 16) & 0x8000
    raw = (bits >> 23) & 0xFF
    frac = bits & 0x7FFFFF
    exp = raw - 127 + 15
    normal = (sign | (np.clip(exp, 0, 31) << 10) | (frac >> 13)) + ((frac >> 12) & 1)
    shift = np.clip(1 - exp, 1, 10)
    full = 0x800000 | frac
    sub = sign | ((full >> (13 + shift)) + ((full >> (12 + shift)) & 1))
    out = np.where(exp > -10, sub, sign)
    out = np.where(exp > 0, normal, out)
    out = np.where(exp >= 31, sign | 0x7C00, out)
    out = np.where(raw == 0xFF, np.where(frac != 0, sign | 0x7C01, sign | 0x7C00), out)
    return out.astype(np.uint16)


def parse_hdr_header(data: bytes) -> tuple[int, int]:
    text = data[:512].decode("latin-1")
    m = re.search(r"-Y\s+(\d+)\s+\+X\s+(\d+)", text)
    if not m:
        raise ValueError("Could not parse HDR resolution from header")
    return int(m.group(2)), int(m.group(1))


def decode_radiance_hdr(data: bytes, expected_width: int, expected_height: int) -> np.ndarray:
    """RGBE scanlines (flat or new-style RLE) -> (H, W, 4) f32, alpha 1."""
    b = np.frombuffer(data, np.uint8)
    width, height = expected_width, expected_height
    offset = 0
    limit = min(len(b), 4096)
    while offset < limit:
        end = offset
        while end < limit and b[end] != 10:
            end += 1
        line = bytes(b[offset:end]).decode("latin-1")
        offset = end + 1
        m = re.match(r"^[-+][YX]\s+(\d+)\s+[-+][YX]\s+(\d+)", line)
        if m:
            if line.startswith("-Y") or line.startswith("+Y"):
                height, width = int(m.group(1)), int(m.group(2))
            else:
                width, height = int(m.group(1)), int(m.group(2))
            break
    out = np.zeros((height, width, 4), np.float32)
    n = len(b)

    def at(i):  # a Uint8Array read past the end is undefined -> 0 in arithmetic
        return int(b[i]) if i < n else 0

    for y in range(height):
        scan = np.zeros((width, 4), np.uint8)
        if offset + 4 <= n and b[offset] == 2 and b[offset + 1] == 2:
            offset += 4
            for ch in range(4):
                x = 0
                while x < width:
                    code = at(offset); offset += 1
                    if code > 128:
                        val = at(offset); offset += 1
                        cnt = code - 128
                        scan[x:x + cnt, ch] = val
                        x += cnt
                    else:
                        for _ in range(code):
                            if x < width:
                                scan[x, ch] = at(offset)
                            offset += 1
                            x += 1
                        if code == 0:
                            break
        else:
            for x in range(width):
                scan[x] = [at(offset), at(offset + 1), at(offset + 2), at(offset + 3)]
                offset += 4
        e = scan[:, 3].astype(np.int32)
        scale = np.power(2.0, (e - 128 - 8).astype(np.float64))
        rgb = scan[:, :3].astype(np.float64) * scale[:, None]
        rgb[e == 0] = 0.0
        out[y, :, :3] = rgb.astype(np.float32)
        out[y, :, 3] = 1.0
    return out


def synthetic_environment(width: int = 1024, height: int = 512, seed: int = 0) -> np.ndarray:
    """A seeded HDR equirect (sky gradient, a sun, ground, low-frequency noise)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    lat = (0.5 - v)[:, None] * math.pi
    lon = (u - 0.5)[None, :] * 2 * math.pi
    sky = np.stack([0.35 + 0.3 * np.sin(lat), 0.5 + 0.3 * np.sin(lat), 0.9 + 0.2 * np.sin(lat)], -1)
    ground = np.array([0.25, 0.2, 0.15])
    img = np.where((lat > 0)[..., None], sky * np.ones_like(lon)[..., None], ground)
    sun_lat, sun_lon = 0.6, 0.8
    cosang = np.sin(lat) * math.sin(sun_lat) + np.cos(lat) * math.cos(sun_lat) * np.cos(lon - sun_lon)
    img = img + 40.0 * np.power(np.clip(cosang, 0, 1), 800)[..., None] * np.array([1.0, 0.95, 0.85])
    noise = rng.normal(0, 1, (height // 16 + 1, width // 16 + 1, 3))
    img = img * (1 + 0.1 * np.kron(noise, np.ones((16, 16, 1)))[:height, :width])
    out = np.ones((height, width, 4), np.float32)
    out[..., :3] = np.clip(img, 0, None)
    return out


def default_params() -> _lib.PostParams:
    q = _lib.PostParams()
    _lib.load().hdsr_post_default_params(ctypes.byref(q))
    return q


def frame_params(camera, width: int, height: int, light_mode: str = "camera", normal_recovery_mode: int = 0,
                 frame_counter: int = 0, **overrides) -> _lib.PostParams:
    """The uniforms splatRenderer.renderFrame hands each pass for an OrbitCamera frame."""
    fr = camera.frame(width, height)
    q = default_params()
    inv = mat4_inverse(fr["view_proj"])
    if inv is None:
        raise ValueError("view-projection is singular")
    q.view_proj_inverse[:] = [float(v) for v in inv]
    q.camera_pos[:] = [float(v) for v in fr["camera_pos"]]
    q.normal_recovery_mode = int(normal_recovery_mode)
    q.proj[:] = [float(v) for v in fr["proj"]]
    q.view[:] = [float(v) for v in fr["view"]]
    q.near_plane, q.far_plane = float(camera.near), float(camera.far)
    q.frame_counter = int(frame_counter)
    target = tuple(camera.target[i] + camera.pan_offset[i] for i in range(3))
    q.light_dir[:] = [float(np.float32(v)) for v in light_direction(light_mode, fr["camera_pos"], target)]
    for k, v in overrides.items():
        if not hasattr(q, k):
            raise KeyError(k)
        if isinstance(v, (list, tuple, np.ndarray)):
            getattr(q, k)[:] = [float(x) for x in v]
        else:
            setattr(q, k, v)
    return q


class DeferredPasses:
    """One hdsr_post handle: the frame tail's images for one viewport size."""

    def __init__(self, width: int, height: int):
        self._lib = _lib.load()
        self.width, self.height = int(width), int(height)
        h = ctypes.c_void_p()
        st = self._lib.hdsr_post_create(self.width, self.height, ctypes.byref(h))
        if st != _lib.HDSR_OK:
            raise _lib.HdsrError(st, "post_create")
        self.handle = h
        self._keep = None
        self.env_size = (1, 1)

    def _check(self, st, what):
        if st != _lib.HDSR_OK:
            err = self._lib.hdsr_post_last_error(self.handle)
            raise _lib.HdsrError(st, f"{what}: {err.decode() if err else ''}")

    def set_environment(self, rgba_f32, stream=None) -> None:
        """Level 0 of the equirect (H, W, 4) f32; None restores the 1x1 placeholder (no IBL)."""
        if rgba_f32 is None:
            self._check(self._lib.hdsr_post_set_environment(self.handle, None, 0, 0, _stream_handle(stream)),
                        "set_environment")
            self.env_size = (1, 1)
            return
        img = np.asarray(rgba_f32, np.float32)
        h16 = np.ascontiguousarray(f32_to_f16_ibl(img.reshape(-1)))
        self._check(self._lib.hdsr_post_set_environment(self.handle, h16.ctypes.data, img.shape[1], img.shape[0],
                                                        _stream_handle(stream)), "set_environment")
        self.env_size = (int(img.shape[1]), int(img.shape[0]))

    def set_material_curves(self, roughness=(1.0, 0.0, 1.0), metalness=(1.0, 0.0, 1.0), albedo=(1.0, 0.0, 1.0)):
        """(contrast, brightness, gamma) per curve, MaterialCurveParams of materialCurves.ts."""
        c = (ctypes.c_float * 9)(*[float(v) for v in (*roughness, *metalness, *albedo)])
        self._check(self._lib.hdsr_post_set_material_curves(self.handle, c), "set_material_curves")

    def encode(self, stream, color, gbuffer: dict, params: _lib.PostParams, lit) -> None:
        """color/gbuffer: the compositor's output textures; lit: (H, W, 4) float16."""
        import torch

        def pitch(t):
            return int(t.stride(0) * t.element_size())

        assert lit.dtype == torch.float16 and lit.shape == (self.height, self.width, 4)
        inp = _lib.PostInputs(_ptr(color), pitch(color),
                              _lib.COLOR_RGBA32F if color.dtype == torch.float32 else _lib.COLOR_RGBA16F, 0,
                              _ptr(gbuffer["depth"]), pitch(gbuffer["depth"]), _ptr(gbuffer["normal"]),
                              pitch(gbuffer["normal"]), _ptr(gbuffer["material"]), pitch(gbuffer["material"]))
        self._keep = (color, gbuffer, lit)
        self._check(self._lib.hdsr_post_encode(self.handle, ctypes.byref(inp), ctypes.byref(params), _ptr(lit),
                                               pitch(lit), _stream_handle(stream)), "post_encode")

    def buffer(self, name: str, dtype=None):
        """Zero-copy torch view of an intermediate image (flat)."""
        import torch

        ptr = ctypes.c_void_p()
        size = ctypes.c_uint64()
        self._check(self._lib.hdsr_post_get_buffer(self.handle, _lib.POST_BUFFER_IDS[name], ctypes.byref(ptr),
                                                   ctypes.byref(size)), f"get_buffer({name})")
        dtype = dtype or (torch.float32 if name.startswith("depth_mip") else torch.int32)
        item = torch.empty((), dtype=dtype).element_size()
        return _DeviceView(int(ptr.value or 0), int(size.value) // item, dtype).tensor()

    def set_profiling(self, enable: bool = True) -> None:
        self._check(self._lib.hdsr_post_set_profiling(self.handle, 1 if enable else 0), "set_profiling")

    def pass_times(self) -> list[tuple[str, float]]:
        ms = (ctypes.c_float * 7)()
        self._check(self._lib.hdsr_post_pass_times(self.handle, ms), "pass_times")
        return list(zip(_lib.POST_PASSES, (float(v) for v in ms)))

    def destroy(self) -> None:
        if getattr(self, "handle", None):
            self._lib.hdsr_post_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
