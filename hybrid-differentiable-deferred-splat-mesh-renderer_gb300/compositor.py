"""Python mirror of the reference compute-compositor operator API.

Same names (snake_case), argument meaning and call order as
src/gpuTileSplatCompositor.ts, over the C ABI of libhdsr.so:

  plan_tile_splat_compositor              planTileSplatCompositor   :109-139
  create_tile_splat_compositor            createTileSplatCompositor :141-728
  create_tile_splat_bind_groups           createTileSplatBindGroups :792-995
  write_tile_splat_frame_uniforms         writeTileSplatFrameUniforms :730-774
  write_frame_uniform_buffer              device.queue.writeBuffer (splatRenderer.ts:1030)
  encode_full_compute_compositor_pipeline encodeFullComputeCompositorPipeline :1023-1179
  encode_composite_only                   encodeCompositeOnly :1001-1014

The "encoder" is a CUDA stream (torch.cuda.Stream, a raw handle, or None for
torch's current stream). Device buffers are torch tensors; the handle only
borrows them, and the bind-group object keeps them alive.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib

TILE_SPLAT_FRAME_UNIFORM_FLOATS = 64
PROJ_STRIDE_U32 = 14


@dataclass(frozen=True)
class TileSplatCompositorPlan:
    viewport_width: int
    viewport_height: int
    tile_size_px: int
    tile_columns: int
    tile_rows: int
    tile_count: int
    morton_tile_count: int
    splat_count: int
    max_total_tile_refs: int

    def _c(self) -> _lib.Plan:
        return _lib.Plan(self.viewport_width, self.viewport_height, self.tile_size_px, self.tile_columns,
                         self.tile_rows, self.tile_count, self.morton_tile_count, self.splat_count,
                         self.max_total_tile_refs)


def plan_tile_splat_compositor(viewport_width: int, viewport_height: int, tile_size_px: int, splat_count: int,
                               tile_entry_multiplier: float | None = None) -> TileSplatCompositorPlan:
    lib = _lib.load()
    inp = _lib.PlanInput(viewport_width, viewport_height, tile_size_px, splat_count,
                         float(tile_entry_multiplier or 0.0))
    out = _lib.Plan()
    _lib.check(lib.hdsr_plan_tile_splat_compositor(ctypes.byref(inp), ctypes.byref(out)), None, "plan")
    return TileSplatCompositorPlan(*(getattr(out, f) for f, _ in _lib.Plan._fields_))


def _stream_handle(stream) -> ctypes.c_void_p:
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(stream.cuda_stream)


class TileSplatCompositorResources:
    """Owner of one compositor handle (and of every internal device buffer)."""

    def __init__(self, plan: TileSplatCompositorPlan, pair_capacity: int = 0, f32_color: bool = False,
                 keep_sorted_keys: bool = False, backward: bool = False, tile_entries: bool = False,
                 f16: bool = False):
        self.plan = plan
        self._lib = _lib.load()
        flags = ((_lib.CFG_KEEP_SORTED_KEYS if keep_sorted_keys else 0) | (_lib.CFG_BACKWARD if backward else 0)
                 | (_lib.CFG_TILE_ENTRIES if tile_entries else 0) | (_lib.CFG_F16_COMPOSITE if f16 else 0))
        cfg = _lib.Config(int(pair_capacity), _lib.COLOR_RGBA32F if f32_color else _lib.COLOR_RGBA16F, flags)
        handle = ctypes.c_void_p()
        status = self._lib.hdsr_create_tile_splat_compositor(ctypes.byref(plan._c()), ctypes.byref(cfg),
                                                             ctypes.byref(handle))
        _lib.check(status, None, "create_tile_splat_compositor")
        self.handle = handle
        self.f32_color = f32_color
        self.bind_groups = None
        # no frame yet: the lookup builds nothing
        self._pair_capacity = self.buffer_address("tile_entries")[1] // 4

    @property
    def pair_capacity(self) -> int:
        return self._pair_capacity

    def destroy(self) -> None:
        if self.handle:
            self._lib.hdsr_destroy_tile_splat_compositor(self.handle)
            self.handle = None
        self.bind_groups = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def buffer_address(self, name: str) -> tuple[int, int]:
        ptr = ctypes.c_void_p()
        size = ctypes.c_uint64()
        status = self._lib.hdsr_get_buffer(self.handle, _lib.BUFFER_IDS[name], ctypes.byref(ptr), ctypes.byref(size))
        _lib.check(status, self.handle, f"get_buffer({name})")
        return int(ptr.value or 0), int(size.value)

    def buffer(self, name: str, dtype=None, count: int | None = None):
        """Zero-copy torch view of an internal device buffer."""
        import torch

        ptr, size = self.buffer_address(name)
        dtype = dtype or (torch.int64 if name in ("sorted_keys", "superblock_lists", "chunk_masks") else torch.int32)
        itemsize = torch.empty((), dtype=dtype).element_size()
        n = size // itemsize if count is None else count
        return _DeviceView(ptr, n, dtype).tensor()

    def rank_bits(self) -> int:
        return int(self._lib.hdsr_rank_bits(self.handle))

    def chunk_ranges(self):
        """The hot-tile chunk table of the last full frame (chunkRanges of
        gpu_tile_bucket_sort.wgsl:110-143), from the tile counts and offsets."""
        return chunk_ranges_from_tiles(self.buffer("tile_counts").cpu().numpy().view(np.uint32),
                                       self.buffer("tile_offsets").cpu().numpy().view(np.uint32))

    def set_profiling(self, enable: bool = True) -> None:
        _lib.check(self._lib.hdsr_set_profiling(self.handle, 1 if enable else 0), self.handle, "set_profiling")

    def set_scan_wait(self, spin_limit: int = 0, withheld_tile: int | None = None) -> None:
        """Bound of the scans' decoupled-lookback waits (0: the default 2^22
        spins) and the test hook that keeps one scan tile from posting."""
        tile = 0xFFFFFFFF if withheld_tile is None else int(withheld_tile)
        _lib.check(self._lib.hdsr_set_scan_wait(self.handle, int(spin_limit), tile), self.handle, "set_scan_wait")

    def pass_times(self) -> list[tuple[str, float]]:
        """(pass name, ms) of the last profiled encode, in launch order."""
        ms = (ctypes.c_float * 32)()
        ids = (ctypes.c_uint32 * 32)()
        n = ctypes.c_uint32()
        _lib.check(self._lib.hdsr_pass_times(self.handle, ms, ids, 32, ctypes.byref(n)), self.handle, "pass_times")
        return [(self._lib.hdsr_pass_name(ids[i]).decode(), float(ms[i])) for i in range(n.value)]

    def launch_count(self) -> int:
        return int(self._lib.hdsr_launch_count(self.handle))

    def query_status(self) -> dict:
        st = _lib.FrameStats()
        status = self._lib.hdsr_query_status(self.handle, ctypes.byref(st))
        out = {f: getattr(st, f) for f, _ in _lib.FrameStats._fields_ if not f.startswith("_")}
        out["status"] = status
        return out

    def check_frame(self) -> dict:
        st = self.query_status()
        if st["status"] != _lib.HDSR_OK:
            _lib.check(st["status"], self.handle, "frame")
        return st


class _DeviceView:
    """__cuda_array_interface__ wrapper so torch can alias handle memory."""

    _typestr = {"torch.int32": "<i4", "torch.int64": "<i8", "torch.float32": "<f4", "torch.uint8": "|u1"}

    def __init__(self, ptr: int, n: int, dtype):
        self.ptr, self.n, self.dtype = ptr, n, dtype

    @property
    def __cuda_array_interface__(self):
        return {"shape": (self.n,), "typestr": self._typestr[str(self.dtype)], "data": (self.ptr, False),
                "version": 2, "strides": None}

    def tensor(self):
        import torch

        return torch.as_tensor(self, device="cuda")


def chunk_ranges_from_tiles(tile_counts, tile_offsets, max_tile_entries: int = 4096) -> np.ndarray:
    """(start, count) per chunk of every hot tile (more than 4096 entries), in
    ascending Morton order, as the bucket cascade packs them
    (gpu_tile_bucket_sort.wgsl:110-143: buckets in order, 4096 entries per
    chunk, the last one partial). The entries of a tile are already in bucket
    order at its offset, so chunk k is positions [4096 k, 4096 k + 4096) of it."""
    counts = np.asarray(tile_counts, np.int64)
    offsets = np.asarray(tile_offsets, np.int64)
    rows = []
    for t in np.nonzero(counts > max_tile_entries)[0]:
        c, o = int(counts[t]), int(offsets[t])
        rows.extend((o + k, min(max_tile_entries, c - k)) for k in range(0, c, max_tile_entries))
    return np.asarray(rows, np.uint32).reshape(-1, 2)


def create_tile_splat_compositor(plan: TileSplatCompositorPlan, pair_capacity: int = 0, f32_color: bool = False,
                                 keep_sorted_keys: bool = False, backward: bool = False,
                                 tile_entries: bool = False, f16: bool = False) -> TileSplatCompositorResources:
    """createTileSplatCompositor (gpuTileSplatCompositor.ts:141-728); `f16` is its
    {f16} option, the f16 composite variant."""
    return TileSplatCompositorResources(plan, pair_capacity, f32_color, keep_sorted_keys, backward, tile_entries,
                                        f16)


def sort_back_to_front(stream, resources: TileSplatCompositorResources, view, out) -> None:
    """sortedIndices on the device (hdsr_sort_back_to_front): the back-to-front
    order of the bound positions for `view` (16 floats, column-major) into
    `out` (int32/uint32 CUDA tensor of splat_count), as back_to_front_order
    computes it on the host."""
    v = np.ascontiguousarray(np.asarray(view, np.float32).reshape(-1))
    assert v.size == 16
    st = resources._lib.hdsr_sort_back_to_front(resources.handle, v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                ctypes.c_void_p(_ptr(out)), _stream_handle(stream))
    _lib.check(st, resources.handle, "sort_back_to_front")


def encode_backward(stream, resources: TileSplatCompositorResources, d_color, grads: dict) -> None:
    """Adjoint of the last full encode (hdsr_encode_backward).

    d_color: (H, W, 4) float32 CUDA tensor, dL/d(color output). grads: float32
    CUDA tensors positions (N, 3), log_scales (N, 3), rotations (N, 4),
    opacities (N,), sh (N, 6 + 3K); overwritten with the gradients."""
    assert d_color.dtype.itemsize == 4 and d_color.is_contiguous()
    gv = _lib.GradViews(_ptr(d_color), int(d_color.stride(0) * 4), _ptr(grads["positions"]),
                        _ptr(grads["log_scales"]), _ptr(grads["rotations"]), _ptr(grads["opacities"]),
                        _ptr(grads["sh"]))
    _lib.check(resources._lib.hdsr_encode_backward(resources.handle, ctypes.byref(gv), _stream_handle(stream)),
               resources.handle, "encode_backward")


@dataclass
class TileSplatCompositorBindGroups:
    splat_buffers: dict
    output_texture: object
    gbuffer_textures: dict


def _ptr(t) -> int:
    return 0 if t is None else int(t.data_ptr())


def create_tile_splat_bind_groups(resources: TileSplatCompositorResources, splat_buffers: dict, output_texture,
                                  gbuffer_textures: dict) -> TileSplatCompositorBindGroups:
    """Bind the caller's splat buffers and output textures (headless buffers).

    splat_buffers: positions, scales, rotations, opacities, material, normals
    (or None), sh_data, sorted_indices (torch CUDA tensors), sh_degree.
    output_texture: (H, W, 4) float16 or float32 tensor; gbuffer_textures:
    depth (H, W) float32, normal (H, W) int32, material (H, W, 4) int32.
    """
    lib = resources._lib
    p = resources.plan
    normals = splat_buffers.get("normals")
    sv = _lib.SceneViews(
        p.splat_count, int(splat_buffers.get("sh_degree", 0)), _ptr(splat_buffers["positions"]),
        _ptr(splat_buffers["scales"]), _ptr(splat_buffers["rotations"]), _ptr(splat_buffers["opacities"]),
        _ptr(splat_buffers["material"]), _ptr(normals), 0 if normals is None else int(normals.numel()),
        _ptr(splat_buffers["sh_data"]), _ptr(splat_buffers["sorted_indices"]))
    _lib.check(lib.hdsr_bind_scene(resources.handle, ctypes.byref(sv)), resources.handle, "bind_scene")
    color = output_texture
    depth, normal, material = gbuffer_textures["depth"], gbuffer_textures["normal"], gbuffer_textures["material"]

    def pitch(t):
        return int(t.stride(0) * t.element_size())

    ov = _lib.OutputViews(_ptr(color), pitch(color), _ptr(depth), pitch(depth), _ptr(normal), pitch(normal),
                          _ptr(material), pitch(material))
    _lib.check(lib.hdsr_bind_outputs(resources.handle, ctypes.byref(ov)), resources.handle, "bind_outputs")
    bg = TileSplatCompositorBindGroups(dict(splat_buffers), output_texture, dict(gbuffer_textures))
    resources.bind_groups = bg
    return bg


def create_output_textures(plan: TileSplatCompositorPlan, f32_color: bool = False, device="cuda"):
    """Headless stand-ins for the output and G-buffer textures."""
    import torch

    h, w = plan.viewport_height, plan.viewport_width
    color = torch.zeros((h, w, 4), dtype=torch.float32 if f32_color else torch.float16, device=device)
    gb = {
        "depth": torch.zeros((h, w), dtype=torch.float32, device=device),
        "normal": torch.zeros((h, w), dtype=torch.int32, device=device),
        "material": torch.zeros((h, w, 4), dtype=torch.int32, device=device),
    }
    return color, gb


def write_tile_splat_frame_uniforms(target, view_proj, plan: TileSplatCompositorPlan, splat_scale: float = 1.0,
                                    sh_degree: int = 0, camera_pos=None, view_matrix=None, proj_matrix=None,
                                    normal_matrix=None) -> np.ndarray:
    lib = _lib.load()
    if target is None:
        target = np.zeros(TILE_SPLAT_FRAME_UNIFORM_FLOATS, np.float32)
    assert target.dtype == np.float32 and target.size == TILE_SPLAT_FRAME_UNIFORM_FLOATS

    def fp(a, n):
        if a is None:
            return None
        arr = np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
        assert arr.size == n
        return arr

    vp, cam, view, proj, nm = (fp(view_proj, 16), fp(camera_pos, 3), fp(view_matrix, 16), fp(proj_matrix, 16),
                               fp(normal_matrix, 9))
    keep = [vp, cam, view, proj, nm]

    def cptr(a):
        return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    lib.hdsr_write_tile_splat_frame_uniforms(target.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), cptr(vp),
                                             ctypes.byref(plan._c()), float(splat_scale), int(sh_degree), cptr(cam),
                                             cptr(view), cptr(proj), cptr(nm))
    del keep
    return target


def write_frame_uniform_buffer(resources: TileSplatCompositorResources, data: np.ndarray) -> None:
    data = np.ascontiguousarray(data, np.float32)
    status = resources._lib.hdsr_set_frame_uniforms(resources.handle,
                                                    data.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    _lib.check(status, resources.handle, "set_frame_uniforms")


def encode_full_compute_compositor_pipeline(stream, resources: TileSplatCompositorResources,
                                            bind_groups: TileSplatCompositorBindGroups | None = None) -> None:
    status = resources._lib.hdsr_encode_full(resources.handle, _stream_handle(stream))
    _lib.check(status, resources.handle, "encode_full")


def encode_composite_only(stream, resources: TileSplatCompositorResources,
                          bind_groups: TileSplatCompositorBindGroups | None = None) -> None:
    status = resources._lib.hdsr_encode_composite_only(resources.handle, _stream_handle(stream))
    _lib.check(status, resources.handle, "encode_composite_only")


def frame_uniforms_for(plan: TileSplatCompositorPlan, camera, sh_degree: int = 0, splat_scale: float = 1.0):
    """Uniform block for an OrbitCamera, as splatRenderer.renderFrame builds it."""
    fr = camera.frame(plan.viewport_width, plan.viewport_height)
    u = write_tile_splat_frame_uniforms(None, fr["view_proj"], plan, splat_scale, sh_degree, fr["camera_pos"],
                                        fr["view"], fr["proj"], None)
    return u, fr
