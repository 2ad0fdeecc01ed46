"""Serving loop: many (scene, camera, viewport) requests over resident scenes.

A thin Python face of the C ABI's hdsr_server_* (the scheduler, slot pool,
HBM admission, CUDA graphs and streams live in libhdsr.so). Scenes are the
device tensors of splats.upload_splat_attribute_buffers, kept alive by the
server object; each request renders into caller-owned output tensors, which
are kept alive until its wait().

sortedIndices only assigns sortRanks: the frame orders every tile by (depth,
sortRank), so any fixed permutation (the identity, for serving) gives the
image of the camera's own back-to-front order except where depths tie.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .compositor import _ptr


class Server:
    def __init__(self, hbm_budget_bytes: int, max_in_flight: int = 8, use_graphs: bool = True):
        self._lib = _lib.load()
        cfg = _lib.ServerConfig(int(hbm_budget_bytes), int(max_in_flight), 0 if use_graphs else _lib.SERVER_NO_GRAPH)
        handle = ctypes.c_void_p()
        st = self._lib.hdsr_server_create(ctypes.byref(cfg), ctypes.byref(handle))
        if st != _lib.HDSR_OK:
            raise _lib.HdsrError(st, "server_create")
        self.handle = handle
        self._scenes = {}
        self._pending = {}

    def _check(self, st, what):
        if st != _lib.HDSR_OK:
            err = self._lib.hdsr_server_last_error(self.handle)
            raise _lib.HdsrError(st, f"{what}: {err.decode() if err else ''}")

    def add_scene(self, scene_id: int, bufs: dict) -> None:
        """bufs: splats.upload_splat_attribute_buffers output (kept alive)."""
        normals = bufs.get("normals")
        sv = _lib.SceneViews(
            int(bufs["count"]), int(bufs.get("sh_degree", 0)), _ptr(bufs["positions"]), _ptr(bufs["scales"]),
            _ptr(bufs["rotations"]), _ptr(bufs["opacities"]), _ptr(bufs["material"]), _ptr(normals),
            0 if normals is None else int(normals.numel()), _ptr(bufs["sh_data"]), _ptr(bufs["sorted_indices"]))
        self._check(self._lib.hdsr_server_add_scene(self.handle, int(scene_id), ctypes.byref(sv)), "add_scene")
        self._scenes[scene_id] = bufs

    def submit(self, scene_id: int, uniforms, color, gb: dict) -> int:
        """Queue one frame; color (H, W, 4) f16 or f32, gb as create_output_textures."""
        import torch

        u = np.ascontiguousarray(uniforms, np.float32)
        req = _lib.Request()
        req.scene_id = int(scene_id)
        req.color_format = _lib.COLOR_RGBA32F if color.dtype == torch.float32 else _lib.COLOR_RGBA16F
        ctypes.memmove(req.uniforms, u.ctypes.data, 256)

        def pitch(t):
            return int(t.stride(0) * t.element_size())

        req.outputs = _lib.OutputViews(_ptr(color), pitch(color), _ptr(gb["depth"]), pitch(gb["depth"]),
                                       _ptr(gb["normal"]), pitch(gb["normal"]), _ptr(gb["material"]),
                                       pitch(gb["material"]))
        ticket = ctypes.c_uint64()
        self._check(self._lib.hdsr_server_submit(self.handle, ctypes.byref(req), ctypes.byref(ticket)), "submit")
        self._pending[ticket.value] = (color, gb)
        return ticket.value

    def wait(self, ticket: int) -> dict:
        res = _lib.RequestResult()
        st = self._lib.hdsr_server_wait(self.handle, int(ticket), ctypes.byref(res))
        self._pending.pop(ticket, None)
        out = {f: getattr(res, f) for f, _ in _lib.RequestResult._fields_}
        out["wait_status"] = st
        return out

    def stats(self) -> dict:
        st = _lib.ServerStats()
        self._check(self._lib.hdsr_server_query(self.handle, ctypes.byref(st)), "query")
        return {f: getattr(st, f) for f, _ in _lib.ServerStats._fields_}

    def destroy(self) -> None:
        if self.handle:
            self._lib.hdsr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
