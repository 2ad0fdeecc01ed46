"""ctypes binding of the C ABI in include/hdsr.h (libhdsr.so).

The library is the only implementation of the compositor: when it is missing
or cannot be loaded every entry point raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_uint32, c_uint64, c_void_p
from pathlib import Path

from . import _build

HDSR_OK = 0
STATUS_NAMES = {
    0: "HDSR_OK",
    1: "HDSR_ERR_INVALID_ARG",
    2: "HDSR_ERR_OOM",
    3: "HDSR_ERR_CUDA",
    4: "HDSR_ERR_OVERFLOW",
    5: "HDSR_ERR_TIMEOUT",
    6: "HDSR_ERR_UNSUPPORTED",
    7: "HDSR_ERR_NOT_BOUND",
}
HDSR_ERR_INVALID_ARG = 1
HDSR_ERR_OOM = 2
HDSR_ERR_CUDA = 3
HDSR_ERR_OVERFLOW = 4
HDSR_ERR_TIMEOUT = 5
HDSR_ERR_UNSUPPORTED = 6
HDSR_ERR_NOT_BOUND = 7

COLOR_RGBA16F = 0
COLOR_RGBA32F = 1
CFG_KEEP_SORTED_KEYS = 0x1
CFG_NO_GRAPH = 0x2
CFG_BACKWARD = 0x4
CFG_TILE_ENTRIES = 0x8
CFG_F16_COMPOSITE = 0x10

DEV_OVERFLOW = 0x1
DEV_TIMEOUT = 0x2
DEV_BAD_INDEX = 0x4

BUFFER_IDS = {
    "cache_geo": 0,
    "cache_app": 1,
    "cache_gb": 2,
    "cache_aux": 3,
    "depth": 4,
    "tile_counts": 5,
    "tile_offsets": 6,
    "tile_entries": 7,
    "sorted_keys": 8,
    "pair_offsets": 9,
    "depth_order": 10,
    "backward_params": 11,
    "work_order": 12,
    "tile_costs": 13,
    "superblock_lists": 14,
    "chunk_masks": 15,
}


class PlanInput(ctypes.Structure):
    _fields_ = [("viewport_width", c_uint32), ("viewport_height", c_uint32), ("tile_size_px", c_uint32),
                ("splat_count", c_uint32), ("tile_entry_multiplier", c_double)]


class Plan(ctypes.Structure):
    _fields_ = [("viewport_width", c_uint32), ("viewport_height", c_uint32), ("tile_size_px", c_uint32),
                ("tile_columns", c_uint32), ("tile_rows", c_uint32), ("tile_count", c_uint32),
                ("morton_tile_count", c_uint32), ("splat_count", c_uint32), ("max_total_tile_refs", c_uint32)]


class Config(ctypes.Structure):
    _fields_ = [("pair_capacity", c_uint64), ("color_format", c_uint32), ("flags", c_uint32)]


class SceneViews(ctypes.Structure):
    _fields_ = [("splat_count", c_uint32), ("sh_degree", c_uint32), ("positions", c_void_p),
                ("scales", c_void_p), ("rotations", c_void_p), ("opacities", c_void_p), ("material", c_void_p),
                ("normals", c_void_p), ("normals_len", c_uint64), ("sh_data", c_void_p),
                ("sorted_indices", c_void_p)]


class OutputViews(ctypes.Structure):
    _fields_ = [("color", c_void_p), ("color_pitch", c_uint64), ("depth", c_void_p), ("depth_pitch", c_uint64),
                ("normal", c_void_p), ("normal_pitch", c_uint64), ("material", c_void_p),
                ("material_pitch", c_uint64)]


class GradViews(ctypes.Structure):
    _fields_ = [("d_color", c_void_p), ("d_color_pitch", c_uint64), ("d_positions", c_void_p),
                ("d_log_scales", c_void_p), ("d_rotations", c_void_p), ("d_opacities", c_void_p),
                ("d_sh", c_void_p)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", c_uint64), ("max_in_flight", c_uint32), ("flags", c_uint32)]


class Request(ctypes.Structure):
    _fields_ = [("scene_id", c_uint32), ("color_format", c_uint32), ("uniforms", c_float * 64),
                ("outputs", OutputViews)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("reruns", c_uint32), ("total_pairs", c_uint64),
                ("submit_ms", c_double), ("start_ms", c_double), ("done_ms", c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("budget_bytes", c_uint64), ("scene_bytes", c_uint64), ("slot_bytes", c_uint64),
                ("scenes", c_uint32), ("slots", c_uint32), ("graphs", c_uint32), ("evictions", c_uint32),
                ("completed", c_uint64), ("reruns", c_uint64)]


SERVER_NO_GRAPH = 0x1


class PostInputs(ctypes.Structure):
    _fields_ = [("color", c_void_p), ("color_pitch", c_uint64), ("color_format", c_uint32), ("_pad", c_uint32),
                ("depth", c_void_p), ("depth_pitch", c_uint64), ("normal", c_void_p), ("normal_pitch", c_uint64),
                ("material", c_void_p), ("material_pitch", c_uint64)]


class PostParams(ctypes.Structure):
    """hdsr_post_params; the oracle's orp_params has the same layout."""

    _fields_ = [("view_proj_inverse", c_float * 16), ("camera_pos", c_float * 3), ("normal_recovery_mode", c_uint32),
                ("grazing_start", c_float), ("grazing_end", c_float), ("bilateral_spatial_sigma", c_float),
                ("bilateral_depth_sigma", c_float), ("bilateral_normal_sigma", c_float),
                ("bilateral_radius", c_uint32), ("proj", c_float * 16), ("view", c_float * 16),
                ("near_plane", c_float), ("far_plane", c_float), ("ao_radius_world", c_float),
                ("ao_falloff_end", c_float), ("ao_intensity", c_float), ("ao_thickness", c_float),
                ("ao_slices", c_uint32), ("ao_steps", c_uint32), ("frame_counter", c_uint32),
                ("ao_denoise_strength", c_float), ("bloom_threshold", c_float), ("bloom_soft_knee", c_float),
                ("light_dir", c_float * 3), ("light_intensity", c_float), ("ambient_intensity", c_float),
                ("specular_only", c_uint32), ("emissive_intensity", c_float), ("emissive_threshold", c_float),
                ("env_intensity", c_float), ("env_rotation", c_float), ("exposure", c_float),
                ("fallback_roughness", c_float), ("fallback_metallic", c_float)]


POST_BUFFER_IDS = {
    "screen_normals": 0, "normals": 1, "depth_mip0": 2, "depth_mip1": 3, "depth_mip2": 4, "ao_raw": 5, "ao": 6,
    "bloom": 7, "bloom_h": 8, "brdf_lut": 9, "env": 10, "curves": 11,
}
POST_PASSES = ("ss_normals", "bilateral", "gtao_prefilter", "gtao_main", "gtao_denoise", "bloom", "lighting")


class FrameStats(ctypes.Structure):
    _fields_ = [("total_pairs", c_uint64), ("pair_capacity", c_uint64), ("visible_splats", c_uint32),
                ("superblock_entries", c_uint32), ("hot_tiles", c_uint32), ("chunks", c_uint32),
                ("device_flags", c_uint32), ("segments", c_uint32), ("depth_sort_passes", c_uint32),
                ("reserved", c_uint32)]


class HdsrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# name -> (restype, argtypes)
SIGNATURES = {
    "hdsr_abi_version": (c_uint32, []),
    "hdsr_plan_tile_splat_compositor": (c_int, [POINTER(PlanInput), POINTER(Plan)]),
    "hdsr_create_tile_splat_compositor": (c_int, [POINTER(Plan), POINTER(Config), POINTER(c_void_p)]),
    "hdsr_destroy_tile_splat_compositor": (None, [c_void_p]),
    "hdsr_bind_scene": (c_int, [c_void_p, POINTER(SceneViews)]),
    "hdsr_bind_outputs": (c_int, [c_void_p, POINTER(OutputViews)]),
    "hdsr_encode_backward": (c_int, [c_void_p, POINTER(GradViews), c_void_p]),
    "hdsr_sort_back_to_front": (c_int, [c_void_p, POINTER(c_float), c_void_p, c_void_p]),
    "hdsr_server_create": (c_int, [POINTER(ServerConfig), POINTER(c_void_p)]),
    "hdsr_server_destroy": (None, [c_void_p]),
    "hdsr_server_add_scene": (c_int, [c_void_p, c_uint32, POINTER(SceneViews)]),
    "hdsr_server_submit": (c_int, [c_void_p, POINTER(Request), POINTER(c_uint64)]),
    "hdsr_server_wait": (c_int, [c_void_p, c_uint64, POINTER(RequestResult)]),
    "hdsr_server_query": (c_int, [c_void_p, POINTER(ServerStats)]),
    "hdsr_server_last_error": (c_char_p, [c_void_p]),
    "hdsr_write_tile_splat_frame_uniforms": (None, [POINTER(c_float), POINTER(c_float), POINTER(Plan), c_float,
                                                    c_uint32, POINTER(c_float), POINTER(c_float),
                                                    POINTER(c_float), POINTER(c_float)]),
    "hdsr_set_frame_uniforms": (c_int, [c_void_p, POINTER(c_float)]),
    "hdsr_encode_full": (c_int, [c_void_p, c_void_p]),
    "hdsr_encode_composite_only": (c_int, [c_void_p, c_void_p]),
    "hdsr_query_status": (c_int, [c_void_p, POINTER(FrameStats)]),
    "hdsr_last_error": (c_char_p, [c_void_p]),
    "hdsr_get_buffer": (c_int, [c_void_p, c_int, POINTER(c_void_p), POINTER(c_uint64)]),
    "hdsr_rank_bits": (c_uint32, [c_void_p]),
    "hdsr_set_profiling": (c_int, [c_void_p, c_int]),
    "hdsr_pass_times": (c_int, [c_void_p, POINTER(c_float), POINTER(c_uint32), c_uint32, POINTER(c_uint32)]),
    "hdsr_pass_name": (c_char_p, [c_uint32]),
    "hdsr_launch_count": (c_uint64, [c_void_p]),
    "hdsr_set_scan_wait": (c_int, [c_void_p, c_uint32, c_uint32]),
    "hdsr_post_create": (c_int, [c_uint32, c_uint32, POINTER(c_void_p)]),
    "hdsr_post_destroy": (None, [c_void_p]),
    "hdsr_post_default_params": (None, [POINTER(PostParams)]),
    "hdsr_post_set_environment": (c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p]),
    "hdsr_post_set_material_curves": (c_int, [c_void_p, POINTER(c_float)]),
    "hdsr_post_encode": (c_int, [c_void_p, POINTER(PostInputs), POINTER(PostParams), c_void_p, c_uint64, c_void_p]),
    "hdsr_post_get_buffer": (c_int, [c_void_p, c_int, POINTER(c_void_p), POINTER(c_uint64)]),
    "hdsr_post_set_profiling": (c_int, [c_void_p, c_int]),
    "hdsr_post_pass_times": (c_int, [c_void_p, POINTER(c_float)]),
    "hdsr_post_last_error": (c_char_p, [c_void_p]),
    "hdsr_count_tile_refs_static": (c_int, [c_void_p, c_uint32, c_uint64, c_uint32, c_uint32, c_void_p, c_uint64,
                                            c_void_p]),
}

_LIB = None


def library_path() -> Path:
    return _build.library_path()


def load(path: str | Path | None = None) -> ctypes.CDLL:
    """Load libhdsr.so (raises when it is missing: build() first)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else library_path()
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run the package build (nvcc for sm_103a) before use")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def check(status: int, handle=None, what: str = "") -> None:
    if status != HDSR_OK:
        msg = what
        if handle is not None:
            err = load().hdsr_last_error(handle)
            msg = f"{what}: {err.decode() if err else ''}"
        raise HdsrError(status, msg)
