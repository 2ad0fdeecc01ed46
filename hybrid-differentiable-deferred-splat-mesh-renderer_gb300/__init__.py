"""GB300 tile-splat compositor (drop-in for the reference compute compositor).

The compute path is libhdsr.so (hand-written sm_103a CUDA behind the C ABI in
include/hdsr.h); this package is the host-side mirror of the reference's
operator API plus scene packing, camera conventions and synthetic workloads.
"""
from . import _build, _lib, assets, camera, deferred, differentiable, ply, serving, splats, workloads
from .compositor import (
    TileSplatCompositorPlan,
    TileSplatCompositorResources,
    create_output_textures,
    create_tile_splat_bind_groups,
    create_tile_splat_compositor,
    encode_backward,
    encode_composite_only,
    encode_full_compute_compositor_pipeline,
    frame_uniforms_for,
    plan_tile_splat_compositor,
    sort_back_to_front,
    write_frame_uniform_buffer,
    write_tile_splat_frame_uniforms,
)

build = _build.build
load_library = _lib.load

__all__ = [
    "TileSplatCompositorPlan",
    "TileSplatCompositorResources",
    "assets",
    "build",
    "camera",
    "create_output_textures",
    "create_tile_splat_bind_groups",
    "create_tile_splat_compositor",
    "deferred",
    "differentiable",
    "encode_backward",
    "serving",
    "encode_composite_only",
    "encode_full_compute_compositor_pipeline",
    "frame_uniforms_for",
    "load_library",
    "plan_tile_splat_compositor",
    "ply",
    "sort_back_to_front",
    "splats",
    "workloads",
    "write_frame_uniform_buffer",
    "write_tile_splat_frame_uniforms",
]
