"""hdsr_count_tile_refs_static: the allocation-free tile count entry point.

Collected last on purpose: it shares the library's static scratch with
nothing else, and must pass both alone and after every other test. Its
counts are integers, so the tolerance is exact equality with the tile
counts of the full-frame entry point (hdsr_encode_full) on the same frame.
"""
import ctypes

import numpy as np
import pytest

from gpu_helpers import render_gpu, u32


def _static_counts(pkg, lib, boxes_ptr, stride, n, plan, out, stream=None):
    return lib.hdsr_count_tile_refs_static(
        ctypes.c_void_p(boxes_ptr), stride, n, plan.tile_columns, plan.tile_rows,
        ctypes.c_void_p(out.data_ptr()), out.numel(),
        ctypes.c_void_p(0 if stream is None else stream.cuda_stream))


def test_rejects_grids_beyond_the_static_scratch(hdsr_lib):
    # argument checks run before any device work: no GPU needed
    rc = hdsr_lib.hdsr_count_tile_refs_static(None, 1, 0, 256, 8, ctypes.c_void_p(16), 1 << 20, None)
    assert rc == 6  # HDSR_ERR_UNSUPPORTED
    rc = hdsr_lib.hdsr_count_tile_refs_static(None, 1, 0, 8, 300, ctypes.c_void_p(16), 1 << 20, None)
    assert rc == 6
    rc = hdsr_lib.hdsr_count_tile_refs_static(None, 1, 0, 8, 8, ctypes.c_void_p(16), 3, None)
    assert rc == 1  # output shorter than the Morton tile count


@pytest.mark.gpu
def test_static_counts_match_full_frame_two_calls_in_a_row(cuda, pkg, orc, hdsr_lib):
    import torch

    frames = []
    # two different frames (different tile grids), counted back to back
    wl = pkg.workloads.plain50k()
    frames.append(render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height, keep_keys=False))
    scene = pkg.workloads.hot_scene(40_000, 6)
    cam = pkg.camera.OrbitCamera(**pkg.workloads.HOT760K_CAMERA)
    frames.append(render_gpu(pkg, scene, cam, 1920, 1080, keep_keys=False, pair_capacity=8_000_000))
    outs = []
    stream = torch.cuda.Stream()
    for g in frames:
        plan = g["plan"]
        aux = g["res"].buffer("cache_aux", count=2 * plan.splat_count)
        out = torch.full((plan.morton_tile_count,), -1, dtype=torch.int32, device="cuda")
        # the fill above ran on the current stream: order the side stream
        # after it, and keep both tensors alive for the side stream's use
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(stream):
            rc = _static_counts(pkg, hdsr_lib, aux.data_ptr(), 2, plan.splat_count, plan, out, stream)
        out.record_stream(stream)
        aux.record_stream(stream)
        assert rc == 0
        outs.append(out)
    stream.synchronize()
    for g, out in zip(frames, outs):
        want = u32(g["res"].buffer("tile_counts"))
        got = u32(out)
        assert np.array_equal(got, want)
        assert got.sum() == g["res"].query_status()["total_pairs"]
    # a second round on the default stream: scratch left over from the
    # calls above must not leak into the counts
    for g in reversed(frames):
        plan = g["plan"]
        aux = g["res"].buffer("cache_aux", count=2 * plan.splat_count)
        out = torch.zeros((plan.morton_tile_count,), dtype=torch.int32, device="cuda")
        assert _static_counts(pkg, hdsr_lib, aux.data_ptr(), 2, plan.splat_count, plan, out) == 0
        torch.cuda.synchronize()
        assert np.array_equal(u32(out), u32(g["res"].buffer("tile_counts")))
    # the reference's 14-word projection cache rows: the tile box is word 7,
    # so the caller passes the address of row 0's word 7 with stride 14
    g = frames[0]
    plan = g["plan"]
    aux = g["res"].buffer("cache_aux", count=2 * plan.splat_count).view(-1, 2)
    rows = torch.zeros((plan.splat_count, 14), dtype=torch.int32, device="cuda")
    rows[:, 7] = aux[:, 0]
    rows[:, 0:7] = -1  # other words hold unrelated bits
    rows[:, 8:] = -1
    out = torch.full((plan.morton_tile_count,), 3, dtype=torch.int32, device="cuda")
    assert _static_counts(pkg, hdsr_lib, rows.data_ptr() + 7 * 4, 14, plan.splat_count, plan, out) == 0
    torch.cuda.synchronize()
    assert np.array_equal(u32(out), u32(g["res"].buffer("tile_counts")))
    for g in frames:
        g["res"].destroy()


@pytest.mark.gpu
def test_static_counts_of_an_empty_frame(cuda, pkg, hdsr_lib):
    import torch

    plan = pkg.plan_tile_splat_compositor(40, 24, 16, 0)
    out = torch.full((plan.morton_tile_count,), 7, dtype=torch.int32, device="cuda")
    assert _static_counts(pkg, hdsr_lib, 0, 1, 0, plan, out) == 0
    torch.cuda.synchronize()
    assert not u32(out).any()
