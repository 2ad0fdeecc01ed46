"""The rasteriser's work order.

Every full frame records each half tile's cost; from the second full frame
after a bind, `k_work_order` orders the tiles by the larger of their halves'
costs, most expensive first, in buckets of four per octave (the first frame
keeps the tile scan's order). The order only decides which warp takes a
tile when: the images must not depend on it.
"""
import numpy as np
import pytest

from gpu_helpers import assert_frame_parity, read_gpu, render_gpu

pytestmark = pytest.mark.gpu


def cost_bucket(c: np.ndarray) -> np.ndarray:
    """The kernels' bucket of a cost: 4 per octave of c + 1."""
    v = c.astype(np.int64) + 1
    lg = np.array([int(x).bit_length() - 1 for x in v], np.int64)
    frac = np.where(lg >= 2, (v >> np.maximum(lg - 2, 0)) & 3, (v << np.maximum(2 - lg, 0)) & 3)
    return lg * 4 + frac


def _u32(t):
    return t.cpu().numpy().view(np.uint32).copy()


def _tiles(order, cols):
    return (order >> 16) * cols + (order & 0xFFFF)


def test_cost_order_is_a_sorted_permutation_and_changes_no_pixel(cuda, pkg, orc):
    import torch

    wl = pkg.workloads.hot190k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height, keep_keys=False,
                   pair_capacity=int(wl.scene.count * 60))
    res, plan = g["res"], g["plan"]
    cols, T = plan.tile_columns, plan.tile_count
    first = read_gpu(g)
    order1 = _u32(res.buffer("work_order"))
    costs1 = _u32(res.buffer("tile_costs"))
    # the first frame: the tile scan's order, a permutation of the tiles
    assert np.array_equal(np.sort(_tiles(order1, cols)), np.arange(T))
    assert costs1.shape == (2 * T,) and (costs1 > 0).all()

    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    order2 = _u32(res.buffer("work_order"))
    t2 = _tiles(order2, cols)
    assert np.array_equal(np.sort(t2), np.arange(T))
    per_tile = np.maximum(costs1[0::2], costs1[1::2])
    b = cost_bucket(per_tile[t2])
    assert (np.diff(b) <= 0).all()  # most expensive bucket first
    assert b[0] > b[-1]  # the costs do differ on this workload
    assert not np.array_equal(order2, order1)
    # the same camera: the same per-half costs, whatever the order
    assert np.array_equal(_u32(res.buffer("tile_costs")), costs1)
    second = read_gpu(g)
    for k in ("color", "out_depth", "normal", "material"):
        assert np.array_equal(second[k].view(np.uint8), first[k].view(np.uint8)), k
    assert_frame_parity(orc, g, gpu=second, check_keys=False)

    # composite-only keeps the full frame's order
    pkg.encode_composite_only(None, res)
    torch.cuda.synchronize()
    assert np.array_equal(_u32(res.buffer("work_order")), order2)

    # a rebind clears the costs: its first frame takes the scan's order again
    pkg.create_tile_splat_bind_groups(res, g["bufs"], g["color"], g["gb"])
    pkg.write_frame_uniform_buffer(res, g["u"])
    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    t3 = _tiles(_u32(res.buffer("work_order")), cols)
    assert np.array_equal(np.sort(t3), np.arange(T))
    heavy = first["tile_counts"][orc.morton(t3 % cols, t3 // cols)] >= 1024
    assert not (np.diff(heavy.astype(np.int8)) > 0).any()  # tiles of >= 1,024 entries first
    third = read_gpu(g)
    for k in ("color", "out_depth", "normal", "material"):
        assert np.array_equal(third[k].view(np.uint8), first[k].view(np.uint8)), k

    # a camera turn of more than 10 degrees clears the costs as well: the
    # costs of the previous view describe other tiles
    import dataclasses

    cam = dataclasses.replace(wl.cameras[0], azimuth=wl.cameras[0].azimuth + 0.8)
    u2, _ = pkg.frame_uniforms_for(plan, cam, sh_degree=wl.scene.sh_degree)
    pkg.write_frame_uniform_buffer(res, u2)
    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    t4 = _tiles(_u32(res.buffer("work_order")), cols)
    assert np.array_equal(np.sort(t4), np.arange(T))
    counts4 = _u32(res.buffer("tile_counts"))
    heavy4 = counts4[orc.morton(t4 % cols, t4 // cols)] >= 1024
    assert heavy4.any() and not (np.diff(heavy4.astype(np.int8)) > 0).any()
    # a turn of a few degrees keeps them: the next frame orders by cost
    cam = dataclasses.replace(cam, azimuth=cam.azimuth + 0.02)
    u3, _ = pkg.frame_uniforms_for(plan, cam, sh_degree=wl.scene.sh_degree)
    costs4 = _u32(res.buffer("tile_costs"))
    pkg.write_frame_uniform_buffer(res, u3)
    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    t5 = _tiles(_u32(res.buffer("work_order")), cols)
    b5 = cost_bucket(np.maximum(costs4[0::2], costs4[1::2])[t5])
    assert (np.diff(b5) <= 0).all()
    res.destroy()
