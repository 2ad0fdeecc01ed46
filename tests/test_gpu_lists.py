"""The superblock lists and their chunk masks, read back through the C ABI
and compared with lists built from the oracle's frame: every visible splat in
ascending (depth bits, sortRank) order, one entry per superblock of 8x8 tiles
its tile box meets (the box clipped to the superblock as the local rect),
grouped by superblock; and per 32 entries the union of their rects as tile
bits. The rasteriser reads a tile's entries through these (the walk itself is
checked against the per-tile lists in test_oracle.py)."""
import dataclasses

import numpy as np
import pytest

from gpu_helpers import SENTINEL, render_gpu


def rect_tiles(rc: np.ndarray) -> np.ndarray:
    rc = rc.astype(np.uint64)
    x0, x1, y0, y1 = rc & 7, (rc >> 3) & 7, (rc >> 6) & 7, rc >> 9
    m = np.zeros(rc.shape, np.uint64)
    for y in range(8):
        for x in range(8):
            inside = (x0 <= x) & (x <= x1) & (y0 <= y) & (y <= y1)
            m |= np.where(inside, np.uint64(1) << np.uint64(y * 8 + x), np.uint64(0))
    return m


def superblock_lists(box: np.ndarray, depth: np.ndarray, cols: int, rows: int) -> np.ndarray:
    """(superblock << 36 | rect << 24 | sortRank) of every visible splat in
    (depth bits, sortRank) order, grouped by superblock (a stable sort)."""
    sb_cols = (cols + 7) // 8
    vis = np.nonzero(box != SENTINEL)[0]
    o = vis[np.lexsort((vis, depth[vis]))].astype(np.int64)
    b = box[o].astype(np.int64)
    x0, y0, x1, y1 = b & 255, (b >> 8) & 255, (b >> 16) & 255, b >> 24
    keys, pos = [], []
    for dy in range(3):  # a tile box meets at most 3x3 superblocks
        for dx in range(3):
            sx, sy = (x0 >> 3) + dx, (y0 >> 3) + dy
            ok = (sx <= x1 >> 3) & (sy <= y1 >> 3)
            lx0 = np.maximum(x0 - 8 * sx, 0); lx1 = np.minimum(x1 - 8 * sx, 7)
            ly0 = np.maximum(y0 - 8 * sy, 0); ly1 = np.minimum(y1 - 8 * sy, 7)
            rc = lx0 | lx1 << 3 | ly0 << 6 | ly1 << 9
            k = (sy * sb_cols + sx) << 36 | rc << 24 | o
            keys.append(k[ok]); pos.append((np.arange(len(o)) * 9 + dy * 3 + dx)[ok])
    keys, pos = np.concatenate(keys), np.concatenate(pos)
    keys = keys[np.argsort(pos, kind="stable")]  # depth order, then superblocks in row-major order
    return keys[np.argsort(keys >> 36, kind="stable")].astype(np.uint64)


def straddle_case(pkg):
    """A ragged grid (not a whole number of superblocks) with large splats
    (tile boxes up to 17 tiles a side) that straddle superblock edges."""
    scene = pkg.workloads.plain_scene(6000, seed=23)
    scene = dataclasses.replace(scene, scales=scene.scales + 1.5)
    return scene, pkg.workloads.plain50k().cameras[0], 1000, 600


def test_list_construction_filters_to_the_oracle_tile_lists(pkg, orc):
    # the construction the GPU lists are compared with: filtered by each
    # tile's local position it gives the oracle's per-tile lists
    scene, cam, W, H = straddle_case(pkg)
    packed = pkg.splats.pack_splat_attributes(scene)
    plan = pkg.plan_tile_splat_compositor(W, H, 16, scene.count)
    u, fr = pkg.frame_uniforms_for(plan, cam, sh_degree=0)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    ref = orc.render_frame(u, packed, order, composite=False, cap=scene.count * 300)
    cols, rows = (W + 15) // 16, (H + 15) // 16
    lists = superblock_lists(ref["proj_cache"][:, 7], ref["depth"], cols, rows)
    sb, rc = lists >> np.uint64(36), (lists >> np.uint64(24)) & np.uint64(0xFFF)
    ent, cnt, off = ref["tile_entries"], ref["tile_counts"], ref["tile_offsets"]
    for ty in range(rows):
        for tx in range(cols):
            m = int(np.asarray(orc.morton(tx, ty)).reshape(-1)[0])
            lx, ly = tx & 7, ty & 7
            sel = (sb == (ty >> 3) * ((cols + 7) // 8) + (tx >> 3)) & ((rc & 7) <= lx) & (((rc >> 3) & 7) >= lx) \
                & (((rc >> 6) & 7) <= ly) & ((rc >> 9) >= ly)
            got = (lists[sel] & np.uint64(0xFFFFFF)).astype(np.uint32)
            assert np.array_equal(got, ent[off[m]:off[m] + cnt[m]]), (tx, ty)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["plain50k", "sb_straddle"])
def test_superblock_lists_and_chunk_masks_match_the_oracle(cuda, pkg, orc, case):
    import torch

    if case == "plain50k":
        wl = pkg.workloads.plain50k()
        scene, cam, W, H = wl.scene, wl.cameras[0], wl.width, wl.height
    else:
        scene, cam, W, H = straddle_case(pkg)
    g = render_gpu(pkg, scene, cam, W, H, pair_capacity=scene.count * 300)
    st = g["res"].query_status()
    assert st["status"] == 0
    Q = int(st["superblock_entries"])
    lists = g["res"].buffer("superblock_lists", count=Q).cpu().numpy().view(np.uint64)
    masks = g["res"].buffer("chunk_masks", count=(Q + 31) // 32).cpu().numpy().view(np.uint64)
    ref = orc.render_frame(g["u"], g["packed"], g["order"], composite=False, cap=int(st["total_pairs"]) + 16)
    cols, rows = (W + 15) // 16, (H + 15) // 16
    want = superblock_lists(ref["proj_cache"][:, 7], ref["depth"], cols, rows)
    assert Q == len(want)
    assert np.array_equal(lists, want)
    tiles = rect_tiles((want >> np.uint64(24)) & np.uint64(0xFFF))
    pad = np.zeros(((Q + 31) // 32) * 32, np.uint64)
    pad[:Q] = tiles
    want_masks = np.bitwise_or.reduce(pad.reshape(-1, 32), axis=1)
    assert np.array_equal(masks, want_masks)
    # a second frame (graph replay) writes the same masks from zero
    pkg.encode_full_compute_compositor_pipeline(None, g["res"])
    pkg.encode_full_compute_compositor_pipeline(None, g["res"])
    torch.cuda.synchronize()
    assert np.array_equal(g["res"].buffer("chunk_masks", count=(Q + 31) // 32).cpu().numpy().view(np.uint64), want_masks)
    g["res"].destroy()
