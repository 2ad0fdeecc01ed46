"""Shared set-up for the GPU parity tests: render one frame through the C
ABI and the same frame with the oracle, and read every stage back."""
from __future__ import annotations

import numpy as np

SENTINEL = 0xFFFFFFFF


def u32(t):
    return t.cpu().numpy().view(np.uint32)


def render_gpu(pkg, scene, cam, W, H, *, f32_color=False, keep_keys=True, pair_capacity=0, order=None,
               sh_degree=None, tile_entries=False, f16=False):
    import torch

    packed = pkg.splats.pack_splat_attributes(scene)
    deg = scene.sh_degree if sh_degree is None else sh_degree
    plan = pkg.plan_tile_splat_compositor(W, H, 16, scene.count)
    u, fr = pkg.frame_uniforms_for(plan, cam, sh_degree=deg)
    if order is None:
        order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    res = pkg.create_tile_splat_compositor(plan, pair_capacity=pair_capacity, f32_color=f32_color,
                                           keep_sorted_keys=keep_keys, tile_entries=tile_entries, f16=f16)
    bufs = pkg.splats.upload_splat_attribute_buffers(packed, order)
    color, gb = pkg.create_output_textures(plan, f32_color=f32_color)
    pkg.create_tile_splat_bind_groups(res, bufs, color, gb)
    pkg.write_frame_uniform_buffer(res, u)
    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    return dict(res=res, plan=plan, u=u, packed=packed, order=order, color=color, gb=gb, bufs=bufs, f16=f16)


def read_gpu(g) -> dict:
    res = g["res"]
    st = res.query_status()
    P = int(st["total_pairs"])
    N = g["plan"].splat_count
    out = dict(status=st, P=P)
    P = min(P, int(st["pair_capacity"]))  # an overflowing frame fails on its status, not on the readback
    out["geo"] = u32(res.buffer("cache_geo", count=4 * N)).reshape(N, 4)
    out["app"] = u32(res.buffer("cache_app", count=4 * N)).reshape(N, 4)
    out["gb"] = u32(res.buffer("cache_gb", count=4 * N)).reshape(N, 4)
    out["aux"] = u32(res.buffer("cache_aux", count=2 * N)).reshape(N, 2)
    out["depth"] = u32(res.buffer("depth", count=N))
    out["tile_counts"] = u32(res.buffer("tile_counts"))
    out["tile_offsets"] = u32(res.buffer("tile_offsets"))
    out["tile_entries"] = u32(res.buffer("tile_entries", count=P))
    try:
        import torch

        out["sorted_keys"] = res.buffer("sorted_keys", dtype=torch.int64, count=P).cpu().numpy().view(np.uint64)
    except Exception:
        out["sorted_keys"] = None
    out["rank_bits"] = res.rank_bits()
    c = g["color"]
    out["color"] = c.cpu().numpy()
    out["out_depth"] = g["gb"]["depth"].cpu().numpy()
    out["normal"] = g["gb"]["normal"].cpu().numpy().view(np.uint32)
    out["material"] = g["gb"]["material"].cpu().numpy().view(np.uint32)
    return out


def cache_words(gpu: dict) -> np.ndarray:
    """GPU SoA streams re-assembled into the reference's 14-word rows."""
    N = gpu["geo"].shape[0]
    w = np.zeros((N, 14), np.uint32)
    w[:, 0:4] = gpu["geo"]
    w[:, 4], w[:, 6], w[:, 9], w[:, 10] = gpu["app"].T
    w[:, 5], w[:, 8], w[:, 11], w[:, 12] = gpu["gb"].T
    w[:, 7], w[:, 13] = gpu["aux"].T
    return w


def assert_frame_parity(orc, g, gpu=None, check_keys=True):
    """Bit-exact comparison of every stage with the oracle's canonical frame."""
    gpu = gpu or read_gpu(g)
    # the GPU's pair count sizes the oracle's entry list (one pass, no regrow)
    ref = orc.render_frame(g["u"], g["packed"], g["order"], f16=g.get("f16", False), cap=gpu["P"] + 16)
    assert gpu["status"]["status"] == 0, gpu["status"]
    assert gpu["P"] == ref["total_pairs"]
    # projection cache (visible splats: every word; invisible: the sentinel)
    cw = cache_words(gpu)
    vis = ref["proj_cache"][:, 7] != SENTINEL
    assert np.array_equal(cw[:, 7], ref["proj_cache"][:, 7])
    assert np.array_equal(gpu["depth"][vis], ref["depth"][vis])
    diff = cw[vis] != ref["proj_cache"][vis]
    assert not diff.any(), f"cache words differ: {np.nonzero(diff.any(0))[0].tolist()} ({int(diff.sum())} words)"
    assert np.array_equal(gpu["tile_counts"], ref["tile_counts"])
    assert np.array_equal(gpu["tile_offsets"], ref["tile_offsets"])
    if check_keys and gpu["sorted_keys"] is not None:
        # 20-bit log-depth keys: per entry bit-exact against the oracle's
        # mapping, and non-decreasing inside every tile (the final order is
        # the key order refined by depth bits, sortRank)
        keys, vals = orc.sorted_keys20(g["u"], ref["proj_cache"], ref["depth"])
        R = np.uint64(gpu["rank_bits"])
        gk = gpu["sorted_keys"]
        g_rank = (gk & ((np.uint64(1) << R) - np.uint64(1))).astype(np.uint32)
        assert np.array_equal(g_rank, ref["tile_entries"])
        g_key = gk >> R
        ro = np.lexsort((vals, keys))
        go = np.lexsort((g_rank, g_key))
        assert np.array_equal(g_key[go], keys[ro]) and np.array_equal(g_rank[go], vals[ro])
        assert np.all(g_key[1:] >= g_key[:-1])
    assert np.array_equal(gpu["tile_entries"], ref["tile_entries"])
    ref_color = orc.f16_to_f32(ref["color"].reshape(-1)).reshape(ref["H"], ref["W"], 4)
    got_color = gpu["color"].astype(np.float32)
    err = float(np.abs(got_color - ref_color).max()) if got_color.size else 0.0
    assert err <= 1.0 / 255.0, err
    if gpu["color"].dtype == np.float16:
        assert np.array_equal(gpu["color"].view(np.uint16), ref["color"])
    assert np.array_equal(gpu["out_depth"].view(np.uint32), ref["out_depth"].view(np.uint32))
    assert np.array_equal(gpu["normal"], ref["normal"])
    assert np.array_equal(gpu["material"], ref["material"])
    return gpu, ref
