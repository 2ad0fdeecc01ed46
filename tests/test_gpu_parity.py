"""Parity of the CUDA path (through the C ABI) with the oracle.

Integer / index stages (tile counts, offsets, radix keys, per-tile order) are
bit-exact. The image is checked bit-exact too (the kernels and the oracle
share one op sequence); the benchmark spec's tolerance, max |err| <= 1/255 per
channel, is asserted alongside.
"""
import math

import numpy as np
import pytest

from gpu_helpers import assert_frame_parity, read_gpu, render_gpu

pytestmark = pytest.mark.gpu


def _fp64_error(orc, g, gpu, ref):
    """Max |err| and PSNR of the GPU colour against the FP64 twin (same entry
    lists, double arithmetic, no f16 quantisation)."""
    f64 = orc.render_frame_f64(g["u"], g["packed"], g["order"], ref)
    got = gpu["color"].astype(np.float64)
    err = np.abs(got - f64)
    mse = float(np.mean((got[..., :3] - f64[..., :3]) ** 2))
    psnr = 10.0 * math.log10(1.0 / max(mse, 1e-30))
    return float(err.max()), psnr


def test_plain50k_800x600_parity(cuda, pkg, orc):
    wl = pkg.workloads.plain50k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height)
    gpu, ref = assert_frame_parity(orc, g)
    assert ref["total_pairs"] > 50_000
    # accuracy against FP64: PSNR >= 50 dB (the image is the f16 output)
    err, psnr = _fp64_error(orc, g, gpu, ref)
    assert psnr >= 50.0, (err, psnr)
    g["res"].destroy()


def test_profiled_and_forked_frames_are_identical(cuda, pkg, orc):
    # with profiling the frame runs on one stream; without it the tile counts
    # and tile scan run beside the depth sort on the handle's second stream
    import torch

    wl = pkg.workloads.plain50k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height)
    res = g["res"]
    snap = lambda: [t.clone() for t in (g["color"], g["gb"]["depth"], g["gb"]["normal"], g["gb"]["material"],
                                         res.buffer("tile_entries", count=int(res.query_status()["total_pairs"])))]
    forked = snap()
    res.set_profiling(True)
    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    names = [n for n, _ in res.pass_times()]
    res.set_profiling(False)
    serial = snap()
    assert "tile_counts" in names and "raster" in names
    for a, b in zip(forked, serial):
        assert torch.equal(a.view(torch.int16) if a.dtype == torch.float16 else a, b.view(torch.int16) if b.dtype == torch.float16 else b)
    assert_frame_parity(orc, g)
    res.destroy()


def test_one_splat(cuda, pkg, orc):
    scene = pkg.splats.SplatAttributes(
        positions=np.array([[0.1, -0.2, 0.0]], np.float32), scales=np.full((1, 3), -2.0, np.float32),
        rotations=np.array([[0.9, 0.1, 0.3, -0.2]], np.float32), opacities=np.array([0.8], np.float32),
        colors=np.array([[0.9, 0.4, 0.1]], np.float32))
    g = render_gpu(pkg, scene, pkg.camera.look_from((0, 0, 4)), 96, 80)
    assert_frame_parity(orc, g)


def test_empty_scene_writes_background(cuda, pkg, orc):
    scene = pkg.splats.SplatAttributes(
        positions=np.zeros((0, 3), np.float32), scales=np.zeros((0, 3), np.float32),
        rotations=np.zeros((0, 4), np.float32), opacities=np.zeros(0, np.float32), colors=np.zeros((0, 3), np.float32))
    g = render_gpu(pkg, scene, pkg.camera.look_from((0, 0, 4)), 40, 24)
    gpu = read_gpu(g)
    assert gpu["P"] == 0
    c = gpu["color"].astype(np.float32)
    assert np.allclose(c[..., 0], np.float16(0.02)) and np.allclose(c[..., 2], np.float16(0.04))
    assert not c[..., 3].any()


def test_behind_camera_and_ragged_viewport(cuda, pkg, orc):
    rng = np.random.default_rng(8)
    scene = pkg.workloads.plain_scene(3000, seed=8)
    scene.positions[:500, 2] = rng.uniform(5.0, 9.0, 500).astype(np.float32)  # behind the camera at z=4.5
    g = render_gpu(pkg, scene, pkg.camera.look_from((0, 0, 4.5)), 203, 117)
    gpu, ref = assert_frame_parity(orc, g)
    assert (ref["proj_cache"][:, 7] == 0xFFFFFFFF).sum() >= 500


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_sh_normals_material_emissive(cuda, pkg, orc, deg):
    rng = np.random.default_rng(deg)
    n = 4000
    scene = pkg.workloads.plain_scene(n, seed=20 + deg)
    k = (deg + 1) ** 2 - 1
    scene.sh = rng.normal(0, 0.2, (n, 3 * k)).astype(np.float32)
    scene.sh_degree = deg
    scene.normals = rng.normal(0, 1, (n, 3)).astype(np.float32)
    scene.normals[::7] = 0.0  # falls back to the covariance normal
    if deg >= 2:
        scene.detail_normals = rng.normal(0, 0.3, (n, 3)).astype(np.float32) + np.array([0, 0, 1], np.float32)
    scene.roughness = rng.uniform(0, 1, n).astype(np.float32)
    scene.metalness = rng.uniform(0, 1, n).astype(np.float32)
    scene.emissive = rng.uniform(0, 2, (n, 3)).astype(np.float32)
    g = render_gpu(pkg, scene, pkg.camera.OrbitCamera(azimuth=0.3, elevation=0.2, distance=4.5), 160, 128)
    assert_frame_parity(orc, g)


def _hot_scene(pkg, n_stack=9000, n_rand=20000, seed=3):
    rng = np.random.default_rng(seed)
    base = pkg.workloads.plain_scene(n_rand, seed=seed)
    p = np.concatenate([np.tile(np.array([[0.72, -0.72, 0.0]], np.float32), (n_stack, 1)), base.positions])
    p[:n_stack, 2] += rng.uniform(-0.5, 0.5, n_stack).astype(np.float32)
    p[:n_stack, :2] += rng.normal(0, 0.05, (n_stack, 2)).astype(np.float32)
    s = np.concatenate([np.full((n_stack, 3), -4.5, np.float32), base.scales])
    r = np.concatenate([np.tile(np.array([[1, 0, 0, 0]], np.float32), (n_stack, 1)), base.rotations])
    o = np.concatenate([np.full(n_stack, 0.3, np.float32), base.opacities])
    c = np.concatenate([rng.uniform(0, 1, (n_stack, 3)).astype(np.float32), base.colors])
    return pkg.splats.SplatAttributes(positions=p, scales=s, rotations=r, opacities=o, colors=c)


def test_hot_tiles_bucket_cascade(cuda, pkg, orc):
    scene = _hot_scene(pkg)
    g = render_gpu(pkg, scene, pkg.camera.look_from((0, 0, 5)), 128, 96)
    gpu, ref = assert_frame_parity(orc, g)
    assert ref["hot_tiles"] >= 1 and ref["total_chunks"] >= 3
    assert gpu["status"]["hot_tiles"] == ref["hot_tiles"]
    assert gpu["status"]["chunks"] == ref["total_chunks"]


def test_4k_viewport_two_superblock_passes(cuda, pkg, orc):
    # 240 x 135 tiles = 30 x 17 superblocks of 8x8 tiles: more than 256, so
    # the superblock lists take two 8-bit radix passes; ragged last row and
    # column of superblocks
    scene = pkg.workloads.hot_scene(60_000, 4)
    cam = pkg.camera.OrbitCamera(**pkg.workloads.HOT760K_CAMERA)
    g = render_gpu(pkg, scene, cam, 3840, 2160, pair_capacity=16_000_000)
    gpu, ref = assert_frame_parity(orc, g)
    assert g["res"].query_status()["superblock_entries"] > 0
    g["res"].destroy()


def test_single_superblock_viewport(cuda, pkg, orc):
    # 8 x 8 tiles: one superblock, a 1-bit superblock digit
    scene = pkg.workloads.plain_scene(3000, 9)
    g = render_gpu(pkg, scene, pkg.camera.look_from((0.2, 0.1, 3.0)), 128, 128)
    assert_frame_parity(orc, g)
    g["res"].destroy()


def test_near_plane_splats_negative_depth(cuda, pkg, orc):
    """Splats between the camera and the near plane have negative NDC depth:
    their tiles' log-depth range collapses (every entry in bucket 0) and u32
    depth order puts them after every positive depth; order stays exact."""
    scene = pkg.workloads.plain_scene(6000, seed=12)
    cam = pkg.camera.look_from((0.0, 0.0, 4.0))
    rng = np.random.default_rng(12)
    # 40 splats 3-8 mm in front of the camera (near plane at 10 mm)
    scene.positions[:40] = np.stack([rng.uniform(-1e-3, 1e-3, 40), rng.uniform(-1e-3, 1e-3, 40),
                                     4.0 - rng.uniform(0.003, 0.008, 40)], 1).astype(np.float32)
    scene.scales[:40] = -9.0
    g = render_gpu(pkg, scene, cam, 160, 128)
    gpu, ref = assert_frame_parity(orc, g)
    assert (ref["depth"].view(np.float32) < 0).any()


def test_equal_depth_ties(cuda, pkg, orc):
    n = 5000
    rng = np.random.default_rng(4)
    scene = pkg.splats.SplatAttributes(
        positions=np.tile(np.array([[0.72, -0.72, 0.0]], np.float32), (n, 1)),
        scales=np.full((n, 3), -5.0, np.float32), rotations=np.tile(np.array([[1, 0, 0, 0]], np.float32), (n, 1)),
        opacities=np.full(n, 0.02, np.float32), colors=rng.uniform(0, 1, (n, 3)).astype(np.float32))
    g = render_gpu(pkg, scene, pkg.camera.look_from((0, 0, 5)), 64, 64)
    gpu, ref = assert_frame_parity(orc, g)
    t = int(np.argmax(ref["tile_counts"]))
    e = gpu["tile_entries"][ref["tile_offsets"][t]: ref["tile_offsets"][t] + ref["tile_counts"][t]]
    assert np.array_equal(np.sort(e[:4096]), e[:4096])  # ties: ascending sortRank within each chunk


def test_f32_color_output(cuda, pkg, orc):
    wl = pkg.workloads.plain50k()
    g16 = render_gpu(pkg, wl.scene, wl.cameras[0], 400, 300)
    g32 = render_gpu(pkg, wl.scene, wl.cameras[0], 400, 300, f32_color=True)
    c16 = g16["color"].cpu().numpy()
    c32 = g32["color"].cpu().numpy()
    assert np.array_equal(c32.astype(np.float16).view(np.uint16), c16.view(np.uint16))


def test_composite_only_and_determinism(cuda, pkg, orc):
    import torch

    wl = pkg.workloads.plain50k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height)
    first = read_gpu(g)
    g["color"].zero_()
    pkg.encode_composite_only(None, g["res"])
    torch.cuda.synchronize()
    again = read_gpu(g)
    assert np.array_equal(again["color"].view(np.uint16), first["color"].view(np.uint16))
    for _ in range(3):
        pkg.encode_full_compute_compositor_pipeline(None, g["res"])
    torch.cuda.synchronize()
    third = read_gpu(g)
    for k in ("tile_entries", "sorted_keys", "material", "normal"):
        assert np.array_equal(third[k], first[k]), k


def test_frame_graph_replays_match_direct_frames(cuda, pkg, orc):
    # On a stream other than the legacy default one, the second full frame
    # after a bind is captured into a CUDA graph that later frames replay;
    # a rebind drops the graph (the next frames write the new outputs).
    import torch

    wl = pkg.workloads.plain50k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height)  # legacy stream: direct
    res = g["res"]
    first = read_gpu(g)
    per_frame = res.launch_count()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):
            g["color"].zero_()
            pkg.encode_full_compute_compositor_pipeline(s, res)
    s.synchronize()
    assert res.launch_count() == 4 * per_frame
    again = read_gpu(g)
    assert np.array_equal(again["color"].view(np.uint16), first["color"].view(np.uint16))
    for k in ("out_depth", "normal", "material", "tile_entries"):
        assert np.array_equal(again[k], first[k]), k
    color2, gb2 = pkg.create_output_textures(g["plan"])
    pkg.create_tile_splat_bind_groups(res, g["bufs"], color2, gb2)
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):
            pkg.encode_full_compute_compositor_pipeline(s, res)
    s.synchronize()
    assert torch.equal(color2.view(torch.int16), g["color"].view(torch.int16))
    assert torch.equal(gb2["material"], g["gb"]["material"])
    res.destroy()


def test_frame_inside_a_callers_graph_capture(cuda, pkg, orc):
    # a caller that captures hdsr_encode_full into its own CUDA graph gets the
    # kernels in its graph (the handle does not start a capture of its own
    # on a stream that is capturing); replays render the same image
    import torch

    wl = pkg.workloads.plain50k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height)  # one direct frame first
    res = g["res"]
    first = read_gpu(g)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            pkg.encode_full_compute_compositor_pipeline(s, res)
    torch.cuda.synchronize()
    g["color"].zero_()
    graph.replay()
    torch.cuda.synchronize()
    again = read_gpu(g)
    assert np.array_equal(again["color"].view(np.uint16), first["color"].view(np.uint16))
    assert np.array_equal(again["material"], first["material"])
    del graph
    res.destroy()


def test_tile_entries_on_demand(cuda, pkg, orc):
    # The rasteriser reads the superblock lists, so without
    # HDSR_CFG_TILE_ENTRIES / KEEP_SORTED_KEYS a frame writes no per-tile
    # lists: the readback builds them once (3 launches), bit-exact, and the
    # image equals that of a handle that writes them every frame.
    wl = pkg.workloads.plain50k()
    lazy = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height, keep_keys=False)
    eager = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height, keep_keys=False, tile_entries=True)
    n0 = lazy["res"].launch_count()
    gpu = read_gpu(lazy)
    assert lazy["res"].launch_count() == n0 + 3
    assert_frame_parity(orc, lazy, gpu=gpu)
    again = read_gpu(lazy)
    assert lazy["res"].launch_count() == n0 + 3
    assert np.array_equal(again["tile_entries"], gpu["tile_entries"])
    n1 = eager["res"].launch_count()
    ref = read_gpu(eager)
    assert eager["res"].launch_count() == n1
    for k in ("tile_entries", "normal", "material"):
        assert np.array_equal(ref[k], gpu[k]), k
    assert np.array_equal(ref["color"].view(np.uint16), gpu["color"].view(np.uint16))
    lazy["res"].destroy()
    eager["res"].destroy()


@pytest.mark.parametrize("f32_color", [False, True])
def test_f16_composite_variant_parity(cuda, pkg, orc, f32_color):
    # createTileSplatCompositor {f16: true} (gpu_tile_splat_composite_f16.wgsl):
    # f16 transmittance and colour, bit-exact against the oracle's f16 variant
    wl = pkg.workloads.plain50k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height, f16=True, f32_color=f32_color)
    gpu, ref = assert_frame_parity(orc, g)
    f32 = orc.render_frame(g["u"], g["packed"], g["order"])
    a = orc.f16_to_f32(f32["color"].reshape(-1))
    b = orc.f16_to_f32(ref["color"].reshape(-1))
    # the variant's own error against the f32 composite (f16 transmittance
    # has 11 significant bits): measured 0.0054 at most on this frame
    d = np.abs(a - b)
    assert d.max() > 0 and float(d.max()) <= 2.0 / 255.0 and float(d.mean()) < 1e-3
    g["res"].destroy()


def test_f16_composite_hot_tiles_and_no_adjoint(cuda, pkg, orc):
    import torch

    scene = _hot_scene(pkg)
    g = render_gpu(pkg, scene, pkg.camera.look_from((0, 0, 5)), 128, 96, f16=True)
    assert_frame_parity(orc, g)
    res = pkg.create_tile_splat_compositor(g["plan"], backward=True, f16=True)
    pkg.create_tile_splat_bind_groups(res, g["bufs"], g["color"], g["gb"])
    pkg.write_frame_uniform_buffer(res, g["u"])
    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    n = g["plan"].splat_count
    grads = {k: torch.zeros(n * w, device="cuda") for k, w in (("positions", 3), ("log_scales", 3), ("rotations", 4),
                                                              ("opacities", 1), ("sh", 6))}
    d_color = torch.zeros((g["plan"].viewport_height, g["plan"].viewport_width, 4), device="cuda")
    with pytest.raises(pkg._lib.HdsrError):
        pkg.encode_backward(None, res, d_color, grads)
    res.destroy()
    g["res"].destroy()


def test_overflow_is_reported_not_faulted(cuda, pkg, orc):
    import torch

    wl = pkg.workloads.plain50k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height, pair_capacity=1000)
    st = g["res"].query_status()
    assert st["status"] == pkg._lib.HDSR_ERR_OVERFLOW
    assert st["total_pairs"] > 1000 and st["device_flags"] & pkg._lib.DEV_OVERFLOW
    with pytest.raises(pkg._lib.HdsrError):
        pkg.encode_composite_only(None, g["res"])
    # an overflowed frame skips the depth sort, so nothing may read the
    # depth order: with it full of out-of-range values the frame still only
    # reports the overflow
    g["res"].buffer("depth_order").fill_(-1)
    torch.cuda.synchronize()
    pkg.encode_full_compute_compositor_pipeline(None, g["res"])
    st = g["res"].query_status()
    assert st["status"] == pkg._lib.HDSR_ERR_OVERFLOW and st["total_pairs"] > 1000


def test_bad_sorted_index_is_flagged(cuda, pkg, orc):
    scene = pkg.workloads.plain_scene(2000, seed=9)
    order = np.arange(2000, dtype=np.uint32)
    order[5] = 999999
    g = render_gpu(pkg, scene, pkg.camera.look_from((0, 0, 5)), 64, 64, order=order)
    st = g["res"].query_status()
    assert st["device_flags"] & pkg._lib.DEV_BAD_INDEX
    assert_frame_parity(orc, g)


def test_repeated_sorted_index_projects_each_position(cuda, pkg, orc):
    # sortedIndices that is not a permutation (a repeated id, another never
    # named): every position projects the id it names, as the reference does
    # (the repeated splat is drawn twice), and the frame is the oracle's;
    # then the same handle with the permutation again matches too
    import torch

    scene = pkg.workloads.plain_scene(3000, seed=11)
    cam = pkg.camera.look_from((0.2, 0.1, 5.0))
    packed = pkg.splats.pack_splat_attributes(scene)
    plan = pkg.plan_tile_splat_compositor(96, 80, 16, 3000)
    _, fr = pkg.frame_uniforms_for(plan, cam)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"]).copy()
    repeated = order.copy()
    repeated[17] = repeated[1234]
    g = render_gpu(pkg, scene, cam, 96, 80, order=repeated)
    st = g["res"].query_status()
    assert not st["device_flags"] & pkg._lib.DEV_BAD_INDEX
    assert_frame_parity(orc, g)
    g["bufs"]["sorted_indices"].copy_(torch.from_numpy(order.view(np.int32)))
    g["order"] = order
    pkg.encode_full_compute_compositor_pipeline(None, g["res"])
    torch.cuda.synchronize()
    assert_frame_parity(orc, g)
    g["res"].destroy()


def test_bind_validation(cuda, pkg):
    wl = pkg.workloads.plain50k()
    plan = pkg.plan_tile_splat_compositor(64, 64, 16, 10)
    res = pkg.create_tile_splat_compositor(plan)
    with pytest.raises(pkg._lib.HdsrError):
        pkg.encode_full_compute_compositor_pipeline(None, res)  # nothing bound
    bad_plan = pkg.plan_tile_splat_compositor(64, 64, 16, 11)
    u, _ = pkg.frame_uniforms_for(bad_plan, wl.cameras[0])
    with pytest.raises(pkg._lib.HdsrError):
        pkg.write_frame_uniform_buffer(res, u)
    res.destroy()
    with pytest.raises(pkg._lib.HdsrError):
        pkg.create_tile_splat_compositor(pkg.plan_tile_splat_compositor(64, 64, 8, 10))


def test_hot760k_full_frame_parity(cuda, pkg, orc):
    """The 760k-splat 1920x1080 hot-tile workload, full size: every stage
    against the oracle (about 40M pairs, thousands of hot tiles)."""
    wl = pkg.workloads.hot760k()
    g = render_gpu(pkg, wl.scene, wl.cameras[0], wl.width, wl.height, pair_capacity=48_000_000)
    gpu, ref = assert_frame_parity(orc, g, check_keys=False)
    assert ref["hot_tiles"] >= 20
    # every (Morton tile, 20-bit log-depth key, sortRank) of the ~40M pairs,
    # bit for bit against the oracle's key list. The oracle orders a tile's
    # keys by (k20, sortRank); the GPU list is in the frame's (depth bits,
    # sortRank) order, whose k20 is non-decreasing (the log is monotone), so
    # the GPU list sorted as u64 words must equal the oracle's words.
    gk = gpu["sorted_keys"]
    R = np.uint64(gpu["rank_bits"])
    assert np.array_equal((gk & ((np.uint64(1) << R) - np.uint64(1))).astype(np.uint32), ref["tile_entries"])
    assert np.all((gk >> R)[1:] >= (gk >> R)[:-1])
    keys, vals = orc.sorted_keys20(g["u"], ref["proj_cache"], ref["depth"])
    assert len(keys) == len(gk) == ref["total_pairs"]
    want = (keys << R) | vals.astype(np.uint64)
    del keys, vals
    assert np.all(want[1:] > want[:-1])
    got = np.sort(gk)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, f"{bad.size} of {len(want)} keys differ, first at {bad[:5].tolist()}"
    del got, want
    err, psnr = _fp64_error(orc, g, gpu, ref)
    assert psnr >= 50.0, (err, psnr)
    g["res"].destroy()


def test_sh3_3m_4k_orbit_parity_and_fp64_error_per_view(cuda, pkg, orc):
    """3M Gaussians, SH degree 3 (48 coefficients), 3840x2160, 8-camera orbit
    at radius 6. View 0: every stage against the oracle, bit for bit (about
    500M pairs). Every view: the image against the FP64 twin over the frame's
    own entry lists (max |err| and PSNR per view; threshold PSNR >= 50 dB)."""
    import torch

    wl = pkg.workloads.sh3_3m()
    packed = pkg.splats.pack_splat_attributes(wl.scene)
    plan = pkg.plan_tile_splat_compositor(wl.width, wl.height, 16, wl.scene.count)
    res = pkg.create_tile_splat_compositor(plan, pair_capacity=640_000_000)
    color, gb = pkg.create_output_textures(plan)
    errors = []
    for i, cam in enumerate(wl.cameras):
        u, fr = pkg.frame_uniforms_for(plan, cam, sh_degree=3)
        order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
        bufs = pkg.splats.upload_splat_attribute_buffers(packed, order)
        pkg.create_tile_splat_bind_groups(res, bufs, color, gb)
        pkg.write_frame_uniform_buffer(res, u)
        pkg.encode_full_compute_compositor_pipeline(None, res)
        torch.cuda.synchronize()
        g = dict(res=res, plan=plan, u=u, packed=packed, order=order, color=color, gb=gb, bufs=bufs)
        gpu = read_gpu(g)
        assert gpu["status"]["status"] == 0, gpu["status"]
        if i == 0:
            gpu, ref = assert_frame_parity(orc, g, gpu=gpu)
            assert ref["hot_tiles"] > 0
            del ref
        frame = dict(tile_counts=gpu["tile_counts"], tile_offsets=gpu["tile_offsets"],
                     tile_entries=gpu["tile_entries"])
        f64 = orc.render_frame_f64(u, packed, order, frame)
        got = gpu["color"].astype(np.float64)
        err = float(np.abs(got - f64).max())
        mse = float(np.mean((got[..., :3] - f64[..., :3]) ** 2))
        psnr = 10.0 * math.log10(1.0 / max(mse, 1e-30))
        errors.append((i, gpu["P"], err, psnr))
        del gpu, f64, got, bufs
    print("sh3_3m per view (view, pairs, max |err| vs FP64, PSNR dB):", errors)
    for i, P, err, psnr in errors:
        assert P > 100_000_000, (i, P)
        assert psnr >= 50.0, (i, err, psnr)
    res.destroy()


@pytest.mark.parametrize("f16", [False, True])
def test_non_finite_vote_attributes_poison_the_votes_as_in_the_reference(cuda, pkg, orc, f16):
    # The rasteriser drops entries that reach no pixel of a half tile with
    # alpha > 1/255 and skips a lane's G-buffer votes when none of its pixels
    # has a weight above 0.01; both leave the sums as they are only for
    # finite attributes: a NaN or infinite roughness, metalness, normal or
    # emission makes even a zero-weight vote NaN (the reference's select of
    # weight 0 still multiplies, at every pixel of a quad it visits), so such
    # splats are culled by power alone and always vote. Bit-exact against the
    # oracle, which follows the reference.
    rng = np.random.default_rng(41)
    n = 4000
    scene = pkg.workloads.plain_scene(n, seed=41)
    scene.normals = rng.normal(0, 1, (n, 3)).astype(np.float32)
    scene.normals[2::13] = np.inf
    scene.normals[5::17, 1] = np.nan
    scene.roughness = rng.uniform(0, 1, n).astype(np.float32)
    scene.roughness[::29] = np.nan
    scene.metalness = rng.uniform(0, 1, n).astype(np.float32)
    scene.metalness[1::31] = np.inf
    scene.emissive = np.where(rng.uniform(0, 1, (n, 1)) < 0.3, rng.uniform(0, 2, (n, 3)), 0.0).astype(np.float32)
    scene.emissive[7::37, 2] = np.nan
    g = render_gpu(pkg, scene, pkg.camera.OrbitCamera(azimuth=0.3, elevation=0.2, distance=4.5), 160, 128, f16=f16)
    gpu, ref = assert_frame_parity(orc, g)
    # the case is live: some pixels' material or normal sums are NaN
    # (0x7E00 halves), and most are not
    halves = np.concatenate([gpu["material"].reshape(-1) & 0xFFFF, gpu["material"].reshape(-1) >> 16,
                             gpu["normal"].reshape(-1) & 0xFFFF, gpu["normal"].reshape(-1) >> 16])
    nan = (halves & 0x7FFF) > 0x7C00
    assert 0 < nan.sum() < 0.5 * nan.size
