"""Serving loop (hdsr_server_*): every request of a mixed stream renders
exactly what the same request renders alone through the plain C ABI path
(bit-exact images: the frame is deterministic and slots share nothing)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VIEWPORTS = [(256, 256), (320, 180), (480, 270)]


def _scenes(pkg):
    out = {}
    specs = {0: pkg.workloads.plain_scene(20_000, 1), 1: pkg.workloads.hot_scene(40_000, 3),
             2: pkg.workloads.hot_scene(30_000, 4, sh_degree=1)}
    for sid, sc in specs.items():
        packed = pkg.splats.pack_splat_attributes(sc)
        bufs = pkg.splats.upload_splat_attribute_buffers(packed, np.arange(sc.count, dtype=np.uint32))
        out[sid] = (sc, bufs)
    return out


def _camera(pkg, rng):
    return pkg.camera.OrbitCamera(azimuth=float(rng.uniform(0, 6.283)), elevation=float(rng.uniform(-0.5, 0.5)),
                                  distance=float(rng.uniform(3.0, 7.0)))


def _alone(pkg, bufs, sc, u, W, H, f32, pairs):
    plan = pkg.plan_tile_splat_compositor(W, H, 16, sc.count)
    res = pkg.create_tile_splat_compositor(plan, pair_capacity=int(pairs * 1.1) + 4096, f32_color=f32)
    color, gb = pkg.create_output_textures(plan, f32_color=f32)
    pkg.create_tile_splat_bind_groups(res, bufs, color, gb)
    pkg.write_frame_uniform_buffer(res, u)
    pkg.encode_full_compute_compositor_pipeline(None, res)
    st = res.check_frame()
    res.destroy()
    return color, gb, st


def _same(a, b):
    import torch

    return torch.equal(a.view(torch.int32) if a.dtype == torch.float32 else a.view(torch.int16),
                       b.view(torch.int32) if b.dtype == torch.float32 else b.view(torch.int16))


def _check_equal(pkg, scenes, jobs, results):
    for (sid, W, H, f32, u, color, gb), r in zip(jobs, results):
        assert r["status"] == 0 and r["wait_status"] == 0, r
        sc, bufs = scenes[sid]
        c2, g2, st = _alone(pkg, bufs, sc, u, W, H, f32, r["total_pairs"])
        assert st["total_pairs"] == r["total_pairs"]
        assert _same(color, c2)
        for k in ("depth", "normal", "material"):
            assert _same(gb[k], g2[k]), k


def _submit_mix(pkg, server, scenes, rng, n):
    jobs = []
    for _ in range(n):
        sid = int(rng.integers(0, len(scenes)))
        W, H = VIEWPORTS[int(rng.integers(0, len(VIEWPORTS)))]
        f32 = bool(rng.integers(0, 2))
        sc, _ = scenes[sid]
        plan = pkg.plan_tile_splat_compositor(W, H, 16, sc.count)
        u, _ = pkg.frame_uniforms_for(plan, _camera(pkg, rng), sh_degree=sc.sh_degree)
        color, gb = pkg.create_output_textures(plan, f32_color=f32)
        t = server.submit(sid, u, color, gb)
        jobs.append((sid, W, H, f32, u, color, gb, t))
    results = [server.wait(j[-1]) for j in jobs]
    return [j[:-1] for j in jobs], results


def test_mixed_stream_matches_each_request_alone(cuda, pkg):
    scenes = _scenes(pkg)
    server = pkg.serving.Server(hbm_budget_bytes=8 << 30, max_in_flight=6)
    for sid, (_, bufs) in scenes.items():
        server.add_scene(sid, bufs)
    rng = np.random.default_rng(11)
    jobs, results = _submit_mix(pkg, server, scenes, rng, 36)
    _check_equal(pkg, scenes, jobs, results)
    # a second wave reuses the slots: graphs replace the direct launches
    jobs2, results2 = _submit_mix(pkg, server, scenes, rng, 24)
    _check_equal(pkg, scenes, jobs2, results2)
    st = server.stats()
    assert st["completed"] == 60 and st["graphs"] >= 1 and st["slots"] >= 3
    assert all(r["done_ms"] >= r["start_ms"] >= r["submit_ms"] for r in results + results2)
    server.destroy()


def test_tight_budget_evicts_and_stays_exact(cuda, pkg):
    scenes = _scenes(pkg)
    scene_bytes = 0
    probe = pkg.serving.Server(hbm_budget_bytes=8 << 30, max_in_flight=1)
    for sid, (_, bufs) in scenes.items():
        probe.add_scene(sid, bufs)
    scene_bytes = probe.stats()["scene_bytes"]
    rng = np.random.default_rng(5)
    jobs, results = _submit_mix(pkg, probe, scenes, rng, 3)
    slot_bytes = probe.stats()["slot_bytes"] / max(1, probe.stats()["slots"])
    probe.destroy()
    # room for the scenes and about two slots: the mix must evict
    server = pkg.serving.Server(hbm_budget_bytes=int(scene_bytes + 2.2 * slot_bytes), max_in_flight=2)
    for sid, (_, bufs) in scenes.items():
        server.add_scene(sid, bufs)
    jobs, results = _submit_mix(pkg, server, scenes, rng, 18)
    _check_equal(pkg, scenes, jobs, results)
    st = server.stats()
    assert st["evictions"] > 0
    assert st["scene_bytes"] + st["slot_bytes"] <= st["budget_bytes"]
    server.destroy()


def test_overflowing_frame_is_rerun_on_a_larger_slot(cuda, pkg):
    # large splats: about 42 pairs per splat, beyond the default 16 per splat
    rng = np.random.default_rng(12)
    n = 3000
    sc = pkg.splats.SplatAttributes(
        positions=rng.uniform(-1, 1, (n, 3)).astype(np.float32), scales=np.full((n, 3), -1.6, np.float32),
        rotations=np.tile(np.array([1, 0, 0, 0], np.float32), (n, 1)), opacities=np.full(n, 0.5, np.float32),
        colors=rng.uniform(0, 1, (n, 3)).astype(np.float32))
    packed = pkg.splats.pack_splat_attributes(sc)
    bufs = pkg.splats.upload_splat_attribute_buffers(packed, np.arange(sc.count, dtype=np.uint32))
    server = pkg.serving.Server(hbm_budget_bytes=4 << 30, max_in_flight=2)
    server.add_scene(7, bufs)
    W, H = 480, 270
    plan = pkg.plan_tile_splat_compositor(W, H, 16, sc.count)
    u, _ = pkg.frame_uniforms_for(plan, pkg.camera.OrbitCamera(azimuth=0.3, elevation=0.2, distance=3.5))
    color, gb = pkg.create_output_textures(plan)
    r = server.wait(server.submit(7, u, color, gb))
    assert r["status"] == 0 and r["reruns"] == 1 and r["total_pairs"] > 16 * sc.count
    c2, g2, st = _alone(pkg, bufs, sc, u, W, H, False, r["total_pairs"])
    assert _same(color, c2) and _same(gb["depth"], g2["depth"])
    # the next request of that key fits the learned size at once
    r2 = server.wait(server.submit(7, u, color, gb))
    assert r2["status"] == 0 and r2["reruns"] == 0
    server.destroy()
