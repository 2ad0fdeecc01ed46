"""hdsr_sort_back_to_front: sortedIndices on the device, bit-identical to the
reference's back-to-front order (gpuSortPrototype.ts:120-163) as the host
computes it (splats.back_to_front_order)."""
import numpy as np
import pytest

from gpu_helpers import assert_frame_parity, u32

pytestmark = pytest.mark.gpu


def _handle(pkg, scene, W=320, H=240):
    import torch

    packed = pkg.splats.pack_splat_attributes(scene)
    plan = pkg.plan_tile_splat_compositor(W, H, 16, scene.count)
    res = pkg.create_tile_splat_compositor(plan)
    bufs = pkg.splats.upload_splat_attribute_buffers(packed, np.arange(scene.count, dtype=np.uint32))
    color, gb = pkg.create_output_textures(plan)
    pkg.create_tile_splat_bind_groups(res, bufs, color, gb)
    return packed, plan, res, bufs, color, gb


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_device_order_equals_host_order(cuda, pkg, seed):
    import torch

    rng = np.random.default_rng(seed)
    scene = pkg.workloads.plain_scene(50_000, seed)
    # ties: duplicated positions; zero view depth: points on the camera plane
    scene.positions[:2000] = scene.positions[2000:4000]
    cam = pkg.camera.OrbitCamera(azimuth=float(rng.uniform(0, 6.28)), elevation=float(rng.uniform(-0.5, 0.5)),
                                 distance=4.0)
    fr = cam.frame(320, 240)
    view = np.asarray(fr["view"], np.float32).reshape(-1)
    packed, plan, res, bufs, color, gb = _handle(pkg, scene)
    out = torch.empty(scene.count, dtype=torch.int32, device="cuda")
    pkg.sort_back_to_front(None, res, view, out)
    torch.cuda.synchronize()
    want = pkg.splats.back_to_front_order(packed.positions, view)
    assert np.array_equal(u32(out), want)
    res.destroy()


@pytest.mark.parametrize("case", ["inside", "flat", "nan"])
def test_device_order_over_every_depth_range(cuda, pkg, case):
    # Depths of both signs (camera inside the cloud), a nearly flat cloud
    # (keys a few ulps apart, many ties), and non-finite positions (keys that
    # sort last, by id).
    import torch

    scene = pkg.workloads.plain_scene(40_000, 7)
    if case == "inside":
        cam = pkg.camera.OrbitCamera(azimuth=0.7, elevation=0.1, distance=0.05)
    else:
        cam = pkg.camera.OrbitCamera(azimuth=0.0, elevation=0.0, distance=4.0)
    fr = cam.frame(320, 240)
    view = np.asarray(fr["view"], np.float32).reshape(-1)
    if case == "flat":
        # every point on one plane facing the camera, a hair apart in depth
        v = view.astype(np.float64)
        fwd = np.array([v[2], v[6], v[10]])
        p = scene.positions.astype(np.float64)
        p -= np.outer(p @ fwd, fwd) / (fwd @ fwd)
        p += np.outer(np.random.default_rng(3).uniform(0, 1e-4, len(p)), fwd)
        scene.positions[:] = p.astype(np.float32)
    if case == "nan":
        scene.positions[[5, 77, 31000]] = np.nan
    packed, plan, res, bufs, color, gb = _handle(pkg, scene)
    out = torch.empty(scene.count, dtype=torch.int32, device="cuda")
    pkg.sort_back_to_front(None, res, view, out)
    torch.cuda.synchronize()
    want = pkg.splats.back_to_front_order(packed.positions, view)
    assert np.array_equal(u32(out), want)
    if case == "nan":
        assert sorted(u32(out)[-3:].tolist()) == [5, 77, 31000]
    res.destroy()


def test_device_sorted_frame_matches_the_host_sorted_frame(cuda, pkg, orc):
    import torch

    wl = pkg.workloads.plain50k()
    packed, plan, res, bufs, color, gb = _handle(pkg, wl.scene, wl.width, wl.height)
    u, fr = pkg.frame_uniforms_for(plan, wl.cameras[0])
    # sort straight into the bound sortedIndices buffer, then render
    pkg.sort_back_to_front(None, res, fr["view"], bufs["sorted_indices"])
    pkg.write_frame_uniform_buffer(res, u)
    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    assert np.array_equal(u32(bufs["sorted_indices"]), order)
    g = dict(res=res, plan=plan, u=u, packed=packed, order=order, color=color, gb=gb, bufs=bufs)
    assert_frame_parity(orc, g)
    res.destroy()
