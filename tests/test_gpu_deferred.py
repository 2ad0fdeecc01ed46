"""The deferred frame tail (hdsr_post_*) against the oracle, pass by pass.

A compositor frame with per-splat normals, materials and emissive colour is
rendered through the C ABI; its G-buffer feeds the deferred passes. Every
intermediate image is read back and compared bit for bit with the oracle's
restatement of the same pass, fed with the GPU's own input for that pass (so a
difference points at one pass), and the whole oracle chain is run once more
from the G-buffer alone to check that the stages compose. The lit image is
also held to the image tolerance, max |err| <= 1/255 per channel.
"""
import numpy as np
import pytest

from gpu_helpers import render_gpu

pytestmark = pytest.mark.gpu


def _scene(pkg, n=20000, seed=7):
    rng = np.random.default_rng(seed)
    scene = pkg.workloads.plain_scene(n, seed=seed)
    scene.normals = rng.normal(0, 1, (n, 3)).astype(np.float32)
    scene.roughness = rng.uniform(0, 1, n).astype(np.float32)
    scene.metalness = rng.uniform(0, 1, n).astype(np.float32)
    em = np.zeros((n, 3), np.float32)
    hot = rng.uniform(0, 1, n) < 0.05
    em[hot] = rng.uniform(0.5, 3.0, (int(hot.sum()), 3)).astype(np.float32)
    scene.emissive = em
    return scene


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


def _u16(t):
    return t.cpu().numpy().view(np.uint16)


def _run(cuda, pkg, W, H, env=None, recovery=0, light_mode="camera", frame_counter=0, curves=None, **overrides):
    D = pkg.deferred
    cam = pkg.camera.OrbitCamera(azimuth=0.4, elevation=0.25, distance=4.0)
    g = render_gpu(pkg, _scene(pkg), cam, W, H)
    post = D.DeferredPasses(W, H)
    if env is not None:
        post.set_environment(env)
    if curves is not None:
        post.set_material_curves(*curves)
    q = D.frame_params(cam, W, H, light_mode=light_mode, normal_recovery_mode=recovery,
                       frame_counter=frame_counter, **overrides)
    lit = cuda.zeros((H, W, 4), dtype=cuda.float16, device="cuda")
    post.encode(None, g["color"], g["gb"], q, lit)
    cuda.cuda.synchronize()
    return g, post, q, lit


def _check_chain(orc, g, post, q, lit, W, H):
    color = g["color"].float().cpu().numpy()
    depth = g["gb"]["depth"].cpu().numpy()
    normal = g["gb"]["normal"].cpu().numpy()
    material = g["gb"]["material"].cpu().numpy()
    inp, keep = orc.post_inputs(color, depth, normal, material)
    hw, hh = (W + 1) // 2, (H + 1) // 2
    got = {
        "ssn": _u32(post.buffer("screen_normals")).reshape(H, W),
        "nrm": _u32(post.buffer("normals")).reshape(H, W),
        "mip0": post.buffer("depth_mip0").cpu().numpy().reshape(H, W),
        "mip1": post.buffer("depth_mip1").cpu().numpy().reshape((H + 1) // 2, (W + 1) // 2),
        "mip2": post.buffer("depth_mip2").cpu().numpy().reshape((H + 3) // 4, (W + 3) // 4),
        "ao_raw": _u16(post.buffer("ao_raw")).reshape(H, W, 4),
        "ao": _u16(post.buffer("ao")).reshape(H, W, 4),
        "bloom_h": _u16(post.buffer("bloom_h")).reshape(hh, hw, 4),
        "bloom": _u16(post.buffer("bloom")).reshape(hh, hw, 4),
        "brdf": _u32(post.buffer("brdf_lut")).reshape(256, 256),
        "env": _u16(post.buffer("env")).reshape(-1, 4),
        "curves": _u16(post.buffer("curves"))[: 3 * 256].reshape(3, 256),
        "lit": lit.cpu().numpy().view(np.uint16),
    }
    # pass by pass, each fed with the GPU's own input
    assert np.array_equal(got["ssn"], orc.post_ss_normals(inp, q))
    assert np.array_equal(got["nrm"], orc.post_bilateral(inp, q, got["ssn"]))
    m0, m1, m2 = orc.post_gtao_prefilter(inp, q)
    assert np.array_equal(got["mip0"].view(np.uint32), m0.view(np.uint32))
    assert np.array_equal(got["mip1"].view(np.uint32), m1.view(np.uint32))
    assert np.array_equal(got["mip2"].view(np.uint32), m2.view(np.uint32))
    assert np.array_equal(got["ao_raw"], orc.post_gtao_main(inp, q, (got["mip0"], got["mip1"], got["mip2"]), got["nrm"]))
    assert np.array_equal(got["ao"], orc.post_gtao_denoise(inp, q, got["ao_raw"], got["mip0"]))
    bt = orc.post_bloom_threshold(inp, q)
    tx, ty = float(np.float32(1.0 / hw)), float(np.float32(1.0 / hh))
    bh = orc.post_bloom_blur(bt, tx, 0.0, tx, ty)
    assert np.array_equal(got["bloom_h"], bh)
    assert np.array_equal(got["bloom"], orc.post_bloom_blur(bh, 0.0, ty, tx, ty))
    for r in list(range(0, 256, 17)) + [255]:  # a sample of the LUT's rows (1024 samples per texel)
        assert np.array_equal(got["brdf"][r], orc.post_brdf_lut(r, r + 1)[r]), r
    ew, eh = post.env_size
    env = orc.post_env_chain(got["env"][: ew * eh].reshape(eh, ew, 4)) if ew > 1 else orc.placeholder_env()
    assert np.array_equal(got["env"], env["texels"])
    brdf_full = got["brdf"]  # the lighting pass reads the GPU's LUT
    ref_lit = orc.post_lighting(inp, q, got["nrm"], got["ao"], env, brdf_full, got["bloom"], got["curves"])
    assert np.array_equal(got["lit"].reshape(H, W, 4), ref_lit)
    # the oracle chain from the G-buffer alone composes to the same image
    ssn = orc.post_ss_normals(inp, q)
    nrm = orc.post_bilateral(inp, q, ssn)
    ao = orc.post_gtao_denoise(inp, q, orc.post_gtao_main(inp, q, (m0, m1, m2), nrm), m0)
    bloom = orc.post_bloom_blur(orc.post_bloom_blur(bt, tx, 0.0, tx, ty), 0.0, ty, tx, ty)
    chain = orc.post_lighting(inp, q, nrm, ao, env, brdf_full, bloom, got["curves"])
    f_gpu = orc.f16_to_f32(got["lit"].reshape(-1)).reshape(H, W, 4)
    f_ref = orc.f16_to_f32(chain.reshape(-1)).reshape(H, W, 4)
    assert np.array_equal(got["lit"].reshape(H, W, 4), chain)
    finite = np.isfinite(f_ref)
    assert np.array_equal(finite, np.isfinite(f_gpu))
    assert float(np.abs(f_gpu[finite] - f_ref[finite]).max()) <= 1.0 / 255.0
    return got


@pytest.mark.parametrize("W,H,recovery", [(320, 240, 0), (203, 117, 1), (160, 96, 2)])
def test_deferred_chain_without_environment(cuda, pkg, orc, W, H, recovery):
    g, post, q, lit = _run(cuda, pkg, W, H, recovery=recovery)
    got = _check_chain(orc, g, post, q, lit, W, H)
    # identity curves: the LUT is i/255 truncated to f16
    assert np.array_equal(got["curves"][0], orc.post_curve_lut(1.0, 0.0, 1.0))
    # the frame is not trivial: lit pixels, occlusion below 1 somewhere, bloom from the emissive splats
    ao = orc.f16_to_f32(got["ao"][..., 0].reshape(-1))
    assert (ao < 0.99).mean() > 0.01
    assert orc.f16_to_f32(got["bloom"][..., :3].reshape(-1)).max() > 0.0
    post.destroy()
    g["res"].destroy()


def test_deferred_chain_with_environment_and_curves(cuda, pkg, orc):
    W, H = 256, 192
    env = pkg.deferred.synthetic_environment(256, 128, seed=3)
    g, post, q, lit = _run(cuda, pkg, W, H, env=env, light_mode="fixed", frame_counter=5,
                           curves=((1.3, -0.05, 0.8), (0.7, 0.1, 1.6), (1.1, 0.02, 1.2)), env_rotation=0.7,
                           exposure=1.4, specular_only=0)
    assert post.env_size == (256, 128)
    got = _check_chain(orc, g, post, q, lit, W, H)
    for i, c in enumerate(((1.3, -0.05, 0.8), (0.7, 0.1, 1.6), (1.1, 0.02, 1.2))):
        assert np.array_equal(got["curves"][i], orc.post_curve_lut(*[float(np.float32(v)) for v in c]))
    # the environment's level 0 is the host upload, bit for bit
    h16 = pkg.deferred.f32_to_f16_ibl(env.reshape(-1)).reshape(-1, 4)
    assert np.array_equal(got["env"][: 256 * 128], h16)
    post.destroy()
    g["res"].destroy()


def test_specular_only_and_streams(cuda, pkg, orc):
    """specularOnly, and the forked (bloom on the side stream) encode equals the profiled one."""
    W, H = 192, 160
    g, post, q, lit = _run(cuda, pkg, W, H, specular_only=1, light_mode="overhead")
    _check_chain(orc, g, post, q, lit, W, H)
    first = lit.clone()
    post.set_profiling(True)
    post.encode(None, g["color"], g["gb"], q, lit)
    cuda.cuda.synchronize()
    assert cuda.equal(first, lit)
    times = post.pass_times()
    assert [n for n, _ in times] == list(pkg._lib.POST_PASSES) and all(ms > 0 for _, ms in times)
    post.destroy()
    g["res"].destroy()


def test_post_argument_errors(cuda, pkg):
    D = pkg.deferred
    post = D.DeferredPasses(64, 32)
    q = D.default_params()
    color = cuda.zeros((32, 64, 4), dtype=cuda.float16, device="cuda")
    gb = {"depth": cuda.ones((32, 64), device="cuda"), "normal": cuda.zeros((32, 64), dtype=cuda.int32, device="cuda"),
          "material": cuda.zeros((32, 64, 4), dtype=cuda.int32, device="cuda")}
    lit = cuda.zeros((32, 64, 4), dtype=cuda.float16, device="cuda")
    q.bilateral_radius = 9
    with pytest.raises(pkg._lib.HdsrError, match="bilateral_radius"):
        post.encode(None, color, gb, q, lit)
    q.bilateral_radius = 3
    q.ao_slices = 0
    with pytest.raises(pkg._lib.HdsrError, match="slices"):
        post.encode(None, color, gb, q, lit)
    q.ao_slices = 3
    small = {"depth": cuda.ones((32, 32), device="cuda"), "normal": gb["normal"], "material": gb["material"]}
    with pytest.raises(pkg._lib.HdsrError, match="pitch"):
        post.encode(None, color, small, q, lit)
    post.encode(None, color, gb, q, lit)  # a background-only frame is valid
    cuda.cuda.synchronize()
    assert bool((lit[..., 3] == 0).all())
    post.destroy()
