"""The oracle, pinned: the reference's own known-answer vectors, the
arithmetic it defines, and the frame-level invariants of the canonical order."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


# --- splatSort.ts known answers (tests/cpuDepthSort.test.ts) ---------------

@pytest.mark.parametrize("case", GOLDEN["cpu_depth_sort"], ids=lambda c: c["name"])
@pytest.mark.parametrize("threads", [1, 4])
def test_cpu_depth_sort_known_answers(orc, case, threads):
    order = orc.sort_back_to_front(case["positions"], case["view"], threads=threads)
    assert order.tolist() == case["order"]


@pytest.mark.parametrize("case", GOLDEN["cpu_depth_sort"], ids=lambda c: c["name"])
def test_gpu_sort_prototype_order_matches_known_answers(orc, pkg, case):
    """sortedIndices producer (gpuSortPrototype) gives the same order on the
    reference's cases, in the oracle and in the host-side numpy form."""
    assert orc.gpu_sort_prototype_order(case["positions"], case["view"]).tolist() == case["order"]
    assert pkg.splats.back_to_front_order(case["positions"], case["view"]).tolist() == case["order"]


def test_view_space_depth_known_answers():
    case = next(c for c in GOLDEN["cpu_depth_sort"] if c["name"] == "translated_view")
    p = np.array(case["positions"], np.float64).reshape(-1, 3)
    v = np.array(case["view"], np.float64)
    z = v[2] * p[:, 0] + v[6] * p[:, 1] + v[10] * p[:, 2] + v[14]
    assert z.tolist() == case["depths"]


@pytest.mark.parametrize("case", GOLDEN["cpu_depth_sort_errors"], ids=lambda c: c["message"][:20])
def test_cpu_depth_sort_rejects_malformed_input(orc, case):
    with pytest.raises(ValueError, match=case["message"]):
        orc.sort_back_to_front(case["positions"], case["view"])


def test_cpu_depth_sort_rejects_non_finite(orc):
    with pytest.raises(ValueError, match="non-finite"):
        orc.sort_back_to_front([0, 0, np.inf], np.eye(4, dtype=np.float32).reshape(-1))


def test_cpu_depth_sort_parallel_equals_serial(orc):
    rng = np.random.default_rng(3)
    pos = rng.integers(-50, 50, (20000, 3)).astype(np.float32)  # many exact ties
    view = np.eye(4, dtype=np.float32).reshape(-1)
    a = orc.sort_back_to_front(pos, view, threads=1)
    b = orc.sort_back_to_front(pos, view, threads=8)
    assert np.array_equal(a, b)
    z = pos[:, 2].astype(np.float64)
    assert np.array_equal(a, np.lexsort((np.arange(len(z)), z)))


# --- compositor constants (computeCompositorLifecycle.test.mjs) -----------

def test_plan_budget_cap(orc):
    c = GOLDEN["compositor_constants"]
    assert orc.plan(1920, 1080, 16, 2_000_000)[8] == c["max_dispatch_safe_refs"]
    assert orc.plan(1920, 1080, 16, 760_000)[8] == 760_000 * 16
    p = orc.plan(1920, 1080, 16, 1)
    assert p[3:7].tolist() == [120, 68, 8160, 13600]
    assert orc.plan(3840, 2160, 16, 1)[6] == 54398
    assert orc.plan(800, 600, 16, 1)[6] == 3364


def _one_splat_scene(pkg, pos, log_scale, opacity=0.8, color=(1.0, 0.5, 0.25)):
    scene = pkg.splats.SplatAttributes(
        positions=np.array([pos], np.float32), scales=np.array([[log_scale] * 3], np.float32),
        rotations=np.array([[1, 0, 0, 0]], np.float32), opacities=np.array([opacity], np.float32),
        colors=np.array([color], np.float32))
    return scene


def _uniforms(pkg, W, H, N, cam, sh_degree=0):
    fr = cam.frame(W, H)
    import ctypes  # noqa: F401

    plan = _plan(pkg, W, H, N)
    return pkg.write_tile_splat_frame_uniforms(None, fr["view_proj"], plan, 1.0, sh_degree, fr["camera_pos"],
                                               fr["view"], fr["proj"]), fr


def _plan(pkg, W, H, N):
    return pkg.plan_tile_splat_compositor(W, H, 16, N)


def test_footprint_clamped_to_eight_tiles(orc, pkg, hdsr_lib):
    clamp = GOLDEN["compositor_constants"]["footprint_clamp_tiles"]
    scene = _one_splat_scene(pkg, (0.0, 0.0, 0.0), 2.0)
    packed = pkg.splats.pack_splat_attributes(scene)
    u, _ = _uniforms(pkg, 1024, 1024, 1, pkg.camera.look_from((0, 0, 5)))
    fr = orc.render_frame(u, packed, np.zeros(1, np.uint32), composite=False)
    box = int(fr["proj_cache"][0, 7])
    x0, y0, x1, y1 = box & 255, (box >> 8) & 255, (box >> 16) & 255, box >> 24
    assert x1 - x0 + 1 == 2 * clamp + 1 and y1 - y0 + 1 == 2 * clamp + 1
    assert fr["proj_cache"].shape[1] == GOLDEN["compositor_constants"]["proj_stride_u32"]


def test_sh_degree1_follows_the_projection_shader_not_the_cpu_witness(orc, pkg, hdsr_lib):
    # The inputs of the reference's tests/renderer/shViewlight.test.mjs:9-33
    # (DC 0.5, degree-1 coefficients, a view from +x and from -x). Its CPU
    # witness uses the standard 3DGS signs (-C1 y, +C1 z, -C1 x) and asserts
    # red(+x) > red(-x); gpu_project_splats.wgsl:300-314, which this path
    # restates, adds +C1 (c0 y + c1 z + c2 x), so red swaps and green stays.
    C1 = 0.4886025119029199
    coeffs = np.array([[0.0, 0.0, 0.0, 0.0, 0.6, 0.0, -0.8, 0.0, -0.4]], np.float32)
    colours = {}
    for side in (1.0, -1.0):
        scene = _one_splat_scene(pkg, (0.0, 0.0, 0.0), -2.0, color=(0.5, 0.5, 0.5))
        scene.sh, scene.sh_degree = coeffs, 1
        packed = pkg.splats.pack_splat_attributes(scene)
        u, _ = _uniforms(pkg, 64, 64, 1, pkg.camera.look_from((5.0 * side, 0.0, 0.0)), sh_degree=1)
        fr = orc.render_frame(u, packed, np.zeros(1, np.uint32), composite=False)
        w = fr["proj_cache"][0]
        colours[side] = orc.f16_to_f32(np.array([w[9] & 0xFFFF, w[9] >> 16, w[10] & 0xFFFF], np.uint16))
    assert colours[1.0][0] < colours[-1.0][0]
    assert colours[1.0][1] == colours[-1.0][1]
    # the view direction is camera - centre: +x from the +x camera
    assert abs(colours[1.0][0] - (0.5 + C1 * -0.8)) < 1e-3 and abs(colours[-1.0][0] - (0.5 - C1 * -0.8)) < 1e-3


def _witness_rotate_axis(q, axis):
    """rotateAxisWxyz of the reference's src/rendererFidelityProbes/conicProjection.js:31-50."""
    n = max(math.sqrt(sum(c * c for c in q)), 1e-6)
    w, ux, uy, uz = (c / n for c in q)
    x, y, z = axis
    cx, cy, cz = uy * z - uz * y, uz * x - ux * z, ux * y - uy * x
    ix, iy, iz = cx + w * x, cy + w * y, cz + w * z
    return (x + 2 * (uy * iz - uz * iy), y + 2 * (uz * ix - ux * iz), z + 2 * (ux * iy - uy * ix))


def _witness_jacobian_covariance(pos, axes, focal):
    """referenceJacobianCovariance (conicProjection.js:75-117): J S J^T with the
    pinhole Jacobian, camera looking down +z, in double."""
    x, y, z = pos
    jx = (focal / z, 0.0, -focal * x / (z * z))
    jy = (0.0, focal / z, -focal * y / (z * z))
    S = np.zeros((3, 3))
    for a in axes:
        S += np.outer(a, a)
    J = np.array([jx, jy])
    return J @ S @ J.T


def test_projected_covariance_matches_the_reference_jacobian_witness(orc, pkg, hdsr_lib):
    # The projection's 2D covariance (before the +0.3 low-pass, recovered from
    # the cache's inverse conic) against the reference's own EWA witness
    # formula on the same splats: the camera at (0, 0, 5) looks down -z, so a
    # view-space point (x, y, -d) is the witness's (x, y, d) and axis z flips.
    rng = np.random.default_rng(11)
    n = 64
    pos = np.column_stack([rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)]).astype(np.float32)
    lsc = rng.uniform(-4.0, -2.0, (n, 3)).astype(np.float32)
    q = rng.normal(0, 1, (n, 4)).astype(np.float32)
    scene = pkg.splats.SplatAttributes(positions=pos, scales=lsc, rotations=q,
                                       opacities=np.full(n, 0.8, np.float32),
                                       colors=np.full((n, 3), 0.5, np.float32))
    packed = pkg.splats.pack_splat_attributes(scene)
    u, fr = _uniforms(pkg, 512, 512, n, pkg.camera.look_from((0.0, 0.0, 5.0)))
    focal = float(np.float32(u[48]))
    assert focal == float(np.float32(u[49]))
    f = orc.render_frame(u, packed, np.arange(n, dtype=np.uint32), composite=False)
    worst = 0.0
    for r in range(n):
        w = f["proj_cache"][r]
        if w[7] == 0xFFFFFFFF:
            continue
        icx, icy, icz = (float(np.uint32(w[k]).view(np.float32)) for k in (2, 3, 4))
        ours = np.linalg.inv(np.array([[icx, icy], [icy, icz]], np.float64)) - 0.3 * np.eye(2)
        axes = []
        for i, e in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
            a = np.array(_witness_rotate_axis(q[r].astype(np.float64), e)) * math.exp(float(lsc[r, i]))
            axes.append((a[0], a[1], -a[2]))
        ref = _witness_jacobian_covariance((float(pos[r, 0]), float(pos[r, 1]), 5.0 - float(pos[r, 2])), axes, focal)
        worst = max(worst, float(np.abs(ours - ref).max() / max(ref[0, 0], ref[1, 1])))
    assert worst < 1e-4, worst  # measured: 7.9e-7


# --- arithmetic the canonical frame is defined with ------------------------

def test_exp_accuracy(orc):
    x = np.concatenate([np.linspace(-103.0, 88.0, 200001), np.linspace(-4.0, 0.0, 100001),
                        np.random.default_rng(0).normal(-3, 2, 100000)]).astype(np.float32)
    got = orc.expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    normal = ref > 1.2e-38
    rel = np.abs(got[normal] - ref[normal]) / ref[normal]
    assert rel.max() < 3.0e-7  # within ~2.5 ulp
    assert orc.expf([np.float32(-104.0)])[0] == 0.0
    assert np.isinf(orc.expf([np.float32(89.0)])[0])
    assert orc.expf([0.0])[0] == 1.0


def test_composite_exp_accuracy(orc):
    # the two-constant exp (degree-5 fit; the deferred weights' exp) on the
    # power range a pixel uses
    x = np.concatenate([np.linspace(-4.0, 0.0, 400001), -np.random.default_rng(5).uniform(0, 4, 200000)]).astype(np.float32)
    got = orc.composite_expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(got - ref) / ulp) <= 3.0
    assert orc.composite_expf(np.float32(0.0))[0] == np.float32(1.0) + np.float32(2.0 ** -23)


def test_splat_exp_accuracy(orc):
    # the composites' exp (one reduction constant) on the power range whose
    # value is used
    x = np.concatenate([np.linspace(-4.0, 0.0, 400001), -np.random.default_rng(7).uniform(0, 4, 200000),
                        np.float32([-4.0, -3.999999, -1e-30, 0.0, 1e-7])]).astype(np.float32)
    got = orc.splat_expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(got - ref) / ulp) <= 3.0
    assert orc.splat_expf(np.float32(0.0))[0] == np.float32(1.0) + np.float32(2.0 ** -23)


def test_opacity_scaled_by_the_exponent_bits_equals_the_product(orc):
    # the rasterisers form alpha's product as (op with k added to its
    # exponent bits) * p; for every f16 opacity the projection can produce
    # (0 and (0, 0.99]) and powers in (-4, 0] that is op * splat_expf(x) bit
    # for bit, and op = 0 gives a product the validity test rejects
    x = np.concatenate([np.linspace(-4.0, 0.0, 4001)[1:], -np.random.default_rng(8).uniform(0, 4, 2000),
                        np.float32([-1e-30, 1e-7])]).astype(np.float32)
    h = np.arange(0x0001, 0x3C00, dtype=np.uint16)  # positive f16 values below 1
    op = orc.f16_to_f32(h)
    op = op[op <= np.float32(0.99)]
    p, kb = orc.splat_exp_parts(x)
    g = orc.splat_expf(x)
    for i in range(0, op.size, 1024):
        o = op[i:i + 1024, None]
        folded = (o.view(np.uint32) + kb[None, :]).view(np.float32) * p[None, :]
        assert np.array_equal(folded.view(np.uint32), (o * g[None, :]).view(np.uint32))
    zero = (np.uint32(0) + kb).view(np.float32) * p
    assert np.all((zero == 0) | (zero < 0))


def test_composite_exp_accuracy_over_the_weight_range(orc):
    # the deferred bilateral filter's weights use the same exp down to -86
    # (2^k exact for k >= -126), and 0 below
    x = np.concatenate([np.linspace(-86.0, 0.001, 400001),
                        -np.random.default_rng(6).uniform(0, 86, 200000)]).astype(np.float32)
    got = orc.composite_expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(got - ref) / ulp) <= 3.0


def test_log_accuracy(orc):
    x = np.concatenate([np.geomspace(1e-30, 1e30, 200001), np.linspace(0.5, 2.0, 100001),
                        np.array([1e-6, 1.0, 2.0, 0.5], np.float64)]).astype(np.float32)
    got = orc.logf(x).astype(np.float64)
    ref = np.log(x.astype(np.float64))
    err = np.abs(got - ref)
    tol = np.maximum(np.abs(ref), 1e-30) * 2.5e-7 + 1e-9
    assert np.all(err <= tol)
    assert orc.logf([1.0])[0] == 0.0
    assert np.isneginf(orc.logf([0.0])[0])


def test_f16_round_to_nearest_even_matches_ieee(orc):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(0, 1, 200000), rng.normal(0, 1e-5, 50000), rng.uniform(-70000, 70000, 50000),
                        [0.0, -0.0, 65504.0, 65519.0, 65520.0, 1e-8, 6.0e-8, 2.0 ** -24, 2.0 ** -25,
                         3 * 2.0 ** -26, np.inf, -np.inf]]).astype(np.float32)
    got = orc.f16_rne(x)
    with np.errstate(over="ignore"):
        ref = x.astype(np.float16).view(np.uint16)
    assert np.array_equal(got, ref)
    assert orc.f16_rne([np.nan])[0] == 0x7E00
    h = np.arange(65536, dtype=np.uint16)
    finite = (h & 0x7C00) != 0x7C00
    assert np.array_equal(orc.f16_to_f32(h)[finite], h.view(np.float16).astype(np.float32)[finite])


def test_f64_to_f16_round_to_nearest_even_matches_ieee(orc):
    # the f16 composite rounds exact double results once: check the rounding
    # on random doubles and on every f16 midpoint, exactly and a hair off it
    # (the cases a rounding through f32 first would get wrong)
    rng = np.random.default_rng(2)
    h = np.arange(0x7BFF, dtype=np.uint16)
    a = h.view(np.float16).astype(np.float64)
    b = (h + 1).view(np.float16).astype(np.float64)
    m = (a + b) / 2.0
    x = np.concatenate([m, m * (1 + 2.0 ** -40), m * (1 - 2.0 ** -40), -m, rng.normal(0, 1, 100000),
                        rng.normal(0, 1e-6, 20000), rng.uniform(-70000, 70000, 20000),
                        [0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e300, 1e-300, 2.0 ** -24, 2.0 ** -25,
                         2.0 ** -25 * (1 + 2.0 ** -30), np.inf, -np.inf]])
    got = orc.f64_to_f16(x)
    with np.errstate(over="ignore"):
        ref = x.astype(np.float16).view(np.uint16)
    assert np.array_equal(got, ref)
    assert orc.f64_to_f16([np.nan])[0] == 0x7E00


def test_f16_truncation_of_host_packer(orc, pkg):
    """f32ToF16 (splats.ts:431-442): restated in C and in numpy, same bits."""
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.normal(0, 1, 100000), rng.uniform(-1e6, 1e6, 1000),
                        [0.75, 0.0, 1.0, 6.1e-5, 6.0e-5, 65504.0, 70000.0]]).astype(np.float32)
    assert np.array_equal(orc.f16_trunc(x), pkg.splats.f32_to_f16_trunc(x))
    # truncation, not rounding: 0.75 is exact, 1/3 truncates below RNE
    assert pkg.splats.f32_to_f16_trunc([0.75])[0] == 0x3A00
    assert pkg.splats.f32_to_f16_trunc([1.0 / 3.0])[0] == 0x3555
    assert pkg.splats.pack_material_buffer(1)[0] == 0x3A00


def test_morton_interleave(orc):
    x = np.arange(256, dtype=np.uint32).repeat(256)
    y = np.tile(np.arange(256, dtype=np.uint32), 256)
    ref = np.zeros_like(x)
    for b in range(8):
        ref |= ((x >> b) & 1) << (2 * b)
        ref |= ((y >> b) & 1) << (2 * b + 1)
    assert np.array_equal(orc.morton(x, y), ref)


def test_bucket_is_top_bits_of_key20(orc):
    """The 128 log buckets of the hot-tile cascade are k20 >> 13, so sorting
    by the 20-bit key refines the bucket order."""
    rng = np.random.default_rng(5)
    for _ in range(200):
        d = rng.uniform(0.0, 1.0, 4000).astype(np.float32)
        d[rng.integers(0, 4000, 40)] = rng.uniform(-0.01, 0.0, 40).astype(np.float32)
        bits = d.view(np.uint32)
        b, k = orc.bucket_key20(bits, int(bits.min()), int(bits.max()))
        assert np.array_equal(b, k >> 13)
    b, k = orc.bucket_key20(np.full(10, 0x3F000000, np.uint32), 0x3F000000, 0x3F000000)
    assert not b.any() and not k.any()


# --- frame invariants of the canonical order -------------------------------

@pytest.fixture(scope="module")
def small_frame(orc, pkg, hdsr_lib):
    scene = pkg.workloads.plain_scene(6000, seed=4)
    packed = pkg.splats.pack_splat_attributes(scene)
    cam = pkg.camera.look_from((0.5, 0.2, 4.5))
    u, fr = _uniforms(pkg, 320, 240, scene.count, cam)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    return dict(u=u, packed=packed, order=order, frame=orc.render_frame(u, packed, order, threads=4))


def test_counts_offsets_entries_consistent(small_frame, orc):
    f = small_frame["frame"]
    assert f["tile_counts"].sum() == f["total_pairs"]
    assert np.array_equal(f["tile_offsets"], np.concatenate([[0], np.cumsum(f["tile_counts"])[:-1]]))
    depth = f["depth"]
    for t in np.nonzero(f["tile_counts"])[0]:
        e = f["tile_entries"][f["tile_offsets"][t]: f["tile_offsets"][t] + f["tile_counts"][t]]
        key = depth[e].astype(np.uint64) << np.uint64(32) | e.astype(np.uint64)
        if f["tile_counts"][t] <= 4096:
            assert np.all(key[1:] > key[:-1])


def test_keys20_order_matches_frame_tiles(small_frame, orc):
    f = small_frame["frame"]
    keys, vals = orc.sorted_keys20(small_frame["u"], f["proj_cache"], f["depth"])
    assert len(keys) == f["total_pairs"]
    assert np.all(keys[1:] >= keys[:-1])
    tiles = (keys >> np.uint64(20)).astype(np.int64)
    assert np.array_equal(np.bincount(tiles, minlength=f["M"])[: f["M"]], f["tile_counts"])
    # same multiset of entries per tile as the canonical frame
    for t in np.nonzero(f["tile_counts"])[0][:50]:
        a = np.sort(vals[tiles == t])
        b = np.sort(f["tile_entries"][f["tile_offsets"][t]: f["tile_offsets"][t] + f["tile_counts"][t]])
        assert np.array_equal(a, b)


def _rect_tiles(rc: int) -> int:
    """The device's tile mask of a superblock-local rect (rect_tiles in
    hdsr_internal.cuh), formula for formula."""
    x0, x1, y0, y1 = rc & 7, (rc >> 3) & 7, (rc >> 6) & 7, rc >> 9
    row = ((2 << x1) - (1 << x0)) & 0xFF
    hi = (1 << 64) - 1 if y1 == 7 else (1 << (8 * y1 + 8)) - 1
    lo = ~((1 << (8 * y0)) - 1) & ((1 << 64) - 1)
    return (row * 0x0101010101010101) & hi & lo & ((1 << 64) - 1)


def test_rect_tile_mask_formula():
    for rc in range(4096):
        x0, x1, y0, y1 = rc & 7, (rc >> 3) & 7, (rc >> 6) & 7, rc >> 9
        if x0 > x1 or y0 > y1:
            continue
        want = sum(1 << (y * 8 + x) for y in range(y0, y1 + 1) for x in range(x0, x1 + 1))
        assert _rect_tiles(rc) == want, rc


def _morton(x: int, y: int) -> int:
    m = 0
    for b in range(16):
        m |= ((x >> b) & 1) << (2 * b) | ((y >> b) & 1) << (2 * b + 1)
    return m


def test_superblock_walk_yields_the_tile_lists(small_frame):
    # The rasteriser reads a tile's entries from its superblock's list (8x8
    # tiles: every visible splat in ascending (depth bits, sortRank) order,
    # its tile box clipped to the superblock), keeping the entries whose rect
    # covers the tile and visiting only the 32-entry chunks whose mask holds
    # the tile. That walk must give the canonical per-tile list exactly.
    f = small_frame["frame"]
    box, depth = f["proj_cache"][:, 7], f["depth"]
    cols, rows = (f["W"] + 15) // 16, (f["H"] + 15) // 16
    sb_cols, sb_rows = (cols + 7) // 8, (rows + 7) // 8
    vis = np.nonzero(box != 0xFFFFFFFF)[0]
    order = vis[np.lexsort((vis, depth[vis]))]
    lists = [[] for _ in range(sb_cols * sb_rows)]
    for r in order:
        b = int(box[r])
        x0, y0, x1, y1 = b & 255, (b >> 8) & 255, (b >> 16) & 255, b >> 24
        for sy in range(y0 >> 3, (y1 >> 3) + 1):
            for sx in range(x0 >> 3, (x1 >> 3) + 1):
                rc = (max(x0 - 8 * sx, 0) | min(x1 - 8 * sx, 7) << 3 | max(y0 - 8 * sy, 0) << 6
                      | min(y1 - 8 * sy, 7) << 9)
                lists[sy * sb_cols + sx].append((rc, int(r)))
    flat = [e for lst in lists for e in lst]
    starts = np.concatenate([[0], np.cumsum([len(lst) for lst in lists])]).astype(np.int64)
    masks = [0] * ((len(flat) + 31) // 32)
    for i, (rc, _) in enumerate(flat):
        masks[i // 32] |= _rect_tiles(rc)
    walked_chunks = skipped = 0
    for ty in range(rows):
        for tx in range(cols):
            sb = (ty >> 3) * sb_cols + (tx >> 3)
            bit = 1 << ((ty & 7) * 8 + (tx & 7))
            beg, end = int(starts[sb]), int(starts[sb + 1])
            got = []
            for c in range(beg // 32, (end - 1) // 32 + 1 if end > beg else beg // 32):
                if not masks[c] & bit:
                    skipped += 1
                    continue
                walked_chunks += 1
                for i in range(max(beg, 32 * c), min(end, 32 * c + 32)):
                    rc, r = flat[i]
                    if _rect_tiles(rc) & bit:
                        got.append(r)
            t = _morton(tx, ty)
            o, n = int(f["tile_offsets"][t]), int(f["tile_counts"][t])
            assert got == f["tile_entries"][o:o + n].tolist(), (tx, ty)
    assert walked_chunks > 0 and skipped > 0


def test_f16_composite_variant(small_frame, orc):
    # gpu_tile_splat_composite_f16.wgsl: same projection and lists; f16
    # transmittance and colour change the image, within 2/255 of the f32 one
    f = small_frame["frame"]
    h = orc.render_frame(small_frame["u"], small_frame["packed"], small_frame["order"], threads=4, f16=True)
    for k in ("proj_cache", "tile_counts", "tile_offsets", "tile_entries"):
        assert np.array_equal(h[k], f[k]), k
    a = orc.f16_to_f32(f["color"].reshape(-1))
    b = orc.f16_to_f32(h["color"].reshape(-1))
    d = np.abs(a - b)
    assert d.max() > 0 and d.max() <= 2.0 / 255.0 and d.mean() < 5e-4
    # the variant's constants are the f16 roundings of 1/255, 0.001, 0.02, 0.04
    assert orc.f64_to_f16([1 / 255, 0.001, 0.02, 0.04]).tolist() == [0x1C04, 0x1419, 0x251F, 0x291F]


def test_f16_composite_matches_an_independent_numpy_restatement(orc, pkg, hdsr_lib):
    # gpu_tile_splat_composite_f16.wgsl:186-259 once more, vectorised over the
    # pixels of a tile with numpy float16 roundings, against the C oracle's
    # colour bits. An entry invalid for a pixel leaves it unchanged (w = 0),
    # so the quad skip and the early exit of the shader need no restating.
    # f32 fused multiply-adds are emulated in double (exact products; a
    # double rounding of the sum is the only, vanishingly rare, difference).
    scene = pkg.workloads.plain_scene(600, seed=21)
    packed = pkg.splats.pack_splat_attributes(scene)
    cam = pkg.camera.look_from((0.3, 0.2, 3.5))
    W = H = 64
    u, fr = _uniforms(pkg, W, H, scene.count, cam)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    f = orc.render_frame(u, packed, order, threads=2, f16=True)
    pc = f["proj_cache"]
    # (far below the support, where the exp's value is unused, it may overflow)
    h16 = lambda v: np.asarray(v, np.float64).astype(np.float16).astype(np.float64)  # noqa: E731
    fma32 = lambda a, b, c: (np.float64(a) * b + c).astype(np.float32)  # noqa: E731
    th, cut = h16(1.0 / 255.0), h16(0.001)
    bg = h16([0.02, 0.02, 0.04])
    got = orc.f16_to_f32(f["color"].reshape(-1)).reshape(H, W, 4)
    prev = np.seterr(over="ignore")
    try:
        _f16_tiles_match(orc, f, pc, got, h16, fma32, th, cut, bg, W, H)
    finally:
        np.seterr(**prev)


def _f16_tiles_match(orc, f, pc, got, h16, fma32, th, cut, bg, W, H):
    for ty in range(H // 16):
        for tx in range(W // 16):
            t = _morton(tx, ty)
            ents = f["tile_entries"][f["tile_offsets"][t]: f["tile_offsets"][t] + f["tile_counts"][t]]
            ys, xs = np.mgrid[ty * 16:ty * 16 + 16, tx * 16:tx * 16 + 16]
            px, py = (xs + 0.5).astype(np.float32), (ys + 0.5).astype(np.float32)
            T = np.ones((16, 16))
            col = np.zeros((16, 16, 3))
            for r in ents.tolist():
                w = pc[r]
                cx, cy, ia, ib, ic = (np.uint32(w[k]).view(np.float32) for k in range(5))
                ka, kb, kc = np.float32(ia * np.float32(-0.5)), np.float32(-ib), np.float32(ic * np.float32(-0.5))
                op = orc.f16_to_f32(np.array([w[6] >> 16], np.uint16))[0]
                rgb = orc.f16_to_f32(np.array([w[9] & 0xFFFF, w[9] >> 16, w[10] & 0xFFFF], np.uint16)).astype(np.float64)
                dx, dy = (px - cx).astype(np.float32), (py - cy).astype(np.float32)
                pw = fma32((kc * dy).astype(np.float32), dy, fma32((kb * dx).astype(np.float32), dy,
                                                                   ((ka * dx).astype(np.float32) * dx).astype(np.float32)))
                g = orc.splat_expf(pw).reshape(16, 16)
                a32 = np.minimum(np.float32(0.99), (op * g).astype(np.float32))
                a16 = h16(a32)
                valid = (pw > -4.0) & (a32 > th) & (T >= cut)
                nT = h16(T * h16(1.0 - a16))
                w16 = np.where(valid, h16(a16 * T), 0.0)
                col = h16(rgb[None, None, :] * w16[..., None] + col)
                T = np.where(valid, nT, T)
            out = h16(T[..., None] * bg[None, None, :] + col)
            assert np.array_equal(out.astype(np.float32), got[ty * 16:ty * 16 + 16, tx * 16:tx * 16 + 16, :3]), (tx, ty)
            alpha = (np.float32(1.0) - T.astype(np.float32)).astype(np.float16).astype(np.float32)
            assert np.array_equal(alpha, got[ty * 16:ty * 16 + 16, tx * 16:tx * 16 + 16, 3]), (tx, ty)


def _np_project(orc, U, packed, n):
    """See _np_project_body; branches the shader does not take may divide by
    zero in the vectorised form (their values are discarded)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return _np_project_body(orc, U, packed, n)


def _np_project_body(orc, U, packed, n):
    """project_splats (gpu_project_splats.wgsl:112-357) restated with numpy f32
    arithmetic for splat ids 0..n-1 in order: one rounding per operation, sums
    left to right, quotients that share a denominator as one correctly rounded
    reciprocal and products (the canonical form), the projection's own exp.
    Returns the expected cache words, depth and the visibility mask."""
    f32 = np.float32
    U = np.asarray(U, np.float32)
    P = packed.positions.reshape(-1, 3).astype(f32)
    x, y, z = P[:, 0], P[:, 1], P[:, 2]

    def dot(a, b):
        return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]

    def cross(a, b):
        return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])

    def norm(v):
        r = f32(1.0) / np.sqrt(dot(v, v))
        return tuple(c * r for c in v)

    clip = [((U[0 + r] * x + U[4 + r] * y) + U[8 + r] * z) + U[12 + r] * f32(1.0) for r in range(4)]
    vis = clip[3] > 0
    rW = f32(1.0) / np.maximum(clip[3], f32(0.0001))
    ndcx, ndcy = clip[0] * rW, clip[1] * rW
    cpx = (ndcx * f32(0.5) + f32(0.5)) * U[16]
    cpy = (f32(1.0) - (ndcy * f32(0.5) + f32(0.5))) * U[17]
    depth = clip[2] * rW
    sl = packed.scales.reshape(-1, 3).astype(f32)
    q = packed.rotations.reshape(-1, 4).astype(f32)
    scale = [orc.expf(sl[:, k]) * U[24] for k in range(3)]
    qn = q * (f32(1.0) / np.maximum(np.sqrt(((q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1]) + q[:, 2] * q[:, 2])
                                            + q[:, 3] * q[:, 3]), f32(0.000001)))[:, None]
    u3, qw = (qn[:, 1], qn[:, 2], qn[:, 3]), qn[:, 0]
    axes = []
    for k, e in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
        ev = tuple(np.full_like(x, f32(c)) for c in e)
        cu = cross(u3, ev)
        c2 = cross(u3, tuple(cu[i] + qw * ev[i] for i in range(3)))
        axes.append(tuple((ev[i] + f32(2.0) * c2[i]) * scale[k] for i in range(3)))
    vc = [((U[32 + r] * x + U[36 + r] * y) + U[40 + r] * z) + U[44 + r] * f32(1.0) for r in range(3)]
    vz = np.minimum(vc[2], f32(-0.001))
    rvz = f32(1.0) / vz
    J1x, J1y = U[48] * rvz, U[49] * rvz
    J2x, J2y = (-J1x * rvz) * vc[0], (-J1y * rvz) * vc[1]
    w0, w1, w2 = (U[32], U[36], U[40]), (U[33], U[37], U[41]), (U[34], U[38], U[42])
    tt0 = tuple(J1x * w0[i] + J2x * w2[i] for i in range(3))
    tt1 = tuple(J1y * w1[i] + J2y * w2[i] for i in range(3))
    b0, b1 = tuple(dot(a, tt0) for a in axes), tuple(dot(a, tt1) for a in axes)
    cxx, cxy, cyy = dot(b0, b0), dot(b0, b1), dot(b1, b1)
    detO = cxx * cyy - cxy * cxy
    cXX, cYY = cxx + f32(0.3), cyy + f32(0.3)
    detB = cXX * cYY - cxy * cxy
    dinv = f32(1.0) / np.maximum(detB, f32(0.000001))
    aa = np.sqrt(np.maximum(detO * dinv, f32(0.0)))
    mid = f32(0.5) * (cXX + cYY)
    lam = mid + np.sqrt(np.maximum(mid * mid - np.maximum(detB, f32(0.1)), f32(0.1)))
    radius = np.ceil(f32(3.0) * np.sqrt(lam))
    vis &= radius > 0
    ic = (cYY * dinv, -cxy * dinv, cXX * dinv)
    op = np.clip(packed.opacities.astype(f32) * aa, f32(0.0), f32(0.99))
    ts = np.maximum(U[18], f32(1.0))
    gx, gy = (int(np.asarray(U[20:22], np.float32).view(np.uint32)[k]) for k in range(2))
    cr = np.minimum(radius, ts * f32(8.0))
    lo = (np.maximum(cpx - cr, f32(0.0)), np.maximum(cpy - cr, f32(0.0)))
    hi = (np.minimum(cpx + cr, U[16]), np.minimum(cpy + cr, U[17]))
    sat = lambda v, m: np.minimum(np.clip(np.floor(v), 0, 2.0 ** 32 - 1).astype(np.uint64), m)  # noqa: E731
    rts = f32(1.0) / ts
    t0x, t0y = sat(lo[0] * rts, max(gx, 1) - 1), sat(lo[1] * rts, max(gy, 1) - 1)
    t1x = sat(np.maximum((hi[0] - f32(0.000000001)) * rts, f32(0.0)), max(gx, 1) - 1)
    t1y = sat(np.maximum((hi[1] - f32(0.000000001)) * rts, f32(0.0)), max(gy, 1) - 1)
    box = (t0x & 0xFF) | ((t0y & 0xFF) << 8) | ((t1x & 0xFF) << 16) | ((t1y & 0xFF) << 24)
    # normals (:233-291)
    lens = [dot(a, a) for a in axes]
    mn = np.minimum(lens[0], np.minimum(lens[1], lens[2]))
    pick = lambda i: np.where(lens[0] == mn, axes[0][i], np.where(lens[1] == mn, axes[1][i], axes[2][i]))  # noqa: E731
    sn = norm(tuple(pick(i) for i in range(3)))
    nd = np.zeros(0, f32) if packed.normals is None else packed.normals.reshape(-1).astype(f32)
    if nd.size >= 3 * n:
        bk = (nd[0:3 * n:3], nd[1:3 * n:3], nd[2:3 * n:3])
        bl = np.sqrt(dot(bk, bk))
        rbl = f32(1.0) / bl
        sn = tuple(np.where(bl > f32(0.001), bk[i] * rbl, sn[i]) for i in range(3))
    if nd.size >= 6 * n:
        dt = (nd[3 * n::3], nd[3 * n + 1::3], nd[3 * n + 2::3])
        dl = np.sqrt(dot(dt, dt))
        big0 = (lens[0] >= lens[1]) & (lens[0] >= lens[2])
        big1 = lens[1] >= lens[2]
        tc = tuple(np.where(big0, axes[0][i], np.where(big1, axes[1][i], axes[2][i])) for i in range(3))
        d = dot(tc, sn)
        tp = tuple(tc[i] - sn[i] * d for i in range(3))
        tl = np.sqrt(dot(tp, tp))
        rtl, rdl = f32(1.0) / tl, f32(1.0) / dl
        T = tuple(tp[i] * rtl for i in range(3))
        B = cross(sn, T)
        dn = tuple(dt[i] * rdl for i in range(3))
        m = norm(tuple((T[i] * dn[0] + B[i] * dn[1]) + sn[i] * dn[2] for i in range(3)))
        use = (dl > f32(0.001)) & (tl > f32(0.001))
        sn = tuple(np.where(use, m[i], sn[i]) for i in range(3))
    nvd = norm(tuple(U[28 + i] - P[:, i] for i in range(3)))
    fn, fv = norm(sn), norm(nvd)
    flip = dot(fn, fv) < 0
    faced = tuple(np.where(flip, -c, c) for c in fn)
    conf = np.clip(dot(faced, nvd), f32(0.0), f32(1.0))
    wn = norm(tuple((U[52 + k] * faced[0] + U[56 + k] * faced[1]) + U[60 + k] * faced[2] for k in range(3)))
    ox, oy = _oct_encode_np(np.stack(wn, -1), normalize=False, recip=True)
    # SH colour (:293-351) and emissive (:353-357)
    deg = packed.sh_degree
    sh = packed.sh_data.reshape(n, -1).astype(f32)
    K = (deg + 1) * (deg + 1) - 1
    col = [sh[:, c].copy() for c in range(3)]
    if deg >= 1:
        vd = norm(tuple(U[28 + i] - P[:, i] for i in range(3)))
        vx, vy, vzz = vd
        c = lambda j, ch: sh[:, 3 + 3 * j + ch]  # noqa: E731
        C1 = f32(0.4886025119029199)
        for ch in range(3):
            col[ch] = col[ch] + C1 * ((c(0, ch) * vy + c(1, ch) * vzz) + c(2, ch) * vx)
        if deg >= 2:
            xx, yy, zz = vx * vx, vy * vy, vzz * vzz
            xy, yz, xz = vx * vy, vy * vzz, vx * vzz
            b2 = [f32(1.0925484305920792) * xy, f32(1.0925484305920792) * yz,
                  f32(0.31539156525252005) * ((f32(2.0) * zz - xx) - yy), f32(1.0925484305920792) * xz,
                  f32(0.5462742152960396) * (xx - yy)]
            for ch in range(3):
                acc = c(3, ch) * b2[0]
                for j in range(1, 5):
                    acc = acc + c(3 + j, ch) * b2[j]
                col[ch] = col[ch] + acc
            if deg >= 3:
                b3 = [f32(0.5900435899266435) * vy * (f32(3.0) * xx - yy), f32(2.890611442640554) * vx * vy * vzz,
                      f32(0.4570457994644658) * vy * ((f32(4.0) * zz - xx) - yy),
                      f32(0.3731763325901154) * vzz * ((f32(2.0) * zz - f32(3.0) * xx) - f32(3.0) * yy),
                      f32(0.4570457994644658) * vx * ((f32(4.0) * zz - xx) - yy),
                      f32(1.445305721320277) * vzz * (xx - yy), f32(0.5900435899266435) * vx * (xx - f32(3.0) * yy)]
                for ch in range(3):
                    acc = c(8, ch) * b3[0]
                    for j in range(1, 7):
                        acc = acc + c(8 + j, ch) * b3[j]
                    col[ch] = col[ch] + acc
    col = [np.clip(v, f32(0.0), f32(1.0)) for v in col]
    em = sh[:, 3 + 3 * K: 6 + 3 * K]
    pk = lambda a, b: orc.f16_rne(a).astype(np.uint32) | (orc.f16_rne(b).astype(np.uint32) << 16)  # noqa: E731
    zero = np.zeros_like(x)
    bits = lambda v: np.asarray(v, np.float32).view(np.uint32)  # noqa: E731
    words = {0: bits(cpx), 1: bits(cpy), 2: bits(ic[0]), 3: bits(ic[1]), 4: bits(ic[2]),
             5: packed.material.reshape(-1).astype(np.uint32), 6: pk(radius, op), 7: box.astype(np.uint32),
             8: pk(ox, oy), 9: pk(col[0], col[1]), 10: pk(col[2], zero), 11: pk(em[:, 0], em[:, 1]),
             12: pk(em[:, 2], zero), 13: pk(conf, zero)}
    return words, bits(depth), vis


def _check_projection(orc, f, words, depth, vis):
    pc = f["proj_cache"]
    assert np.all(pc[~vis, 7] == 0xFFFFFFFF)
    for word, val in words.items():
        assert np.array_equal(pc[vis, word], val[vis]), word
    assert np.array_equal(f["depth"][vis], depth[vis])


def test_projection_geometry_matches_an_independent_numpy_restatement(orc, pkg, hdsr_lib):
    # every word of the cache row and the depth, bit for bit against the C
    # oracle; splats behind the camera get the sentinel (SH 0, no normals)
    scene = pkg.workloads.plain_scene(3000, seed=23)
    packed = pkg.splats.pack_splat_attributes(scene)
    cam = pkg.camera.look_from((0.4, 0.3, 2.0))
    u, fr = _uniforms(pkg, 320, 240, scene.count, cam)
    f = orc.render_frame(u, packed, np.arange(scene.count, dtype=np.uint32), threads=2, composite=False)
    words, depth, vis = _np_project(orc, u, packed, scene.count)
    assert vis.sum() > 1000 and (~vis).sum() > 0
    _check_projection(orc, f, words, depth, vis)


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_projection_sh_and_normals_match_an_independent_numpy_restatement(orc, pkg, hdsr_lib, deg):
    # the same with SH degrees 1-3, baked normals (some zero: the covariance
    # normal is kept) and tangent-space detail normals, emissive, materials
    rng = np.random.default_rng(30 + deg)
    scene = pkg.workloads.plain_scene(2000, seed=24)
    n = scene.count
    scene.sh_degree = deg
    scene.sh = rng.normal(0, 0.3, (n, 3 * ((deg + 1) ** 2 - 1))).astype(np.float32)
    nrm = rng.normal(0, 1, (n, 3)).astype(np.float32)
    nrm[::7] = 0.0
    scene.normals = nrm
    det = np.column_stack([rng.normal(0, 0.3, (n, 2)), np.ones(n)]).astype(np.float32)
    det[::5] = 0.0
    scene.detail_normals = det
    scene.emissive = rng.uniform(0, 2, (n, 3)).astype(np.float32)
    scene.roughness = rng.uniform(0, 1, n).astype(np.float32)
    scene.metalness = rng.uniform(0, 1, n).astype(np.float32)
    packed = pkg.splats.pack_splat_attributes(scene)
    assert packed.normals is not None and packed.normals.size == 6 * n
    cam = pkg.camera.look_from((0.6, 0.4, 2.5))
    u, fr = _uniforms(pkg, 320, 240, n, cam, sh_degree=deg)
    f = orc.render_frame(u, packed, np.arange(n, dtype=np.uint32), threads=2, composite=False)
    words, depth, vis = _np_project(orc, u, packed, n)
    assert vis.sum() > 500
    _check_projection(orc, f, words, depth, vis)


def _oct_decode_np(e):
    """octDecode (gpu_tile_splat_composite.wgsl:143-149) on one f16 pair, f32 steps,
    normalised by one correctly rounded reciprocal (the composites' canonical
    form of normalize)."""
    f32 = np.float32
    x, y = f32(e[0]), f32(e[1])
    z = (f32(1.0) - abs(x)) - abs(y)
    if z < 0:
        x, y = (f32(1.0) - abs(y)) * (f32(1.0) if x >= 0 else f32(-1.0)), (f32(1.0) - abs(x)) * (f32(1.0) if y >= 0 else f32(-1.0))
    r = f32(1.0) / np.sqrt((x * x + y * y) + z * z)
    return np.array([x * r, y * r, z * r], np.float32)


def test_finite_octahedral_halves_decode_to_a_finite_normal(orc):
    # The rasteriser decides from the stored bits whether a splat's vote
    # inputs are finite: an octahedral normal counts as finite when its two
    # f16 halves are, which holds because the decoded vector is never zero
    # (z = 1 - |x| - |y| is 1 where x = y = 0, and the fold leaves |x| or |y|
    # at 1 - |.| > 0 where z < 0) and its squares stay far below f32 overflow.
    f32 = np.float32
    bits = np.concatenate([np.arange(0, 0x7C00, 97, dtype=np.uint16),
                           np.array([0x0000, 0x0001, 0x03FF, 0x0400, 0x3BFF, 0x3C00, 0x3C01, 0x7BFF], np.uint16)])
    h = orc.f16_to_f32(np.concatenate([bits, bits | 0x8000]))
    x, y = np.meshgrid(h, h)
    x, y = x.reshape(-1).astype(f32), y.reshape(-1).astype(f32)
    z = (f32(1.0) - np.abs(x)) - np.abs(y)
    fold = z < 0
    x2 = (f32(1.0) - np.abs(y)) * np.where(x >= 0, f32(1.0), f32(-1.0))
    y2 = (f32(1.0) - np.abs(x)) * np.where(y >= 0, f32(1.0), f32(-1.0))
    x, y = np.where(fold, x2, x), np.where(fold, y2, y)
    l2 = (x * x + y * y) + z * z
    assert np.all(l2 > 0) and np.all(np.isfinite(l2))
    r = f32(1.0) / np.sqrt(l2)
    assert np.all(np.isfinite(x * r)) and np.all(np.isfinite(y * r)) and np.all(np.isfinite(z * r))


def _oct_encode_np(v, normalize=True, recip=False):
    """octEncode(normalize(v)) (gpu_tile_splat_composite.wgsl:134-141), or octEncode(v)
    for an already unit v, vectorised, f32 steps; recip: each normalisation by one
    correctly rounded reciprocal and products (the composites' canonical form)."""
    f32 = np.float32
    x, y, z = v[..., 0], v[..., 1], v[..., 2]
    if normalize:
        if recip:
            r = f32(1.0) / np.sqrt((x * x + y * y) + z * z)
            x, y, z = x * r, y * r, z * r
        else:
            ln = np.sqrt((x * x + y * y) + z * z)
            x, y, z = x / ln, y / ln, z / ln
    s = (np.abs(x) + np.abs(y)) + np.abs(z)
    if recip:
        rs = f32(1.0) / s
        px, py = x * rs, y * rs
    else:
        px, py = x / s, y / s
    sx, sy = np.where(px >= 0, f32(1.0), f32(-1.0)), np.where(py >= 0, f32(1.0), f32(-1.0))
    nx, ny = (f32(1.0) - np.abs(py)) * sx, (f32(1.0) - np.abs(px)) * sy
    neg = z < 0
    return np.where(neg, nx, px).astype(np.float32), np.where(neg, ny, py).astype(np.float32)


def test_f32_composite_matches_an_independent_numpy_restatement(orc, pkg, hdsr_lib):
    # gpu_tile_splat_composite.wgsl:134-370 (the canonical f32 form: fused
    # power and accumulations) restated with numpy over the pixels of each
    # tile, against the C oracle's colour, alpha, depth, normal and material
    # bits (see the f16 test for why the quad skip and early exit need no
    # restating).
    scene = pkg.workloads.plain_scene(600, seed=22)
    packed = pkg.splats.pack_splat_attributes(scene)
    cam = pkg.camera.look_from((-0.2, 0.3, 3.5))
    W = H = 64
    u, fr = _uniforms(pkg, W, H, scene.count, cam)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    f = orc.render_frame(u, packed, order, threads=2)
    pc = f["proj_cache"]
    got = orc.f16_to_f32(f["color"].reshape(-1)).reshape(H, W, 4)
    fma32 = lambda a, b, c: (np.asarray(a, np.float64) * b + c).astype(np.float32)  # noqa: E731
    bg = np.array([0.02, 0.02, 0.04], np.float32)
    prev = np.seterr(over="ignore", invalid="ignore")
    try:
        for ty in range(H // 16):
            for tx in range(W // 16):
                t = _morton(tx, ty)
                ents = f["tile_entries"][f["tile_offsets"][t]: f["tile_offsets"][t] + f["tile_counts"][t]]
                ys, xs = np.mgrid[ty * 16:ty * 16 + 16, tx * 16:tx * 16 + 16]
                px, py = (xs + 0.5).astype(np.float32), (ys + 0.5).astype(np.float32)
                T = np.ones((16, 16), np.float32)
                col = np.zeros((16, 16, 3), np.float32)
                gd, gW, gc = (np.zeros((16, 16), np.float32) for _ in range(3))
                mat, nrm, em = np.zeros((16, 16, 2), np.float32), np.zeros((16, 16, 3), np.float32), np.zeros((16, 16, 3), np.float32)
                for r in ents.tolist():
                    w = pc[r]
                    cx, cy, ia, ib, ic = (np.uint32(w[k]).view(np.float32) for k in range(5))
                    ka, kb, kc = np.float32(ia * np.float32(-0.5)), np.float32(-ib), np.float32(ic * np.float32(-0.5))
                    op = orc.f16_to_f32(np.array([w[6] >> 16], np.uint16))[0]
                    rgb = orc.f16_to_f32(np.array([w[9] & 0xFFFF, w[9] >> 16, w[10] & 0xFFFF], np.uint16))
                    dx, dy = (px - cx).astype(np.float32), (py - cy).astype(np.float32)
                    pw = fma32((kc * dy).astype(np.float32), dy, fma32((kb * dx).astype(np.float32), dy,
                                                                       ((ka * dx).astype(np.float32) * dx).astype(np.float32)))
                    g = orc.splat_expf(pw).reshape(16, 16)
                    al = np.minimum(np.float32(0.99), (op * g).astype(np.float32))
                    nT = (T * (np.float32(1.0) - al).astype(np.float32)).astype(np.float32)
                    valid = (pw > -4.0) & (al > np.float32(1.0) / np.float32(255.0)) & (T >= np.float32(0.001))
                    wt = np.where(valid, (al * T).astype(np.float32), np.float32(0.0))
                    col = fma32(rgb[None, None, :], wt[..., None], col)
                    T = np.where(valid, nT, T)
                    gw = np.where(wt > np.float32(0.01), wt, np.float32(0.0))
                    sd = np.uint32(f["depth"][r]).view(np.float32)
                    mr = orc.f16_to_f32(np.array([w[5] & 0xFFFF, w[5] >> 16], np.uint16))
                    sn = _oct_decode_np(orc.f16_to_f32(np.array([w[8] & 0xFFFF, w[8] >> 16], np.uint16)))
                    sc = orc.f16_to_f32(np.array([w[13] & 0xFFFF], np.uint16))[0]
                    er = orc.f16_to_f32(np.array([w[11] & 0xFFFF, w[11] >> 16, w[12] & 0xFFFF], np.uint16))
                    gd = fma32(gw, sd, gd)
                    gW = (gW + gw).astype(np.float32)
                    mat = fma32(mr[None, None, :], gw[..., None], mat)
                    nrm = fma32(sn[None, None, :], gw[..., None], nrm)
                    gc = fma32(sc, gw, gc)
                    em = fma32(er[None, None, :], wt[..., None], em)
                out = fma32(T[..., None], bg[None, None, :], col).astype(np.float16).astype(np.float32)
                assert np.array_equal(out, got[ty * 16:ty * 16 + 16, tx * 16:tx * 16 + 16, :3]), (tx, ty)
                alpha = (np.float32(1.0) - T).astype(np.float16).astype(np.float32)
                assert np.array_equal(alpha, got[ty * 16:ty * 16 + 16, tx * 16:tx * 16 + 16, 3]), (tx, ty)
                rsw = (np.float32(1.0) / np.maximum(gW, np.float32(0.0001))).astype(np.float32)
                sl = np.s_[ty * 16:ty * 16 + 16, tx * 16:tx * 16 + 16]
                assert np.array_equal((gd * rsw).astype(np.float32), f["out_depth"][sl]), (tx, ty)
                nn = nrm + np.array([0.0, 0.0001, 0.0], np.float32)
                ox, oy = _oct_encode_np(nn, recip=True)
                pk = lambda a, b: orc.f16_rne(a.reshape(-1)).astype(np.uint32) | (orc.f16_rne(b.reshape(-1)).astype(np.uint32) << 16)  # noqa: E731
                assert np.array_equal(pk(ox, oy), f["normal"][sl].reshape(-1)), (tx, ty)
                zero = np.zeros((16, 16), np.float32)
                m = f["material"][sl].reshape(-1, 4)
                assert np.array_equal(pk((mat[..., 0] * rsw).astype(np.float32), (mat[..., 1] * rsw).astype(np.float32)), m[:, 0])
                assert np.array_equal(pk(em[..., 0], em[..., 1]), m[:, 1])
                assert np.array_equal(pk(em[..., 2], zero), m[:, 2])
                assert np.array_equal(pk((gc * rsw).astype(np.float32), zero), m[:, 3])
    finally:
        np.seterr(**prev)


def test_composite_close_to_fp64(small_frame, orc):
    f = small_frame["frame"]
    img = orc.f16_to_f32(f["color"].reshape(-1)).reshape(f["H"], f["W"], 4).astype(np.float64)
    ref = orc.render_frame_f64(small_frame["u"], small_frame["packed"], small_frame["order"], f, threads=4)
    err = np.abs(img - ref)
    assert err.mean() < 2e-3
    mse = np.mean((img[..., :3] - ref[..., :3]) ** 2)
    assert 10 * np.log10(1.0 / max(mse, 1e-20)) > 40.0


def test_oracle_deterministic_across_threads(pkg, orc, small_frame):
    a = orc.render_frame(small_frame["u"], small_frame["packed"], small_frame["order"], threads=1)
    b = small_frame["frame"]
    for k in ("proj_cache", "depth", "tile_counts", "tile_offsets", "tile_entries", "color", "material"):
        assert np.array_equal(a[k], b[k]), k


def _stack_scene(pkg, n, pos=(0.0, 0.0, 0.0), log_scale=-6.0, depth_jitter=0.0, seed=0):
    rng = np.random.default_rng(seed)
    p = np.tile(np.array(pos, np.float32), (n, 1))
    p[:, 2] += rng.uniform(-depth_jitter, depth_jitter, n).astype(np.float32)
    return pkg.splats.SplatAttributes(
        positions=p, scales=np.full((n, 3), log_scale, np.float32),
        rotations=np.tile(np.array([1, 0, 0, 0], np.float32), (n, 1)),
        opacities=np.full(n, 0.5, np.float32), colors=rng.uniform(0, 1, (n, 3)).astype(np.float32))


@pytest.mark.parametrize("n,hot", [(4096, 0), (4097, 1), (9000, 1)])
def test_hot_tile_threshold_and_chunks(orc, pkg, hdsr_lib, n, hot):
    """A tile with exactly 4096 entries stays small; 4097 makes it hot and
    splits it into 4096-entry chunks in bucket order."""
    scene = _stack_scene(pkg, n, pos=(0.72, -0.72, 0.0), depth_jitter=0.5, seed=n)  # tile (2, 2)
    packed = pkg.splats.pack_splat_attributes(scene)
    cam = pkg.camera.look_from((0, 0, 5))
    u, fr = _uniforms(pkg, 64, 64, n, cam)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    f = orc.render_frame(u, packed, order, composite=False)
    assert f["hot_tiles"] == hot
    busiest = int(np.argmax(f["tile_counts"]))
    assert f["tile_counts"][busiest] == n
    if hot:
        assert f["total_chunks"] == (n + 4095) // 4096
        sizes = f["chunk_ranges"][:, 1].tolist()
        assert sizes[:-1] == [4096] * (len(sizes) - 1)
        assert not (f["flags"] & orc.FLAG_BUCKET_KEY_MISMATCH)
        # chunks are in bucket (k20) order: every entry of chunk c has k20
        # <= every entry of chunk c+1
        keys, vals = orc.sorted_keys20(u, f["proj_cache"], f["depth"])
        tile_keys = keys[(keys >> np.uint64(20)) == busiest] & np.uint64(0xFFFFF)
        k_of = dict(zip(vals[(keys >> np.uint64(20)) == busiest].tolist(), tile_keys.tolist()))
        start = f["tile_offsets"][busiest]
        for c in range(len(sizes) - 1):
            a = f["tile_entries"][start + 4096 * c: start + 4096 * (c + 1)]
            b = f["tile_entries"][start + 4096 * (c + 1): start + 4096 * (c + 2)]
            assert max(k_of[x] for x in a.tolist()) <= min(k_of[x] for x in b.tolist())


@pytest.mark.parametrize("n", [4097, 9000, 12288])
def test_chunk_ranges_readback_matches_the_cascade(orc, pkg, hdsr_lib, n):
    # the chunk table the host derives from tile counts and offsets equals the
    # oracle's greedy chunk packing of the bucket cascade
    scene = _stack_scene(pkg, n, pos=(0.72, -0.72, 0.0), depth_jitter=0.5, seed=n)
    packed = pkg.splats.pack_splat_attributes(scene)
    u, fr = _uniforms(pkg, 64, 64, n, pkg.camera.look_from((0, 0, 5)))
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    f = orc.render_frame(u, packed, order, composite=False)
    got = pkg.compositor.chunk_ranges_from_tiles(f["tile_counts"], f["tile_offsets"])
    assert got.shape[0] == f["total_chunks"] == (n + 4095) // 4096
    assert np.array_equal(got, f["chunk_ranges"])


def test_equal_depth_ties_break_by_sort_rank(orc, pkg, hdsr_lib):
    scene = _stack_scene(pkg, 300, pos=(0.72, -0.72, 0.0), depth_jitter=0.0)
    packed = pkg.splats.pack_splat_attributes(scene)
    u, fr = _uniforms(pkg, 64, 64, 300, pkg.camera.look_from((0, 0, 5)))
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    f = orc.render_frame(u, packed, order, composite=False)
    t = int(np.argmax(f["tile_counts"]))
    e = f["tile_entries"][f["tile_offsets"][t]: f["tile_offsets"][t] + f["tile_counts"][t]]
    assert np.array_equal(e, np.arange(300))


def test_two_overlapping_splats_front_to_back(orc, pkg, hdsr_lib):
    """Hand-computed front-to-back blend at a splat centre pixel."""
    scene = pkg.splats.SplatAttributes(
        positions=np.array([[0, 0, 0], [0, 0, -1.0]], np.float32),
        scales=np.full((2, 3), -1.0, np.float32), rotations=np.array([[1, 0, 0, 0]] * 2, np.float32),
        opacities=np.array([0.5, 0.9], np.float32), colors=np.array([[1, 0, 0], [0, 0, 1]], np.float32))
    packed = pkg.splats.pack_splat_attributes(scene)
    u, fr = _uniforms(pkg, 64, 64, 2, pkg.camera.look_from((0, 0, 5)))
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    f = orc.render_frame(u, packed, order)
    img = orc.f16_to_f32(f["color"].reshape(-1)).reshape(64, 64, 4)
    # near splat (red, the one at z=0) is first after the per-tile depth sort
    a0 = orc.f16_to_f32(np.array([f["proj_cache"][order.tolist().index(0), 6] >> 16], np.uint16))[0]
    a1 = orc.f16_to_f32(np.array([f["proj_cache"][order.tolist().index(1), 6] >> 16], np.uint16))[0]
    px = img[31, 31]
    # pixel (31,31) centre is 0.5 px from the projected centre (32,32) in x and y
    assert px[0] > px[2] > 0
    assert abs((1 - px[3]) - (1 - a0 * np.exp(-0.5 * 0)) * (1 - a1)) < 0.2


def test_log_is_monotone(orc):
    """The hot-tile buckets are monotone in depth only if the log is: check
    every float in [0.5, 4) (2^24 values, all of the mantissa patterns) and a
    stride of all positive floats. An exhaustive pass over every positive
    float (2.1e9 values) found no decreasing step either."""
    dense = np.arange(0x3F000000, 0x40800000, dtype=np.uint32).view(np.float32)
    y = orc.logf(dense)
    assert np.all(y[1:] >= y[:-1])
    sparse = np.arange(1, 0x7F800000, 97, dtype=np.uint32).view(np.float32)
    y = orc.logf(sparse)
    assert np.all(y[1:] >= y[:-1])


@pytest.mark.parametrize("near", [False, True])
def test_every_tile_ends_in_depth_rank_order(orc, pkg, hdsr_lib, near):
    """Canonical frame: small tiles, hot tiles (bucket cascade) and tiles with
    negative depths (bucket range collapsed) all end in ascending (depth bits,
    sortRank) order."""
    rng = np.random.default_rng(31)
    scene = _stack_scene(pkg, 9000, pos=(0.72, -0.72, 0.0), depth_jitter=1.0, seed=31)
    if near:
        scene.positions[:30] = np.array([0.0, 0.0, 5.0 - 0.004], np.float32) + rng.normal(0, 1e-4, (30, 3)).astype(
            np.float32)
    packed = pkg.splats.pack_splat_attributes(scene)
    u, fr = _uniforms(pkg, 64, 64, scene.count, pkg.camera.look_from((0, 0, 5)))
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    f = orc.render_frame(u, packed, order, composite=False)
    assert f["hot_tiles"] >= 1
    if near:
        assert (f["depth"].view(np.float32) < 0).any()
    for t in np.nonzero(f["tile_counts"])[0]:
        e = f["tile_entries"][f["tile_offsets"][t]: f["tile_offsets"][t] + f["tile_counts"][t]]
        key = f["depth"][e].astype(np.uint64) << np.uint64(32) | e.astype(np.uint64)
        assert np.all(key[1:] > key[:-1])
