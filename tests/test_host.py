"""Host-side logic of the drop-in boundary (no GPU needed): the C ABI loads
and exports everything include/hdsr.h declares, the plan and the frame
uniform block match the reference layout, the camera conventions hold."""
import ctypes
import math
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "hdsr.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hdsr_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(hdsr_lib):
    names = declared_functions()
    assert len(names) >= 14
    missing = [n for n in names if not hasattr(hdsr_lib, n)]
    assert not missing, missing


def test_python_mirror_constants_match_the_header(pkg):
    # status codes, config flags, device flags and buffer ids of the Python
    # mirror carry the values include/hdsr.h gives them
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "hdsr.h").read_text(), flags=re.S)
    lib = pkg._lib
    defines = dict((m[0], int(m[1], 16)) for m in re.findall(r"#define HDSR_((?:CFG|DEV)_\w+)\s+(0x[0-9a-fA-F]+)u", text))
    assert {"CFG_F16_COMPOSITE", "CFG_TILE_ENTRIES", "CFG_NO_GRAPH", "DEV_OVERFLOW"} <= set(defines)
    for name, value in defines.items():
        if hasattr(lib, name):
            assert getattr(lib, name) == value, name
    for name in ("CFG_KEEP_SORTED_KEYS", "CFG_NO_GRAPH", "CFG_BACKWARD", "CFG_TILE_ENTRIES", "CFG_F16_COMPOSITE"):
        assert getattr(lib, name) == defines[name], name
    enums = dict((m[0], int(m[1])) for m in re.findall(r"\bHDSR_((?:ERR|BUF)_\w+)\s*=\s*(\d+)", text))
    for name, value in enums.items():
        if name.startswith("ERR_"):
            assert getattr(lib, "HDSR_" + name) == value, name
    buf = {k: v for k, v in enums.items() if k.startswith("BUF_")}
    assert {("BUF_" + k.upper()): v for k, v in lib.BUFFER_IDS.items()} == buf


def test_abi_version(hdsr_lib):
    assert hdsr_lib.hdsr_abi_version() == 4


@pytest.mark.parametrize("W,H,N", [(800, 600, 50_000), (1920, 1080, 760_000), (3840, 2160, 3_000_000),
                                   (512, 512, 1), (1280, 720, 100_000), (1024, 1024, 500_000), (17, 33, 0)])
def test_plan_matches_oracle(pkg, orc, W, H, N):
    p = pkg.plan_tile_splat_compositor(W, H, 16, N)
    o = orc.plan(W, H, 16, N)
    assert [p.viewport_width, p.viewport_height, p.tile_size_px, p.tile_columns, p.tile_rows, p.tile_count,
            p.morton_tile_count, p.splat_count, p.max_total_tile_refs] == o.tolist()


def test_plan_rejects_zero_viewport(pkg):
    with pytest.raises(pkg._lib.HdsrError):
        pkg.plan_tile_splat_compositor(0, 10, 16, 5)


def test_frame_uniform_layout(pkg):
    plan = pkg.plan_tile_splat_compositor(1920, 1080, 16, 760_000)
    vp = np.arange(16, dtype=np.float32) + 1
    view = np.arange(16, dtype=np.float32) + 100
    proj = np.zeros(16, np.float32)
    proj[0], proj[5] = np.float32(0.9742785792574935), np.float32(1.7320508075688774)
    nm = np.arange(9, dtype=np.float32) + 50
    u = pkg.write_tile_splat_frame_uniforms(None, vp, plan, 1.5, 3, [7, 8, 9], view, proj, nm)
    uu = u.view(np.uint32)
    assert np.array_equal(u[:16], vp)
    assert u[16] == 1920 and u[17] == 1080 and u[18] == 16 and u[19] == 0
    assert uu[20:24].tolist() == [120, 68, 760_000, 760_000 * 16]
    assert u[24] == np.float32(1.5) and uu[25] == 3
    assert u[28:31].tolist() == [7, 8, 9]
    assert np.array_equal(u[32:48], view)
    assert u[48] == np.float32(1920 * float(proj[0]) * 0.5)
    assert u[49] == np.float32(1080 * float(proj[5]) * 0.5)
    assert u[52:55].tolist() == [50, 51, 52] and u[55] == 0
    assert u[56:59].tolist() == [53, 54, 55] and u[59] == 0
    assert u[60:63].tolist() == [56, 57, 58] and u[63] == 0


@pytest.mark.parametrize("W,H,N,deg", [(1920, 1080, 760_000, 0), (3840, 2160, 3_000_000, 3), (203, 117, 7, 1)])
def test_oracle_frame_uniforms_match_the_c_abi(pkg, orc, W, H, N, deg):
    # the reference arm of the benchmark builds its uniform blocks with the
    # oracle (no product library): the same 64 words as the C ABI's writer
    plan = pkg.plan_tile_splat_compositor(W, H, 16, N)
    cam = pkg.camera.OrbitCamera(azimuth=0.7, elevation=0.3, distance=5.5)
    u, fr = pkg.frame_uniforms_for(plan, cam, sh_degree=deg)
    o = orc.frame_uniforms(orc.plan(W, H, 16, N), fr["view_proj"], 1.0, deg, fr["camera_pos"], fr["view"],
                           fr["proj"], None)
    assert np.array_equal(o.view(np.uint32), u.view(np.uint32))


def test_frame_uniform_defaults(pkg):
    plan = pkg.plan_tile_splat_compositor(800, 600, 16, 10)
    u = pkg.write_tile_splat_frame_uniforms(None, np.eye(4, dtype=np.float32).reshape(-1), plan)
    assert u[24] == 1.0 and u.view(np.uint32)[25] == 0
    assert not u[28:31].any() and not u[32:50].any()
    assert u[52] == 1 and u[57] == 1 and u[62] == 1


def test_camera_at_0_0_5_looking_at_origin(pkg):
    cam = pkg.camera.look_from((0.0, 0.0, 5.0))
    fr = cam.frame(800, 600)
    v = fr["view"].reshape(4, 4)  # column-major rows = columns
    assert np.allclose(v[:3, :3], np.eye(3), atol=1e-7)
    assert np.allclose(v[3, :3], [0, 0, -5], atol=1e-6)
    f = 1 / math.tan(math.pi / 6)
    p = fr["proj"]
    assert np.isclose(p[0], f / (800 / 600)) and np.isclose(p[5], f)
    assert p[11] == -1 and np.isclose(p[10], 100 / (0.01 - 100))
    vp = fr["view_proj"]
    assert np.isclose(vp[5], -f)  # viewer vertical flip
    assert np.allclose(fr["camera_pos"], [0, 0, 5], atol=1e-6)


def test_orbit_matches_reference_basis(pkg):
    cam = pkg.camera.OrbitCamera(azimuth=0.7, elevation=0.3, distance=4.0)
    v = cam.view_matrix().reshape(4, 4)
    R = v[:3, :3].T  # rows: right, up, back
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-6)
    eye = np.array(cam.position())
    assert np.allclose(R @ eye + v[3, :3], 0, atol=1e-5)


def test_sh_data_packing_layout(pkg):
    dc = np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]], np.float32)
    sh = np.arange(18, dtype=np.float32).reshape(2, 9)
    em = np.array([[7, 8, 9], [10, 11, 12]], np.float32)
    out = pkg.splats.pack_sh_data_buffer(dc, sh, em).reshape(2, 15)
    assert np.array_equal(out[:, :3], dc) and np.array_equal(out[:, 3:12], sh) and np.array_equal(out[:, 12:], em)
    assert pkg.splats.pack_sh_data_buffer(dc).reshape(2, 6)[:, 3:].sum() == 0


def test_normal_buffer_packing(pkg):
    n = np.ones((3, 3), np.float32)
    d = np.full((3, 3), 2, np.float32)
    assert pkg.splats.pack_normal_buffer(3, n).size == 9
    out = pkg.splats.pack_normal_buffer(3, n, d)
    assert out.size == 18 and out[:9].sum() == 9 and out[9:].sum() == 18


def test_hot_camera_has_twenty_hot_tiles(orc, pkg, hdsr_lib):
    """The recorded camera of the 760k hot-tile workload puts >= 20 tiles
    above 4096 entries (checked with the oracle's projection + count)."""
    wl = pkg.workloads.hot760k()
    packed = pkg.splats.pack_splat_attributes(wl.scene)
    plan = pkg.plan_tile_splat_compositor(wl.width, wl.height, 16, wl.scene.count)
    u, fr = pkg.frame_uniforms_for(plan, wl.cameras[0])
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    import oracle

    scene, keep = oracle.scene_struct(packed, order)
    cache = np.zeros(wl.scene.count * 14, np.uint32)
    depth = np.zeros(wl.scene.count, np.uint32)
    L = oracle.lib()
    L.orc_project(u.ctypes.data_as(ctypes.c_void_p), ctypes.byref(scene), cache.ctypes.data_as(ctypes.c_void_p),
                  depth.ctypes.data_as(ctypes.c_void_p), 8)
    counts = np.zeros(plan.morton_tile_count, np.uint32)
    L.orc_count_tile_refs(u.ctypes.data_as(ctypes.c_void_p), wl.scene.count, cache.ctypes.data_as(ctypes.c_void_p),
                          plan.morton_tile_count, counts.ctypes.data_as(ctypes.c_void_p))
    assert int((counts > 4096).sum()) >= 20


def test_server_rejects_bad_configs_without_a_gpu(pkg, hdsr_lib):
    import ctypes

    out = ctypes.c_void_p()
    for budget, inflight in ((0, 4), (1 << 30, 0), (1 << 30, 65)):
        cfg = pkg._lib.ServerConfig(budget, inflight, 0)
        assert hdsr_lib.hdsr_server_create(ctypes.byref(cfg), ctypes.byref(out)) == pkg._lib.HDSR_ERR_INVALID_ARG
    assert hdsr_lib.hdsr_server_create(None, ctypes.byref(out)) == pkg._lib.HDSR_ERR_INVALID_ARG
    assert hdsr_lib.hdsr_server_submit(None, None, None) == pkg._lib.HDSR_ERR_INVALID_ARG
