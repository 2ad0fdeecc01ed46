"""Oracle: CPU restatement of the reference compute compositor.

TEST INFRASTRUCTURE ONLY — the checker, never the product. Only tests/,
__graft_entry__.smoke() and the CPU-baseline leg of bench.py load it. See
hdsr_oracle.h for what it restates (file:line), the canonical tie-break
order and its parity status ("parity unpinned" for the compositor passes;
pinned for the CPU depth sort and constants by the reference's unit tests).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_uint16, c_uint32, c_uint64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRC = HERE / "hdsr_oracle.c"
POST_SRC = HERE / "hdsr_post_oracle.c"
CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]

FLAG_LARGE_SPLAT_CAP = 1
FLAG_REF_BUDGET_DROP = 2
FLAG_OVERFLOW_SKIP = 4
FLAG_CHUNK_CAP = 8
FLAG_BUCKET_KEY_MISMATCH = 16


def build(force: bool = False) -> Path:
    """gcc recipe for liboracle.so (no -march flags: identical on x86 and Arm)."""
    deps = [SRC, POST_SRC, HERE / "hdsr_oracle.h"]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        cc = os.environ.get("CC", "gcc")
        subprocess.run([cc, *CFLAGS, str(SRC), str(POST_SRC), "-o", str(LIB), "-lm"], check=True)
    return LIB


class Scene(ctypes.Structure):
    _fields_ = [("splat_count", c_uint32), ("sh_degree", c_uint32), ("positions", c_void_p), ("scales", c_void_p),
                ("rotations", c_void_p), ("opacities", c_void_p), ("sorted_indices", c_void_p),
                ("material", c_void_p), ("normals", c_void_p), ("normals_len", c_uint64), ("sh_data", c_void_p)]


class Frame(ctypes.Structure):
    _fields_ = [("proj_cache", c_void_p), ("depth", c_void_p), ("tile_counts", c_void_p),
                ("tile_offsets", c_void_p), ("tile_entries", c_void_p), ("entries_cap", c_uint64),
                ("chunk_ranges", c_void_p), ("chunk_cap", c_uint32), ("total_pairs", c_uint64),
                ("small_tiles", c_uint32), ("hot_tiles", c_uint32), ("total_chunks", c_uint32),
                ("large_splats", c_uint32), ("flags", c_uint32), ("composite_f16", c_uint32), ("out_color", c_void_p),
                ("out_depth", c_void_p), ("out_normal", c_void_p), ("out_material", c_void_p)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        L.orc_expf.restype = c_float
        L.orc_expf.argtypes = [c_float]
        L.orc_logf.restype = c_float
        L.orc_logf.argtypes = [c_float]
        L.orc_morton.restype = c_uint32
        L.orc_morton.argtypes = [c_uint32, c_uint32]
        L.orc_plan.argtypes = [c_uint32, c_uint32, c_uint32, c_uint32, c_double, c_void_p]
        L.orc_project.argtypes = [c_void_p, POINTER(Scene), c_void_p, c_void_p, c_int]
        L.orc_count_tile_refs.argtypes = [c_void_p, c_uint32, c_void_p, c_uint32, c_void_p]
        L.orc_exclusive_scan.argtypes = [c_void_p, c_uint32, c_void_p]
        L.orc_render_frame.restype = c_int
        L.orc_render_frame.argtypes = [c_void_p, POINTER(Scene), POINTER(Frame), c_int]
        L.orc_sorted_keys20.restype = c_int
        L.orc_sorted_keys20.argtypes = [c_void_p, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p, c_uint64,
                                        POINTER(c_uint64)]
        L.orc_composite.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, POINTER(Frame),
                                    c_int]
        L.orc_render_frame_f64.restype = c_int
        L.orc_render_frame_f64.argtypes = [c_void_p, POINTER(Scene), c_void_p, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_project_f64.argtypes = [c_void_p, POINTER(Scene), c_void_p, c_int]
        L.orc_sort_back_to_front.restype = c_int
        L.orc_sort_back_to_front.argtypes = [c_void_p, c_uint32, c_void_p, c_void_p, c_int]
        L.orc_gpu_sort_prototype_order.restype = c_int
        L.orc_gpu_sort_prototype_order.argtypes = [c_void_p, c_uint32, c_void_p, c_void_p]
        for nm in ("orc_expf_n", "orc_logf_n", "orc_f16_rne_n", "orc_f16_trunc_n", "orc_f16_to_f32_n", "orc_f64_to_f16_n",
                   "orc_composite_expf_n", "orc_splat_expf_n"):
            getattr(L, nm).argtypes = [c_void_p, c_void_p, c_uint64]
        L.orc_morton_n.argtypes = [c_void_p, c_void_p, c_void_p, c_uint64]
        L.orc_splat_exp_parts_n.argtypes = [c_void_p, c_void_p, c_void_p, c_uint64]
        L.orc_bucket_key20_n.argtypes = [c_void_p, c_uint64, c_uint32, c_uint32, c_void_p, c_void_p]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(c_void_p)


def threads_default() -> int:
    return os.cpu_count() or 1


def scene_struct(packed, sorted_indices):
    """orc_scene over a splats.PackedSplats; returns (struct, keepalive)."""
    arrays = dict(
        positions=np.ascontiguousarray(packed.positions, np.float32),
        scales=np.ascontiguousarray(packed.scales, np.float32),
        rotations=np.ascontiguousarray(packed.rotations, np.float32),
        opacities=np.ascontiguousarray(packed.opacities, np.float32),
        sorted_indices=np.ascontiguousarray(sorted_indices, np.uint32),
        material=np.ascontiguousarray(packed.material, np.uint32),
        normals=None if packed.normals is None else np.ascontiguousarray(packed.normals, np.float32),
        sh_data=np.ascontiguousarray(packed.sh_data, np.float32),
    )
    s = Scene(packed.count, packed.sh_degree, _p(arrays["positions"]), _p(arrays["scales"]),
              _p(arrays["rotations"]), _p(arrays["opacities"]), _p(arrays["sorted_indices"]),
              _p(arrays["material"]), _p(arrays["normals"]),
              0 if arrays["normals"] is None else arrays["normals"].size, _p(arrays["sh_data"]))
    return s, arrays


def _u32(u):
    return np.asarray(u, np.float32).view(np.uint32)


def render_frame(U: np.ndarray, packed, sorted_indices, threads: int | None = None, composite: bool = True,
                 cap: int | None = None, f16: bool = False) -> dict:
    """Full canonical frame: cache, counts, offsets, per-tile order, outputs.
    `cap` is the initial entry capacity (grown and retried when too small);
    `f16` selects the f16 composite variant (gpu_tile_splat_composite_f16.wgsl)."""
    L = lib()
    U = np.ascontiguousarray(U, np.float32)
    uu = _u32(U)
    N, cols, rows = int(uu[22]), int(uu[20]), int(uu[21])
    W, H = int(U[16]), int(U[17])
    M = int(L.orc_morton(cols - 1, rows - 1)) + 1
    scene, keep = scene_struct(packed, sorted_indices)
    nt = threads or threads_default()
    cap = max(16, N * 16, int(cap or 0))
    chunk_cap = max(1024, (cap + 4095) // 4096 + 1)
    while True:
        out = dict(
            proj_cache=np.zeros(max(N, 1) * 14, np.uint32), depth=np.zeros(max(N, 1), np.uint32),
            tile_counts=np.zeros(M, np.uint32), tile_offsets=np.zeros(M, np.uint32),
            tile_entries=np.zeros(cap, np.uint32), chunk_ranges=np.zeros(2 * chunk_cap, np.uint32))
        if composite:
            out.update(color=np.zeros(W * H * 4, np.uint16), out_depth=np.zeros(W * H, np.float32),
                       normal=np.zeros(W * H, np.uint32), material=np.zeros(W * H * 4, np.uint32))
        f = Frame(_p(out["proj_cache"]), _p(out["depth"]), _p(out["tile_counts"]), _p(out["tile_offsets"]),
                  _p(out["tile_entries"]), cap, _p(out["chunk_ranges"]), chunk_cap, 0, 0, 0, 0, 0, 0,
                  1 if f16 else 0,
                  _p(out.get("color")), _p(out.get("out_depth")), _p(out.get("normal")), _p(out.get("material")))
        rc = L.orc_render_frame(U.ctypes.data_as(c_void_p), ctypes.byref(scene), ctypes.byref(f), nt)
        if rc == -2:
            cap = max(cap, int(f.total_pairs) + 16)
            chunk_cap = max(chunk_cap, int(f.total_chunks) + 1)
            continue
        if rc != 0:
            raise RuntimeError(f"orc_render_frame failed ({rc})")
        break
    P = int(f.total_pairs)
    res = dict(
        proj_cache=out["proj_cache"][: N * 14].reshape(N, 14), depth=out["depth"][:N],
        tile_counts=out["tile_counts"], tile_offsets=out["tile_offsets"], tile_entries=out["tile_entries"][:P],
        chunk_ranges=out["chunk_ranges"][: 2 * f.total_chunks].reshape(-1, 2), total_pairs=P,
        small_tiles=int(f.small_tiles), hot_tiles=int(f.hot_tiles), total_chunks=int(f.total_chunks),
        large_splats=int(f.large_splats), flags=int(f.flags), M=M, W=W, H=H)
    if composite:
        res.update(color=out["color"].reshape(H, W, 4), out_depth=out["out_depth"].reshape(H, W),
                   normal=out["normal"].reshape(H, W), material=out["material"].reshape(H, W, 4))
    del keep
    return res


def sorted_keys20(U: np.ndarray, proj_cache: np.ndarray, depth: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    L = lib()
    U = np.ascontiguousarray(U, np.float32)
    N = int(_u32(U)[22])
    pc = np.ascontiguousarray(proj_cache, np.uint32).reshape(-1)
    d = np.ascontiguousarray(depth, np.uint32)
    total = c_uint64(0)
    cap = 16
    while True:
        keys = np.zeros(cap, np.uint64)
        vals = np.zeros(cap, np.uint32)
        rc = L.orc_sorted_keys20(U.ctypes.data_as(c_void_p), N, _p(pc), _p(d), _p(keys), _p(vals), cap,
                                 ctypes.byref(total))
        if rc == -2:
            cap = int(total.value) + 1
            continue
        if rc != 0:
            raise RuntimeError("orc_sorted_keys20 failed")
        return keys[: total.value], vals[: total.value]


def render_frame_f64(U, packed, sorted_indices, frame: dict, threads: int | None = None) -> np.ndarray:
    L = lib()
    U = np.ascontiguousarray(U, np.float32)
    W, H = int(U[16]), int(U[17])
    scene, keep = scene_struct(packed, sorted_indices)
    out = np.zeros(W * H * 4, np.float64)
    rc = L.orc_render_frame_f64(U.ctypes.data_as(c_void_p), ctypes.byref(scene), _p(frame["tile_counts"]),
                                _p(frame["tile_offsets"]), _p(np.ascontiguousarray(frame["tile_entries"])), _p(out),
                                threads or threads_default())
    del keep
    if rc != 0:
        raise RuntimeError("orc_render_frame_f64 failed")
    return out.reshape(H, W, 4)


def project_f64(U, packed, sorted_indices, threads: int | None = None) -> np.ndarray:
    """(N, 10) FP64 screen-space parameters per sortRank: cx, cy, ia, ib, ic,
    opacity, r, g, b, visible."""
    L = lib()
    U = np.ascontiguousarray(U, np.float32)
    scene, keep = scene_struct(packed, sorted_indices)
    n = int(packed.count)
    out = np.zeros((max(n, 1), 10), np.float64)
    L.orc_project_f64(U.ctypes.data_as(c_void_p), ctypes.byref(scene), _p(out), threads or threads_default())
    del keep
    return out[:n]


def sort_back_to_front(positions, view, threads: int = 1) -> np.ndarray:
    """splatSort.ts sortSplatIdsBackToFront; raises ValueError like the
    reference's RangeError on malformed input or a non-finite depth."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
    v = np.ascontiguousarray(view, np.float32).reshape(-1)
    if pos.size % 3 != 0:
        raise ValueError("positions length must be a multiple of 3")
    if v.size != 16:
        raise ValueError("view matrix must contain 16 values")
    n = pos.size // 3
    out = np.zeros(max(n, 1), np.uint32)
    rc = lib().orc_sort_back_to_front(_p(pos), n, _p(v), _p(out), threads)
    if rc == -1:
        raise ValueError("a splat produced a non-finite view-space depth")
    if rc != 0:
        raise RuntimeError("orc_sort_back_to_front failed")
    return out[:n]


def gpu_sort_prototype_order(positions, view) -> np.ndarray:
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
    v = np.ascontiguousarray(view, np.float32).reshape(-1)
    n = pos.size // 3
    out = np.zeros(max(n, 1), np.uint32)
    lib().orc_gpu_sort_prototype_order(_p(pos), n, _p(v), _p(out))
    return out[:n]


def _map(name, x, out_dtype, in_dtype=np.float32):
    x = np.ascontiguousarray(x, in_dtype).reshape(-1)
    out = np.zeros(x.size, out_dtype)
    getattr(lib(), name)(_p(x), _p(out), x.size)
    return out


def expf(x):
    return _map("orc_expf_n", x, np.float32)


def composite_expf(x):
    return _map("orc_composite_expf_n", x, np.float32)


def splat_expf(x):
    return _map("orc_splat_expf_n", x, np.float32)


def splat_exp_parts(x):
    """(p, kb) with splat_expf(x) = p * 2^k and kb = k << 23 (mod 2^32)."""
    a = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1))
    p = np.empty(a.size, np.float32)
    kb = np.empty(a.size, np.uint32)
    lib().orc_splat_exp_parts_n(a.ctypes.data, p.ctypes.data, kb.ctypes.data, a.size)
    return p, kb


def logf(x):
    return _map("orc_logf_n", x, np.float32)


def f16_rne(x):
    return _map("orc_f16_rne_n", x, np.uint16)


def f64_to_f16(x):
    return _map("orc_f64_to_f16_n", x, np.uint16, np.float64)


def f16_trunc(x):
    return _map("orc_f16_trunc_n", x, np.uint16)


def f16_to_f32(h):
    return _map("orc_f16_to_f32_n", h, np.float32, np.uint16)


def morton(x, y):
    x = np.ascontiguousarray(x, np.uint32)
    y = np.ascontiguousarray(y, np.uint32)
    out = np.zeros(x.size, np.uint32)
    lib().orc_morton_n(_p(x), _p(y), _p(out), x.size)
    return out


def bucket_key20(depth_bits, dmin: int, dmax: int):
    d = np.ascontiguousarray(depth_bits, np.uint32)
    b = np.zeros(d.size, np.uint32)
    k = np.zeros(d.size, np.uint32)
    lib().orc_bucket_key20_n(_p(d), d.size, dmin, dmax, _p(b), _p(k))
    return b, k


def plan(W, H, tile, N, mult=16.0) -> np.ndarray:
    out = np.zeros(9, np.uint32)
    lib().orc_plan(W, H, tile, N, mult, _p(out))
    return out


def frame_uniforms(plan_words, view_proj, splat_scale=1.0, sh_degree=0, camera_pos=None, view_matrix=None,
                   proj_matrix=None, normal_matrix=None) -> np.ndarray:
    """writeTileSplatFrameUniforms (gpuTileSplatCompositor.ts:730-774) over the
    9 words of plan(): the 64-float block, u32 fields stored as their bits.
    The focal terms are JS double products stored to f32 (:765-766)."""
    W, H, tile, cols, rows, _, _, N, budget = (int(x) for x in plan_words)
    t = np.zeros(64, np.float32)
    tu = t.view(np.uint32)
    t[0:16] = np.asarray(view_proj, np.float32).reshape(-1)
    t[16], t[17], t[18], t[19] = W, H, tile, 0.0
    tu[20], tu[21], tu[22], tu[23] = cols, rows, N, budget
    t[24] = splat_scale
    tu[25] = sh_degree
    if camera_pos is not None:
        t[28:31] = np.asarray(camera_pos, np.float32).reshape(-1)[:3]
    if view_matrix is not None:
        t[32:48] = np.asarray(view_matrix, np.float32).reshape(-1)
    if proj_matrix is not None:
        pm = np.asarray(proj_matrix, np.float32).reshape(-1)
        t[48] = np.float32(float(W) * float(pm[0]) * 0.5)
        t[49] = np.float32(float(H) * float(pm[5]) * 0.5)
    nm = [1, 0, 0, 0, 1, 0, 0, 0, 1] if normal_matrix is None else np.asarray(normal_matrix, np.float32).reshape(-1)
    for c in range(3):
        t[52 + 4 * c: 55 + 4 * c] = nm[3 * c: 3 * c + 3]
        t[55 + 4 * c] = 0.0
    return t


# ---------------------------------------------------------------------------
# deferred frame tail (hdsr_post_oracle.c)
# ---------------------------------------------------------------------------
class PostInputs(ctypes.Structure):
    _fields_ = [("W", c_int), ("H", c_int), ("color", c_void_p), ("depth", c_void_p), ("normal", c_void_p),
                ("material", c_void_p)]


class PostParams(ctypes.Structure):
    """orp_params: the field layout of hdsr_post_params."""

    _fields_ = [("view_proj_inverse", c_float * 16), ("camera_pos", c_float * 3), ("normal_recovery_mode", c_uint32),
                ("grazing_start", c_float), ("grazing_end", c_float), ("bilateral_spatial_sigma", c_float),
                ("bilateral_depth_sigma", c_float), ("bilateral_normal_sigma", c_float),
                ("bilateral_radius", c_uint32), ("proj", c_float * 16), ("view", c_float * 16),
                ("near_plane", c_float), ("far_plane", c_float), ("ao_radius_world", c_float),
                ("ao_falloff_end", c_float), ("ao_intensity", c_float), ("ao_thickness", c_float),
                ("ao_slices", c_uint32), ("ao_steps", c_uint32), ("frame_counter", c_uint32),
                ("ao_denoise_strength", c_float), ("bloom_threshold", c_float), ("bloom_soft_knee", c_float),
                ("light_dir", c_float * 3), ("light_intensity", c_float), ("ambient_intensity", c_float),
                ("specular_only", c_uint32), ("emissive_intensity", c_float), ("emissive_threshold", c_float),
                ("env_intensity", c_float), ("env_rotation", c_float), ("exposure", c_float),
                ("fallback_roughness", c_float), ("fallback_metallic", c_float)]


class PostEnv(ctypes.Structure):
    _fields_ = [("texels", c_void_p), ("w", c_int), ("h", c_int), ("levels", c_int), ("lw", c_int * 16),
                ("lh", c_int * 16), ("offset", c_uint32 * 16)]


_post_ready = False


def _post_lib():
    global _post_ready
    L = lib()
    if not _post_ready:
        vp = c_void_p
        for nm, args in (("orp_ss_normals", [vp, vp, vp]), ("orp_bilateral", [vp, vp, vp, vp]),
                         ("orp_gtao_prefilter", [vp, vp, vp, vp, vp]),
                         ("orp_gtao_main", [vp, vp, vp, vp, vp, vp, vp]),
                         ("orp_gtao_denoise", [vp, vp, vp, vp, vp]), ("orp_bloom_threshold", [vp, vp, vp]),
                         ("orp_bloom_blur", [c_int, c_int, vp, vp, c_float, c_float, c_float, c_float]),
                         ("orp_lighting", [vp, vp, vp, vp, vp, vp, vp, vp, vp]),
                         ("orp_brdf_lut", [c_int, c_int, vp]), ("orp_env_mip", [vp, c_int, c_int, vp, c_int, c_int]),
                         ("orp_curve_lut", [c_float, c_float, c_float, vp])):
            getattr(L, nm).argtypes = args
            getattr(L, nm).restype = None
        for nm in ("orp_asin", "orp_sin", "orp_cos", "orp_log2"):
            getattr(L, nm).argtypes = [c_float]
            getattr(L, nm).restype = c_float
        for nm in ("orp_atan2", "orp_pow", "orp_weight_pow"):
            getattr(L, nm).argtypes = [c_float, c_float]
            getattr(L, nm).restype = c_float
        _post_ready = True
    return L


def post_inputs(color, depth, normal, material):
    """(orp_inputs, keepalive) over host copies of the compositor's output images."""
    keep = dict(color=np.ascontiguousarray(color, np.float32), depth=np.ascontiguousarray(depth, np.float32),
                normal=np.ascontiguousarray(normal).view(np.uint32),
                material=np.ascontiguousarray(material).view(np.uint32))
    H, W = keep["depth"].shape
    s = PostInputs(W, H, _p(keep["color"]), _p(keep["depth"]), _p(keep["normal"]), _p(keep["material"]))
    return s, keep


def _addr(q):
    return ctypes.addressof(q)


def post_ss_normals(inp, params) -> np.ndarray:
    out = np.zeros((inp.H, inp.W), np.uint32)
    _post_lib().orp_ss_normals(ctypes.addressof(inp), _addr(params), _p(out))
    return out


def post_bilateral(inp, params, ssn) -> np.ndarray:
    ssn = np.ascontiguousarray(ssn).view(np.uint32)
    out = np.zeros((inp.H, inp.W), np.uint32)
    _post_lib().orp_bilateral(ctypes.addressof(inp), _addr(params), _p(ssn), _p(out))
    return out


def post_gtao_prefilter(inp, params):
    W, H = inp.W, inp.H
    m0 = np.zeros((H, W), np.float32)
    m1 = np.zeros(((H + 1) // 2, (W + 1) // 2), np.float32)
    m2 = np.zeros(((H + 3) // 4, (W + 3) // 4), np.float32)
    _post_lib().orp_gtao_prefilter(ctypes.addressof(inp), _addr(params), _p(m0), _p(m1), _p(m2))
    return m0, m1, m2


def post_gtao_main(inp, params, mips, normals) -> np.ndarray:
    m0, m1, m2 = (np.ascontiguousarray(m, np.float32) for m in mips)
    nrm = np.ascontiguousarray(normals).view(np.uint32)
    out = np.zeros((inp.H, inp.W, 4), np.uint16)
    _post_lib().orp_gtao_main(ctypes.addressof(inp), _addr(params), _p(m0), _p(m1), _p(m2), _p(nrm), _p(out))
    return out


def post_gtao_denoise(inp, params, ao_raw, mip0) -> np.ndarray:
    a = np.ascontiguousarray(ao_raw).view(np.uint16)
    m0 = np.ascontiguousarray(mip0, np.float32)
    out = np.zeros((inp.H, inp.W, 4), np.uint16)
    _post_lib().orp_gtao_denoise(ctypes.addressof(inp), _addr(params), _p(a), _p(m0), _p(out))
    return out


def post_bloom_threshold(inp, params) -> np.ndarray:
    out = np.zeros(((inp.H + 1) // 2, (inp.W + 1) // 2, 4), np.uint16)
    _post_lib().orp_bloom_threshold(ctypes.addressof(inp), _addr(params), _p(out))
    return out


def post_bloom_blur(src, dirx: float, diry: float, tx: float, ty: float) -> np.ndarray:
    s = np.ascontiguousarray(src).view(np.uint16)
    hh, hw = s.shape[:2]
    out = np.zeros_like(s)
    _post_lib().orp_bloom_blur(hw, hh, _p(s), _p(out), dirx, diry, tx, ty)
    return out


def post_env_chain(level0) -> dict:
    """ibl_mipgen.wgsl chain over level 0 (h, w, 4) rgba16f bits; the PostEnv fields."""
    L = _post_lib()
    l0 = np.ascontiguousarray(level0).view(np.uint16)
    h, w = l0.shape[:2]
    levels = 1
    while (max(w, h) >> levels) > 0:
        levels += 1
    dims = [(max(1, w >> k), max(1, h >> k)) for k in range(levels)]
    offs = np.cumsum([0] + [a * b for a, b in dims])
    tex = np.zeros((int(offs[-1]), 4), np.uint16)
    tex[: w * h] = l0.reshape(-1, 4)
    for k in range(1, levels):
        (sw, sh), (dw, dh) = dims[k - 1], dims[k]
        src = np.ascontiguousarray(tex[offs[k - 1]:offs[k]])
        dst = np.zeros((dh * dw, 4), np.uint16)
        L.orp_env_mip(_p(src), sw, sh, _p(dst), dw, dh)
        tex[offs[k]:offs[k + 1]] = dst
    return dict(texels=tex, w=w, h=h, levels=levels, dims=dims, offsets=[int(o) for o in offs[:-1]])


def placeholder_env() -> dict:
    return dict(texels=np.full((1, 4), 0x3C00, np.uint16), w=1, h=1, levels=1, dims=[(1, 1)], offsets=[0])


def _env_struct(env: dict):
    e = PostEnv(_p(env["texels"]), env["w"], env["h"], env["levels"])
    for k in range(16):
        lw, lh = env["dims"][k] if k < env["levels"] else (1, 1)
        e.lw[k], e.lh[k] = lw, lh
        e.offset[k] = env["offsets"][k] if k < env["levels"] else 0
    return e


def post_lighting(inp, params, normals, ao, env: dict, brdf, bloom, curves) -> np.ndarray:
    keep = [np.ascontiguousarray(normals).view(np.uint32), np.ascontiguousarray(ao).view(np.uint16),
            np.ascontiguousarray(brdf).view(np.uint32), np.ascontiguousarray(bloom).view(np.uint16),
            np.ascontiguousarray(curves).view(np.uint16)]
    e = _env_struct(env)
    out = np.zeros((inp.H, inp.W, 4), np.uint16)
    _post_lib().orp_lighting(ctypes.addressof(inp), _addr(params), _p(keep[0]), _p(keep[1]), ctypes.addressof(e),
                             _p(keep[2]), _p(keep[3]), _p(keep[4]), _p(out))
    return out


def post_brdf_lut(y0: int = 0, y1: int = 256) -> np.ndarray:
    out = np.zeros((256, 256), np.uint32)
    _post_lib().orp_brdf_lut(y0, y1, _p(out))
    return out


def post_curve_lut(contrast: float, brightness: float, gamma: float) -> np.ndarray:
    out = np.zeros(256, np.uint16)
    _post_lib().orp_curve_lut(contrast, brightness, gamma, _p(out))
    return out


def post_math(name: str, *args) -> float:
    return float(getattr(_post_lib(), "orp_" + name)(*[float(a) for a in args]))
