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
CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]

FLAG_LARGE_SPLAT_CAP = 1
FLAG_REF_BUDGET_DROP = 2
FLAG_OVERFLOW_SKIP = 4
FLAG_CHUNK_CAP = 8
FLAG_BUCKET_KEY_MISMATCH = 16


def build(force: bool = False) -> Path:
    """gcc recipe for liboracle.so (no -march flags: identical on x86 and Arm)."""
    deps = [SRC, HERE / "hdsr_oracle.h"]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        cc = os.environ.get("CC", "gcc")
        subprocess.run([cc, *CFLAGS, str(SRC), "-o", str(LIB), "-lm"], check=True)
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
                ("large_splats", c_uint32), ("flags", c_uint32), ("_pad", c_uint32), ("out_color", c_void_p),
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
        for nm in ("orc_expf_n", "orc_logf_n", "orc_f16_rne_n", "orc_f16_trunc_n", "orc_f16_to_f32_n"):
            getattr(L, nm).argtypes = [c_void_p, c_void_p, c_uint64]
        L.orc_morton_n.argtypes = [c_void_p, c_void_p, c_void_p, c_uint64]
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
                 cap: int | None = None) -> dict:
    """Full canonical frame: cache, counts, offsets, per-tile order, outputs.
    `cap` is the initial entry capacity (grown and retried when too small)."""
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
                  _p(out["tile_entries"]), cap, _p(out["chunk_ranges"]), chunk_cap, 0, 0, 0, 0, 0, 0, 0,
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


def logf(x):
    return _map("orc_logf_n", x, np.float32)


def f16_rne(x):
    return _map("orc_f16_rne_n", x, np.uint16)


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
