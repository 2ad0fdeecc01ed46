#!/usr/bin/env python
"""Benchmark of the GB300 tile-splat compositor.

Headline: frames/s of the 760k-splat 1920x1080 hot-tile workload (seeded
synthetic scene; see the package's workloads module), one full frame per
step: projection, tile counting, scans, key emission, radix sort, per-tile
sort with the hot-tile cascade, rasteriser.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value   frames/s with the scene resident in HBM; each step is timed with CUDA
        events on the launching stream and a 256 MiB buffer is written between
        steps to flush the 129 MB L2 (the flush is outside the timed events).
e2e     the same frames/s through the C ABI with host buffers: every step
        copies the scene from pinned host memory to the device, encodes the
        frame and copies the four output images back.
--impl reference  times the reference's CPU path restated in C (the oracle;
        the reference itself is TypeScript/WGSL and cannot run here) on the
        same workload with all host threads, one full frame per step, stopping
        after 120 s of frames (steps_run says how many ran).
N > 1   runs N independent replicas (one per GPU); value = frames of all ranks
        / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

METRIC = "760k-splat 1080p frames/s"


def metric_name(wl) -> str:
    """The headline metric for the default workload; for another workload the
    same form with its own splat count and height."""
    if wl.scene.count == 760_000 and (wl.width, wl.height) == (1920, 1080):
        return METRIC
    return f"{round(wl.scene.count / 1000)}k-splat {wl.height}p frames/s"
REFERENCE_TIME_CAP_S = 120.0
UNIT = "frames/s"


def log(msg: str) -> None:
    """Progress on stderr (stdout carries the one JSON line)."""
    print(f"[bench] {msg}", file=sys.stderr, flush=True)


def slowest_rank_seconds(seconds: float, world: int, device) -> float:
    """The timed region of the slowest rank (MAX all-reduce; one rank: itself)."""
    if world <= 1:
        return seconds
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replicas_value(steps: int, world: int, slowest_s: float) -> float:
    """Frames of all replicas per second of the slowest replica (weak scaling)."""
    return steps * world / slowest_s


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, sampled every 20 ms from before the
    warm-up until after the timed loop; summary(t0, t1) keeps the samples that
    arrived during the timed region [t0, t1] (host clock), or, when the region
    is shorter than the sampling interval, the first sample after t0."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float | None = None, t1: float | None = None) -> dict:
        rows = [r for t, r in self.rows if t0 is None or t0 <= t <= t1]
        window = "timed region"
        if not rows and t0 is not None:
            after = [r for t, r in self.rows if t >= t0]
            rows, window = after[:1], "first sample after the timed region began"
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "window": window}


def setup_frame(pkg, wl, device_index=0):
    """Packed scene, plan, uniforms, bound compositor sized to the frame."""
    import torch

    scene = wl.scene
    cam = wl.cameras[0]
    packed = pkg.splats.pack_splat_attributes(scene)
    plan = pkg.plan_tile_splat_compositor(wl.width, wl.height, 16, scene.count)
    u, fr = pkg.frame_uniforms_for(plan, cam, sh_degree=scene.sh_degree)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    bufs = pkg.splats.upload_splat_attribute_buffers(packed, order, device=f"cuda:{device_index}")
    color, gb = pkg.create_output_textures(plan, device=f"cuda:{device_index}")
    res = pkg.create_tile_splat_compositor(plan)
    pkg.create_tile_splat_bind_groups(res, bufs, color, gb)
    pkg.write_frame_uniform_buffer(res, u)
    pkg.encode_full_compute_compositor_pipeline(None, res)
    st = res.query_status()
    if st["status"] == pkg._lib.HDSR_ERR_OVERFLOW:
        # the reference grows its tile-entry budget from a readback of the
        # frame's needs (gpuTileSplatCompositor.ts:123-126); size it exactly
        need = int(st["total_pairs"])
        res.destroy()
        res = pkg.create_tile_splat_compositor(plan, pair_capacity=int(need * 1.02) + 1024)
        pkg.create_tile_splat_bind_groups(res, bufs, color, gb)
        pkg.write_frame_uniform_buffer(res, u)
        pkg.encode_full_compute_compositor_pipeline(None, res)
        st = res.check_frame()
    torch.cuda.synchronize()
    return dict(packed=packed, plan=plan, u=u, order=order, bufs=bufs, color=color, gb=gb, res=res, stats=st)


def pass_bytes(name: str, N: int, P: int, Q: int, S: int, sh_floats: int, depth_passes: int = 4) -> float | None:
    """Algorithmic HBM bytes of one pass of the frame (None: not HBM-bound).

    N splats, P (tile, splat) pairs, Q superblock list entries, S segments,
    depth_passes the 9-bit passes the depth sort ran this frame."""
    if name == "project":
        # indices, position, scale, rotation, opacity, material, SH in; geo,
        # app, gb, aux, depth, ntiles, nsb, depth key out
        return N * (4 + 12 + 12 + 16 + 4 + 4 + 4 * sh_floats + 16 + 16 + 16 + 8 + 4 + 4 + 4 + 8)
    if name == "tile_counts":
        return N * 8  # tile boxes
    if name == "depth_sort":
        # the first histogram reads the keys; every pass reads them, the last
        # writes the 4-byte order words, the others the 8-byte keys
        return N * 8 + depth_passes * N * 8 + (depth_passes - 1) * N * 8 + N * 4
    if name == "superblock_lists":
        # scan: depth-order words (counts ride in them) and gathered tile boxes
        # in, offsets and Q keys out; one radix pass: Q keys read twice, written once
        return N * 4 + N * 8 + N * 4 + Q * 8 + Q * 24
    if name == "tile_entries":
        # count and scatter read the Q keys; segment tables 3x; P entries out
        return Q * 16 + S * 256 * 3 + P * 4
    if name == "chunk_masks":
        # the Q sorted list keys in, one 8-byte tile mask per 32 keys out
        return Q * 8 + (Q + 31) // 32 * 8
    return None


def run_train(pkg, args, dev) -> dict:
    """fwd+bwd iterations/s on the training workload (500k splats, SH 1,
    1024x1024) against plain forward frames/s on the same scene.

    One iteration: hdsr_encode_full, the L2 loss gradient against a fixed
    target (a torch elementwise kernel), hdsr_encode_backward. The target is
    the frame of the scene with means + N(0, 0.01) and colours + N(0, 0.05).
    Timed with CUDA events over K iterations, no host synchronisation inside."""
    import torch

    wl = pkg.workloads.train500k()
    n = wl.scene.count
    packed = pkg.splats.pack_splat_attributes(wl.scene)
    rng = np.random.default_rng(17)
    plan = pkg.plan_tile_splat_compositor(wl.width, wl.height, 16, n)
    u, fr = pkg.frame_uniforms_for(plan, wl.cameras[0], sh_degree=wl.scene.sh_degree)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    r = pkg.differentiable.SplatFrameRenderer(wl.width, wl.height, n, sh_degree=wl.scene.sh_degree, device=dev)

    def t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    pos, lsc, rot = t(packed.positions.reshape(n, 3)), t(packed.scales.reshape(n, 3)), t(packed.rotations.reshape(n, 4))
    opa, sh = t(packed.opacities.reshape(n)), t(packed.sh_data.reshape(n, -1))
    srt = t(np.asarray(order, np.uint32).view(np.int32))
    tpos = pos + t(rng.normal(0.0, 0.01, (n, 3)).astype(np.float32))
    tsh = sh.clone()
    tsh[:, :3] += t(rng.normal(0.0, 0.05, (n, 3)).astype(np.float32))
    target = r.forward_frame(tpos, lsc, rot, opa, tsh, srt, u).clone()
    r.forward_frame(pos, lsc, rot, opa, sh, srt, u)  # sizes the pair capacity, binds the scene
    res = r.res
    grads = {"positions": torch.empty_like(pos), "log_scales": torch.empty_like(lsc),
             "rotations": torch.empty_like(rot), "opacities": torch.empty_like(opa), "sh": torch.empty_like(sh)}
    d_color = torch.empty_like(target)
    scale = 2.0 / target.numel()
    stream = torch.cuda.current_stream()

    def fwd():
        pkg.encode_full_compute_compositor_pipeline(stream, res)

    def it():
        fwd()
        torch.sub(r.color, target, out=d_color)
        d_color.mul_(scale)
        pkg.encode_backward(stream, res, d_color, grads)

    def timed(fn, k):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(k):
            fn()
        e.record(stream)
        e.synchronize()
        return s.elapsed_time(e) / k

    k = max(args.steps, 5)
    fwd_ms = timed(fwd, k)
    it_ms = timed(it, k)
    st = res.check_frame()
    loss = float(((r.color - target) ** 2).mean())
    ok = all(bool(torch.isfinite(g).all()) for g in grads.values())
    r.destroy()
    return {"workload": "train500k_1024x1024", "splats": n, "sh_degree": wl.scene.sh_degree,
            "pairs": int(st["total_pairs"]), "fwd_bwd_it_per_s": round(1000.0 / it_ms, 2),
            "fwd_frames_per_s": round(1000.0 / fwd_ms, 2), "fwd_bwd_ms": round(it_ms, 4),
            "fwd_ms": round(fwd_ms, 4), "bwd_over_fwd": round((it_ms - fwd_ms) / fwd_ms, 3),
            "loss": loss, "grads_finite": ok, "timing": "CUDA events, K iterations back to back"}


def run_sh3_orbit(pkg, args, dev, peak: float) -> dict:
    """3M Gaussians, SH degree 3, 3840x2160, 8-camera orbit at radius 6.

    The scene is resident; every view sorts the splats back to front on the
    device (hdsr_sort_back_to_front into the bound sortedIndices), uploads its
    uniform block and renders a full frame, all on one stream. Timed: whole
    orbits with CUDA events (inputs far larger than L2). Then, per view, the
    image against the oracle's FP64 twin over the frame's own entry lists
    (max |err| and PSNR), and per-pass times (profiled) with the projection's
    fraction of measured HBM bandwidth (SH3 makes it read ~260 B per splat)."""
    import oracle
    import torch

    wl = pkg.workloads.sh3_3m()
    n = wl.scene.count
    packed = pkg.splats.pack_splat_attributes(wl.scene)
    plan = pkg.plan_tile_splat_compositor(wl.width, wl.height, 16, n)
    bufs = pkg.splats.upload_splat_attribute_buffers(packed, np.arange(n, dtype=np.uint32), device=dev)
    color, gb = pkg.create_output_textures(plan, device=dev)
    frames = [c.frame(wl.width, wl.height) for c in wl.cameras]
    views = [np.asarray(fr["view"], np.float32).reshape(-1) for fr in frames]
    us = [pkg.frame_uniforms_for(plan, c, sh_degree=3)[0] for c in wl.cameras]
    stream = torch.cuda.current_stream()
    res = pkg.create_tile_splat_compositor(plan, pair_capacity=600_000_000)
    pkg.create_tile_splat_bind_groups(res, bufs, color, gb)

    def view(i):
        pkg.sort_back_to_front(stream, res, views[i], bufs["sorted_indices"])
        pkg.write_frame_uniform_buffer(res, us[i])
        pkg.encode_full_compute_compositor_pipeline(stream, res)

    pairs = []
    for i in range(len(views)):  # size the pair capacity on the orbit itself
        view(i)
        st = res.query_status()
        pairs.append(int(st["total_pairs"]))
    if max(pairs) > res.pair_capacity:
        res.destroy()
        res = pkg.create_tile_splat_compositor(plan, pair_capacity=int(max(pairs) * 1.02) + 1024)
        pkg.create_tile_splat_bind_groups(res, bufs, color, gb)
    for _ in range(max(args.warmup, 3)):
        for i in range(len(views)):
            view(i)
    torch.cuda.synchronize()
    orbits = max(1, min(args.steps, 20))
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(orbits):
        for i in range(len(views)):
            view(i)
    e.record(stream)
    e.synchronize()
    view_ms = s.elapsed_time(e) / (orbits * len(views))
    st = res.check_frame()
    s.record(stream)
    for _ in range(orbits):
        for i in range(len(views)):
            pkg.sort_back_to_front(stream, res, views[i], bufs["sorted_indices"])
    e.record(stream)
    e.synchronize()
    sort_ms = s.elapsed_time(e) / (orbits * len(views))
    # per pass (profiled: one stream, direct launches), mean over the views
    res.set_profiling(True)
    passes = {}
    stats = []
    for i in range(len(views)):
        view(i)
        stats.append(res.check_frame())
        for name, ms in res.pass_times():
            passes.setdefault(name, []).append(ms)
    res.set_profiling(False)
    mean_pass = {k: statistics.mean(v) for k, v in passes.items()}
    proj_b = pass_bytes("project", n, 0, 0, 0, 6 + 3 * 15)
    proj_ach = proj_b / (mean_pass["project"] / 1000.0) / 1e9
    # accuracy per view against the FP64 twin, over the GPU frame's entries
    per_view = []
    for i in range(len(views)):
        view(i)
        st_i = res.check_frame()
        P = int(st_i["total_pairs"])
        order = bufs["sorted_indices"].cpu().numpy().view(np.uint32)
        fr_lists = dict(tile_counts=res.buffer("tile_counts").cpu().numpy().view(np.uint32),
                        tile_offsets=res.buffer("tile_offsets").cpu().numpy().view(np.uint32),
                        tile_entries=res.buffer("tile_entries", count=P).cpu().numpy().view(np.uint32))
        f64 = oracle.render_frame_f64(us[i], packed, order, fr_lists)
        got = color.cpu().numpy().astype(np.float64)
        err = float(np.abs(got - f64).max())
        mse = float(np.mean((got[..., :3] - f64[..., :3]) ** 2))
        per_view.append({"view": i, "pairs": P, "hot_tiles": int(st_i["hot_tiles"]), "max_abs_err_vs_fp64": err,
                         "psnr_db_vs_fp64": round(10.0 * np.log10(1.0 / max(mse, 1e-30)), 2)})
        del fr_lists, f64, got
    res.destroy()
    return {"workload": wl.name, "splats": n, "sh_degree": 3, "width": wl.width, "height": wl.height,
            "cameras": len(views), "orbits_timed": orbits, "ms_per_view": round(view_ms, 4),
            "frames_per_s": round(1000.0 / view_ms, 2), "device_sort_ms_per_view": round(sort_ms, 4),
            "frame_ms_per_view": round(view_ms - sort_ms, 4),
            "timing": "CUDA events over whole orbits; each view = device back-to-front sort + uniform upload + "
                      "full frame; inputs (3M splats, 0.9 GB) far larger than L2",
            "passes_ms": {k: round(v, 4) for k, v in mean_pass.items()},
            "project_roofline": {"bound": "hbm", "algorithmic_bytes": int(proj_b),
                                 "achieved": round(proj_ach, 1), "peak": peak, "unit": "GB/s",
                                 "frac": round(proj_ach / peak, 4)},
            "per_view": per_view,
            "fp64_note": "FP64 twin of the oracle (double projection, SH and composite over the same entry "
                         "lists, no f16 rounding) against the f16 output image"}


SERVE_RESOLUTIONS = [(512, 512), (1280, 720), (1920, 1080)]


def run_serve(pkg, args, dev) -> dict:
    """Serving: 8 resident scenes (N log-uniform in [100k, 3M], the hot-tile
    distribution, SH 0), 2,000 requests of a random scene, random orbit
    camera and a resolution of {512x512, 1280x720, 1920x1080}, 120 GB budget.

    plain: the per-frame path, one request at a time (encode, then read the
    frame status: one host round trip per frame), one handle per
    (scene, resolution). server: hdsr_server_* with every request queued at
    once (saturated throughput), then Poisson arrivals at 70% of that rate
    for p50/p99 latency (submit to completion on the device, host clock).
    Every key is rendered once before timing (slots sized, graphs captured)."""
    import torch

    rng = np.random.default_rng(41)
    n_req = 2000
    ns = np.exp(rng.uniform(np.log(1e5), np.log(3e6), 8)).astype(int)
    scenes = {}
    for sid, n in enumerate(ns):
        sc = pkg.workloads.hot_scene(int(n), 100 + sid)
        packed = pkg.splats.pack_splat_attributes(sc)
        bufs = pkg.splats.upload_splat_attribute_buffers(packed, np.arange(sc.count, dtype=np.uint32), device=dev)
        scenes[sid] = (sc, bufs)
    reqs = []
    for _ in range(n_req):
        sid = int(rng.integers(0, 8))
        W, H = SERVE_RESOLUTIONS[int(rng.integers(0, 3))]
        cam = pkg.camera.OrbitCamera(azimuth=float(rng.uniform(0, 2 * np.pi)), elevation=float(rng.uniform(-0.5, 0.5)),
                                     distance=float(rng.uniform(4.0, 9.0)))
        plan = pkg.plan_tile_splat_compositor(W, H, 16, scenes[sid][0].count)
        u, _ = pkg.frame_uniforms_for(plan, cam)
        reqs.append((sid, W, H, u))
    ring = 32  # output image sets per resolution, reused in submission order
    outs = {r: [pkg.create_output_textures(pkg.plan_tile_splat_compositor(r[0], r[1], 16, 1), device=dev)
                for _ in range(ring)] for r in SERVE_RESOLUTIONS}
    keys = sorted({(sid, W, H) for sid, W, H, _ in reqs})

    # plain per-frame path
    handles = {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    device_ms = [0.0]

    def plain(sid, W, H, u, out):
        sc, bufs = scenes[sid]
        res = handles.get((sid, W, H))
        if res is None:
            res = pkg.create_tile_splat_compositor(pkg.plan_tile_splat_compositor(W, H, 16, sc.count))
            handles[(sid, W, H)] = res
        pkg.create_tile_splat_bind_groups(res, bufs, out[0], out[1])
        pkg.write_frame_uniform_buffer(res, u)
        ev0.record()
        pkg.encode_full_compute_compositor_pipeline(None, res)
        ev1.record()
        st = res.query_status()
        device_ms[0] += ev0.elapsed_time(ev1)
        if st["status"] == pkg._lib.HDSR_ERR_OVERFLOW:
            need = int(st["total_pairs"])
            res.destroy()
            res = pkg.create_tile_splat_compositor(pkg.plan_tile_splat_compositor(W, H, 16, sc.count),
                                                   pair_capacity=need + need // 4 + 4096)
            handles[(sid, W, H)] = res
            return plain(sid, W, H, u, out)
        return st

    log("serving: scenes resident, plain path sizing")
    for sid, W, H, u in reqs:  # size every handle on the requests themselves
        plain(sid, W, H, u, outs[(W, H)][0])
    torch.cuda.synchronize()
    device_ms[0] = 0.0
    t0 = time.perf_counter()
    for i, (sid, W, H, u) in enumerate(reqs):
        plain(sid, W, H, u, outs[(W, H)][i % ring])
    plain_s = time.perf_counter() - t0
    plain_device_s = device_ms[0] / 1000.0
    # the plain path per key (sequential frames of one key, the same handle)
    key_plain = {}
    for key in keys:
        cams = [q[3] for q in reqs if q[:3] == key][:8]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for j, u in enumerate(cams):
            plain(key[0], key[1], key[2], u, outs[(key[1], key[2])][j])
        key_plain[key] = ((time.perf_counter() - t1) / len(cams), cams)
    for res in handles.values():
        res.destroy()
    handles.clear()
    torch.cuda.synchronize()

    log(f"serving: plain path {n_req / plain_s:.1f} frames/s; server warm-up")
    in_flight = 12
    server = pkg.serving.Server(hbm_budget_bytes=120 << 30, max_in_flight=in_flight)
    for sid, (_, bufs) in scenes.items():
        server.add_scene(sid, bufs)

    def run_batch(arrivals=None):
        tickets, lat = [], []
        used = {r: [None] * ring for r in SERVE_RESOLUTIONS}
        t_start = time.perf_counter()
        results = []
        for i, (sid, W, H, u) in enumerate(reqs):
            slot = used[(W, H)]
            if slot[i % ring] is not None:  # the output set is reused: its frame must be done
                results.append(server.wait(slot[i % ring]))
                slot[i % ring] = None
            if arrivals is not None:
                while time.perf_counter() - t_start < arrivals[i]:
                    pass
            color, gb = outs[(W, H)][i % ring]
            slot[i % ring] = server.submit(sid, u, color, gb)
        for r in SERVE_RESOLUTIONS:
            for t in used[r]:
                if t is not None:
                    results.append(server.wait(t))
        return time.perf_counter() - t_start, results

    for rep in range(3):  # warm: every key's slots sized (rep 0), several at once, graphs captured
        for sid, W, H in keys:
            cams = [q[3] for q in reqs if q[:3] == (sid, W, H)][:3]
            tickets = []
            for j, u in enumerate(cams if rep else cams[:1]):
                color, gb = outs[(W, H)][j]
                tickets.append(server.submit(sid, u, color, gb))
            for t in tickets:
                server.wait(t)
    # concurrency ceiling per key: the same key's frames all queued at once
    # (as many slots as max_in_flight) against its sequential plain frames;
    # frames of one key overlap at least as well as a mixed batch can, so the
    # mix's speedup is bounded by sum(plain) / sum(homogeneous) over its
    # requests' keys
    key_served = {}
    for key, (t_plain, cams) in key_plain.items():
        for rep in range(2):  # the first round sizes the key's extra slots; the second is timed
            tickets = []
            t1 = time.perf_counter()
            for j, u in enumerate(cams):
                color, gb = outs[(key[1], key[2])][j]
                tickets.append(server.submit(key[0], u, color, gb))
            for t in tickets:
                server.wait(t)
            key_served[key] = (time.perf_counter() - t1) / len(cams)
    ceil_plain = sum(key_plain[q[:3]][0] for q in reqs)
    ceil_served = sum(key_served[q[:3]] for q in reqs)
    log("serving: saturated run")
    sat_s, sat_res = run_batch()
    log(f"serving: {n_req / sat_s:.1f} frames/s saturated; Poisson run")
    rate = 0.7 * n_req / sat_s
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    _, lat_res = run_batch(arrivals)
    lat = np.array([r["done_ms"] - r["submit_ms"] for r in lat_res])
    st = server.stats()
    bad = sum(1 for r in sat_res + lat_res if r["status"] != 0)
    server.destroy()
    return {"workload": "serve8_mixed", "scene_splats": [int(x) for x in ns], "requests": n_req,
            "resolutions": [f"{w}x{h}" for w, h in SERVE_RESOLUTIONS], "budget_gb": 120,
            "plain_frames_per_s": round(n_req / plain_s, 1), "server_frames_per_s": round(n_req / sat_s, 1),
            "speedup_vs_plain": round(plain_s / sat_s, 2), "offered_rps": round(rate, 1),
            "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "slots": st["slots"], "graphs": st["graphs"], "evictions": st["evictions"], "reruns": st["reruns"],
            "slot_gb": round(st["slot_bytes"] / 2 ** 30, 2), "failed": bad, "max_in_flight": in_flight,
            "plain_device_busy": round(plain_device_s / plain_s, 3),
            "plain_device_ms_per_frame": round(plain_device_s * 1000.0 / n_req, 4),
            "homogeneous_speedup_by_resolution": {
                f"{w}x{h}": round(sum(key_plain[k][0] for k in keys if k[1:] == (w, h)) /
                                  sum(key_served[k] for k in keys if k[1:] == (w, h)), 2) for w, h in SERVE_RESOLUTIONS},
            "speedup_ceiling_from_homogeneous": round(ceil_plain / ceil_served, 2),
            "ceiling_note": "frames of each (scene, viewport) key queued all at once through the server against the "
                            "same frames one by one on the plain path (8 per key); the mix's bound is the sum of "
                            "the per-key plain times over its requests divided by the sum of the per-key served "
                            "times"}


def run_ours(args, rank, world, local):
    import torch

    pkg = __graft_entry__.load_package()
    pkg._build.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl = pkg.workloads.WORKLOADS[args.workload]()
    F = setup_frame(pkg, wl, local)
    res, plan = F["res"], F["plan"]
    N, P = plan.splat_count, int(F["stats"]["total_pairs"])
    # every leg runs on a stream of its own: hdsr_encode_full replays a full
    # frame as a CUDA graph on any stream but the legacy default one
    torch.cuda.set_stream(torch.cuda.Stream(device=dev))
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def frame():
        pkg.encode_full_compute_compositor_pipeline(stream, res)

    clocks = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = res.launch_count()
    times = []
    t_begin = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        frame()
        e.record(stream)
        e.synchronize()
        times.append(s.elapsed_time(e))
    torch.cuda.synchronize()
    t_end = time.perf_counter()
    time.sleep(0.15)  # let the sample taken during the region arrive
    clocks.__exit__(None, None, None)
    launches = res.launch_count() - launches0
    st = res.check_frame()
    # per-pass times: the same frames again with profiling events (one stream)
    res.set_profiling(True)
    passes = {}
    for _ in range(args.steps):
        flush.zero_()
        frame()
        for name, ms in res.pass_times():
            passes.setdefault(name, []).append(ms)
    res.set_profiling(False)
    total_s = slowest_rank_seconds(sum(times) / 1000.0, world, dev)
    value = replicas_value(args.steps, world, total_s)
    # sortedIndices on the device for the same camera (the reference sorts on
    # the host: cpu_baseline's cpu_depth_sort_ms)
    sorted_tmp = torch.empty(N, dtype=torch.int32, device=dev)
    view = np.asarray(wl.cameras[0].frame(wl.width, wl.height)["view"], np.float32).reshape(-1)
    for _ in range(3):
        pkg.sort_back_to_front(stream, res, view, sorted_tmp)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(args.steps):
        pkg.sort_back_to_front(stream, res, view, sorted_tmp)
    e.record(stream)
    e.synchronize()
    sort_ms = s.elapsed_time(e) / args.steps
    # a static camera: composite only (encodeCompositeOnly) over the last full
    # frame's lists, the reference's cheap-frame path (gpuTileSplatCompositor.ts:1001-1014)
    for _ in range(3):
        pkg.encode_composite_only(stream, res)
    s.record(stream)
    for _ in range(args.steps):
        pkg.encode_composite_only(stream, res)
    e.record(stream)
    e.synchronize()
    composite_only_ms = s.elapsed_time(e) / args.steps

    # end to end through the C ABI with host buffers
    log(f"frames timed: {value:.1f} frames/s")
    e2e = None if args.no_e2e else run_e2e(pkg, F, args, stream, world, dev)
    moving = None if args.no_moving else run_moving_camera(pkg, F, wl, args, stream)

    # roofline of the dominant HBM-bound pass
    sh_floats = 6 + 3 * ((wl.scene.sh_degree + 1) ** 2 - 1)
    mean_pass = {k: statistics.mean(v) for k, v in passes.items()}
    frame_ms = statistics.mean(times)
    Q, S, DP = int(st["superblock_entries"]), int(st["segments"]), int(st["depth_sort_passes"])
    hbm_passes = {k: v for k, v in mean_pass.items() if pass_bytes(k, N, P, Q, S, sh_floats, DP)}
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    dom = max(hbm_passes, key=hbm_passes.get) if hbm_passes else None
    # every HBM-accounted pass against the measured copy bandwidth (the
    # committed ncu traffic table is of the default workload only)
    roofline_passes = {}
    for k in hbm_passes:
        b = pass_bytes(k, N, P, Q, S, sh_floats, DP)
        ach = b / (mean_pass[k] / 1000.0) / 1e9
        roofline_passes[k] = {"bound": "hbm", "kernel": k, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                              "frac": round(ach / peak, 4),
                              "traffic": load_traffic(k) if args.workload == "hot760k" else None,
                              "algorithmic_bytes": int(b), "launch_ms": round(mean_pass[k], 4),
                              "peak_source": "measured" if peaks else "fallback"}
    roofline_hbm = roofline_passes.get(dom)
    clock_summary = clocks.summary(t_begin, t_end)
    roofline_raster = None
    if args.workload == "hot760k":  # the committed instruction count is of that workload
        roofline_raster = raster_issue_roofline(mean_pass.get("raster"), clock_summary.get("sm_mhz"),
                                                torch.cuda.get_device_properties(dev).multi_processor_count)
        if roofline_raster:
            roofline_raster["traffic"] = load_traffic("raster")
    # the frame's dominant kernel is the rasteriser (about two thirds of the
    # frame), bound by instruction issue: its roofline heads the line; the
    # HBM-accounted passes follow
    roofline = roofline_raster or roofline_hbm
    out = {
        "metric": metric_name(wl), "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(frame_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {**wl.describe(), "pairs": P, "hot_tiles": int(st["hot_tiles"]), "chunks": int(st["chunks"]),
                   "depth_sort_passes": DP,
                   "l2": "256 MiB flush between timed steps",
                   "parallelism": f"replicas{world}"},
        "e2e": e2e, "gpu_launches": int(launches),
        "passes_ms": {k: round(v, 4) for k, v in mean_pass.items()},
        "pass_share": {k: round(v / frame_ms, 4) for k, v in mean_pass.items()},
        "roofline": roofline, "roofline_hbm": roofline_hbm, "roofline_passes": roofline_passes,
        "clocks": clock_summary,
        "gpu_back_to_front_sort_ms": round(sort_ms, 4),
        "composite_only_ms": round(composite_only_ms, 4),
        "moving_camera": moving,
    }
    if rank == 0 and not args.no_deferred:
        log("deferred tail leg")
        out["deferred"] = run_deferred(pkg, F, wl, args, dev, cpu=not args.no_cpu_baseline)
    if rank == 0 and not args.no_train:
        log("training leg")
        out["train"] = run_train(pkg, args, dev)
    if rank == 0 and not args.no_serve:
        log("serving leg")
        out["serve"] = run_serve(pkg, args, dev)
    if rank == 0 and not args.no_sh3:
        log("sh3 orbit leg")
        out["sh3_orbit"] = run_sh3_orbit(pkg, args, dev, peak)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(pkg, wl, F)
    if world > 1:
        torch.distributed.barrier()
    if rank == 0:
        print(json.dumps(out))
    res.destroy()


def run_moving_camera(pkg, F, wl, args, stream) -> dict:
    """The timed workload under a camera that orbits by a fixed azimuth step
    per frame, as in an interactive viewer: every frame sorts the splats back
    to front on the device into the bound sortedIndices, uploads its uniform
    block and renders a full frame (one stream, CUDA events over a run of
    frames). The raster's work order comes from the previous frame's tile
    costs, so this measures how well that order carries across camera
    motion; the static frame (plus its sort) is the reference point. The
    static camera's state is restored afterwards."""
    import dataclasses

    import torch

    plan, bufs = F["plan"], F["bufs"]
    cam0 = wl.cameras[0]
    frames = max(8, min(args.steps, 60))
    out = {"frames_per_run": frames}
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    seqs = {}
    for deg in (0.25, 1.0, 4.0):
        cams = [dataclasses.replace(cam0, azimuth=cam0.azimuth + math.radians(deg) * i) for i in range(frames)]
        us = [pkg.frame_uniforms_for(plan, c, sh_degree=wl.scene.sh_degree)[0] for c in cams]
        views = [np.asarray(c.frame(wl.width, wl.height)["view"], np.float32).reshape(-1) for c in cams]
        seqs[deg] = (us, views)
    # a handle of its own, its pair capacity sized on the sequences' frames
    res = pkg.create_tile_splat_compositor(plan, pair_capacity=F["res"].pair_capacity)
    pkg.create_tile_splat_bind_groups(res, bufs, F["color"], F["gb"])
    need = 0
    for us, views in seqs.values():
        for u, v in zip(us, views):
            pkg.sort_back_to_front(stream, res, v, bufs["sorted_indices"])
            pkg.write_frame_uniform_buffer(res, u)
            pkg.encode_full_compute_compositor_pipeline(stream, res)
            need = max(need, int(res.query_status()["total_pairs"]))
    if need > res.pair_capacity:
        res.destroy()
        res = pkg.create_tile_splat_compositor(plan, pair_capacity=int(need * 1.02) + 1024)
        pkg.create_tile_splat_bind_groups(res, bufs, F["color"], F["gb"])
    for deg, (us, views) in seqs.items():

        def run():
            for u, v in zip(us, views):
                pkg.sort_back_to_front(stream, res, v, bufs["sorted_indices"])
                pkg.write_frame_uniform_buffer(res, u)
                pkg.encode_full_compute_compositor_pipeline(stream, res)

        run()  # warm: sizes, graph, costs of the sequence's own frames
        torch.cuda.synchronize()
        s.record(stream)
        run()
        e.record(stream)
        e.synchronize()
        res.check_frame()
        out[f"ms_per_frame_{deg:g}deg"] = round(s.elapsed_time(e) / frames, 4)
    # back to the static camera for the legs that follow (they share the
    # bound sortedIndices and the output images)
    view0 = np.asarray(cam0.frame(wl.width, wl.height)["view"], np.float32).reshape(-1)
    pkg.sort_back_to_front(stream, res, view0, bufs["sorted_indices"])
    res.destroy()
    F["res"].check_frame()
    pkg.encode_full_compute_compositor_pipeline(stream, F["res"])
    torch.cuda.synchronize()
    return out


def run_deferred(pkg, F, wl, args, dev, cpu: bool) -> dict:
    """The deferred frame tail (normals, bilateral, GTAO, bloom, lighting) on
    the timed frame's G-buffer at its viewport, unprofiled (bloom on the side
    stream) and per pass (profiled), plus the oracle's time for the same tail."""
    import torch

    D = pkg.deferred
    W, H = wl.width, wl.height
    post = D.DeferredPasses(W, H)
    post.set_environment(D.synthetic_environment(1024, 512, seed=0))
    q = D.frame_params(wl.cameras[0], W, H)
    lit = torch.zeros((H, W, 4), dtype=torch.float16, device=dev)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def tail():
        post.encode(stream, F["color"], F["gb"], q, lit)

    for _ in range(args.warmup):
        tail()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        tail()
        e.record(stream)
        e.synchronize()
        times.append(s.elapsed_time(e))
    post.set_profiling(True)
    passes = {}
    for _ in range(args.steps):
        flush.zero_()
        tail()
        for name, ms in post.pass_times():
            passes.setdefault(name, []).append(ms)
    post.set_profiling(False)
    ms = statistics.mean(times)
    out = {"ms": round(ms, 4), "tails_per_s": round(1000.0 / ms, 1),
           "passes_ms": {k: round(statistics.mean(v), 4) for k, v in passes.items()},
           "kernels_per_tail": 9, "viewport": [W, H],
           "environment": "synthetic 1024x512 equirect, seeded (stand-in for the reference's 1k HDRI)"}
    if cpu:
        import oracle

        torch.cuda.synchronize()
        inp, keep = oracle.post_inputs(F["color"].float().cpu().numpy(), F["gb"]["depth"].cpu().numpy(),
                                       F["gb"]["normal"].cpu().numpy(), F["gb"]["material"].cpu().numpy())
        ew, eh = post.env_size
        env = oracle.post_env_chain(post.buffer("env").cpu().numpy().view(np.uint16)[: ew * eh * 4].reshape(eh, ew, 4))
        brdf = post.buffer("brdf_lut").cpu().numpy().view(np.uint32).reshape(256, 256)
        curves = post.buffer("curves").cpu().numpy().view(np.uint16)[:768].reshape(3, 256)
        hw, hh = (W + 1) // 2, (H + 1) // 2
        tx, ty = float(np.float32(1.0 / hw)), float(np.float32(1.0 / hh))
        t0 = time.perf_counter()
        nrm = oracle.post_bilateral(inp, q, oracle.post_ss_normals(inp, q))
        mips = oracle.post_gtao_prefilter(inp, q)
        ao = oracle.post_gtao_denoise(inp, q, oracle.post_gtao_main(inp, q, mips, nrm), mips[0])
        bloom = oracle.post_bloom_blur(oracle.post_bloom_blur(oracle.post_bloom_threshold(inp, q), tx, 0.0, tx, ty),
                                       0.0, ty, tx, ty)
        ref = oracle.post_lighting(inp, q, nrm, ao, env, brdf, bloom, curves)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(1.0 / dt, 4), "unit": "tails/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": f"one {W}x{H} tail through the oracle (C, OpenMP)"}
        out["matches_oracle"] = bool(np.array_equal(ref, lit.cpu().numpy().view(np.uint16)))
    post.destroy()
    return out


def raster_issue_roofline(raster_ms: float, sm_mhz, sms: int):
    """Issue roofline of the rasteriser: its warp instructions per launch
    (ncu smsp__inst_executed.sum of one warm launch on the same workload,
    committed in profiles/raster_issue.json) over the live CUDA-event time,
    against every SM scheduler issuing one warp instruction per cycle (4 per
    SM) at the SM clock sampled during the timed frames."""
    f = ROOT / "profiles" / "raster_issue.json"
    if not f.exists() or not raster_ms:
        return None
    d = json.loads(f.read_text())
    inst = float(d["inst_executed_per_launch"])
    mhz = float(sm_mhz or 2070.0)
    achieved = inst / (raster_ms / 1000.0) / 1e9  # warp instructions per ns = G/s
    peak = sms * 4 * mhz * 1e6 / 1e9
    return {"bound": "issue", "kernel": "raster", "achieved": round(achieved, 1), "peak": round(peak, 1),
            "unit": "G warp-instructions/s", "frac": round(achieved / peak, 4),
            "inst_per_launch": int(inst), "launch_ms": round(raster_ms, 4), "sm_mhz": mhz,
            "inst_source": f"profiles/raster_issue.json ({d.get('workload')}, {d.get('build', '')})".strip()}


def load_traffic(kernel: str):
    """dram bytes per launch from the committed ncu summary, when present."""
    f = ROOT / "profiles" / "traffic.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get(kernel)
    return None


def _packed(specs, device, pin=False):
    """One allocation holding several typed arrays (256-byte aligned views):
    specs = [(name, shape, dtype)]; returns (raw uint8 buffer, {name: view})."""
    import torch

    offs, total = {}, 0
    for name, shape, dtype in specs:
        n = int(np.prod(shape)) * torch.empty((), dtype=dtype).element_size()
        offs[name] = (total, n)
        total = (total + n + 255) // 256 * 256
    raw = torch.empty(total, dtype=torch.uint8, device=device)
    if pin:
        raw = raw.pin_memory()
    views = {name: raw[o:o + n].view(dtype).view(shape) for (name, shape, dtype), (o, n) in zip(specs, offs.values())}
    return raw, views


def run_e2e(pkg, F, args, stream, world, dev):
    """Frames/s through the C ABI with host buffers: every step uploads the
    whole scene from pinned host memory, encodes the frame and reads the four
    output images back. The scene arrays live in one pinned block and one
    device block, the output images in one device block, so a step is one
    upload, the frame and one readback. Steps are double-buffered over two
    handles (each with its own device scene and output buffers) on an upload,
    a compute and a readback stream, so step k's copies overlap the frames of
    steps k - 1 and k + 1; every copy of every timed step is inside the timed
    region."""
    import torch

    names = ["positions", "scales", "rotations", "opacities", "material", "sh_data", "sorted_indices"]
    specs = [(k, tuple(F["bufs"][k].shape), F["bufs"][k].dtype) for k in names]
    host_raw, host = _packed(specs, "cpu", pin=True)
    for k in names:
        host[k].copy_(F["bufs"][k].cpu())
    plan = F["plan"]
    H, W = plan.viewport_height, plan.viewport_width
    out_specs = [("color", (H, W, 4), torch.float16), ("depth", (H, W), torch.float32),
                 ("normal", (H, W), torch.int32), ("material", (H, W, 4), torch.int32)]
    lanes = []
    for _ in range(2):
        dev_raw, bufs = _packed(specs, dev)
        bufs.update(normals=None, sh_degree=F["bufs"]["sh_degree"], count=F["bufs"]["count"])
        out_raw, o = _packed(out_specs, dev)
        gb = {"depth": o["depth"], "normal": o["normal"], "material": o["material"]}
        res = pkg.create_tile_splat_compositor(plan, pair_capacity=F["res"].pair_capacity)
        pkg.create_tile_splat_bind_groups(res, bufs, o["color"], gb)
        pkg.write_frame_uniform_buffer(res, F["u"])
        lanes.append({"dev_raw": dev_raw, "bufs": bufs, "res": res, "out_raw": out_raw, "outs": o,
                      "host_out": torch.empty(out_raw.numel(), dtype=torch.uint8).pin_memory(),
                      "uploaded": torch.cuda.Event(), "computed": torch.cuda.Event(), "read": torch.cuda.Event()})
    h2d = int(host_raw.numel())
    d2h = int(lanes[0]["out_raw"].numel())
    up, comp, down = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    for L in lanes:  # first use of each lane waits on nothing
        for ev, st in ((L["computed"], comp), (L["read"], down)):
            ev.record(st)

    def step(i):
        L = lanes[i & 1]
        up.wait_event(L["computed"])  # the lane's scene is free once its last frame ran
        with torch.cuda.stream(up):
            L["dev_raw"].copy_(host_raw, non_blocking=True)
        L["uploaded"].record(up)
        comp.wait_event(L["uploaded"])
        comp.wait_event(L["read"])  # the lane's images are free once read back
        pkg.encode_full_compute_compositor_pipeline(comp, L["res"])
        L["computed"].record(comp)
        down.wait_event(L["computed"])
        with torch.cuda.stream(down):
            L["host_out"].copy_(L["out_raw"], non_blocking=True)
        L["read"].record(down)

    for i in range(max(1, args.warmup)):
        step(i)
    torch.cuda.synchronize()
    for L in lanes:
        L["res"].check_frame()
    if world > 1:
        torch.distributed.barrier()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(up)
    for i in range(args.steps):
        step(i)
    e.record(down)
    e.synchronize()
    for L in lanes:
        L["res"].check_frame()
    total_s = slowest_rank_seconds(s.elapsed_time(e) / 1000.0, world, dev)
    for L in lanes:
        L["res"].destroy()
    return {"value": round(replicas_value(args.steps, world, total_s), 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h),
            "pipelining": "2 handles; one upload, the frame and one readback per step on 3 streams"}


def cpu_baseline(pkg, wl, F=None, threads=None, frames=1) -> dict:
    """The oracle (C restatement of the reference passes) on the host cores:
    full frames of the same workload, plus the reference's CPU depth sort."""
    import oracle

    threads = threads or os.cpu_count() or 1
    packed = F["packed"] if F else pkg.splats.pack_splat_attributes(wl.scene)
    if F:
        u, order = F["u"], F["order"]
    else:
        plan = pkg.plan_tile_splat_compositor(wl.width, wl.height, 16, wl.scene.count)
        u, fr = pkg.frame_uniforms_for(plan, wl.cameras[0], sh_degree=wl.scene.sh_degree)
        order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    cap = int(F["stats"]["total_pairs"]) + 16 if F else None
    oracle.render_frame(u, packed, order, threads=threads, cap=cap)  # warm (page-in, allocation)
    t0 = time.perf_counter()
    for _ in range(frames):
        oracle.render_frame(u, packed, order, threads=threads, cap=cap)
    dt = time.perf_counter() - t0
    view = wl.cameras[0].view_matrix()
    sort_ms = {}
    for nt in (1, 8):  # the reference's single-threaded sort, and an 8-thread parallel one
        oracle.sort_back_to_front(packed.positions, view, threads=nt)
        t1 = time.perf_counter()
        oracle.sort_back_to_front(packed.positions, view, threads=nt)
        sort_ms[nt] = (time.perf_counter() - t1) * 1000.0
    return {"value": round(frames / dt, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{frames} full frame(s) of {wl.name} through the oracle (C, OpenMP)",
            "cpu_depth_sort_ms": round(sort_ms[1], 2), "cpu_depth_sort_8t_ms": round(sort_ms[8], 2),
            "cpu_depth_sort": "splatSort.ts sortSplatIdsBackToFront, C restatement: 1 thread (as the reference "
                              "runs it) and 8 threads (8 sorted slices merged pairwise, the same order)"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    # the scene, camera and packing come from the package's pure-Python
    # modules; the plan and the uniform block from the oracle: this arm never
    # loads the product library
    pkg = __graft_entry__.load_package()
    import oracle

    oracle.build()
    wl = pkg.workloads.WORKLOADS[args.workload]()
    threads = os.cpu_count() or 1
    packed = pkg.splats.pack_splat_attributes(wl.scene)
    fr = wl.cameras[0].frame(wl.width, wl.height)
    u = oracle.frame_uniforms(oracle.plan(wl.width, wl.height, 16, wl.scene.count), fr["view_proj"], 1.0,
                              wl.scene.sh_degree, fr["camera_pos"], fr["view"], fr["proj"], None)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    f = oracle.render_frame(u, packed, order, threads=threads, composite=False)
    cap = f["total_pairs"] + 16
    oracle.render_frame(u, packed, order, threads=threads, cap=cap)  # warm (page-in); more would not change it
    # a step is one full frame; the run stops after REFERENCE_TIME_CAP_S so
    # that any --steps finishes within a few minutes
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        oracle.render_frame(u, packed, order, threads=threads, cap=cap)
        done += 1
        if time.perf_counter() - t0 > REFERENCE_TIME_CAP_S:
            break
    dt = time.perf_counter() - t0
    value = done / dt
    out = {"metric": metric_name(wl), "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "steps_run": done, "warmup": args.warmup, "ms_per_step": round(dt * 1000.0 / done, 2),
           "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "impl": "reference", "config": {**wl.describe(), "pairs": int(f["total_pairs"])},
           "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"{done} full frames of {wl.name} (one per step, at most "
                                      f"{REFERENCE_TIME_CAP_S:.0f} s) through the oracle (C restatement of the "
                                      f"reference's WGSL passes; the TypeScript/WebGPU original cannot run on "
                                      f"this machine)"},
           "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hot760k")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiler runs)")
    ap.add_argument("--no-train", action="store_true", help="skip the fwd+bwd leg (train500k)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg (8 scenes, 2,000 requests)")
    ap.add_argument("--no-deferred", action="store_true", help="skip the deferred-tail leg")
    ap.add_argument("--no-sh3", action="store_true", help="skip the 3M-splat SH3 4K orbit leg")
    ap.add_argument("--no-moving", action="store_true", help="skip the moving-camera leg")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    try:
        run_ours(args, rank, world, local)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
