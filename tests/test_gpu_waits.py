"""Bounded device waits of the decoupled-lookback scans.

A scan tile waits for its predecessors' status words; every such wait is
bounded. The test hook of hdsr_set_scan_wait keeps one tile of each scan from
posting its status, with a short spin limit, so the next tile's wait runs
out: the frame must end (no hang), report HDSR_ERR_TIMEOUT with the timeout
device flag, leave the outputs untouched (the kernels after the scan return
at once), and the same handle must render the exact frame again once the hook
is cleared.
"""
import time

import numpy as np
import pytest

from gpu_helpers import assert_frame_parity, render_gpu

pytestmark = pytest.mark.gpu


def test_withheld_scan_tile_times_out_and_the_handle_recovers(cuda, pkg, orc):
    import torch

    # 800x600: 3,364 Morton tiles, so the tile scan has 2 scan tiles of 2,048;
    # 20,000 splats: the per-splat scan has 10. Tile 1 of each waits on tile 0.
    scene = pkg.workloads.plain_scene(20_000, seed=5)
    g = render_gpu(pkg, scene, pkg.camera.look_from((0.1, 0.2, 4.0)), 800, 600)
    res = g["res"]
    assert_frame_parity(orc, g)
    color = g["color"].clone()
    material = g["gb"]["material"].clone()
    g["color"].fill_(0.25)
    g["gb"]["material"].fill_(7)
    torch.cuda.synchronize()
    res.set_scan_wait(spin_limit=1000, withheld_tile=0)
    t0 = time.perf_counter()
    pkg.encode_full_compute_compositor_pipeline(None, res)
    st = res.query_status()
    elapsed = time.perf_counter() - t0
    assert st["status"] == pkg._lib.HDSR_ERR_TIMEOUT, st
    assert st["device_flags"] & pkg._lib.DEV_TIMEOUT
    assert elapsed < 5.0, elapsed
    # the rasteriser returned without writing
    assert bool((g["color"] == 0.25).all()) and bool((g["gb"]["material"] == 7).all())
    # hook cleared, default limit: the same handle renders the frame again
    res.set_scan_wait()
    pkg.encode_full_compute_compositor_pipeline(None, res)
    torch.cuda.synchronize()
    gpu, _ = assert_frame_parity(orc, g)
    assert torch.equal(g["color"].view(torch.int16), color.view(torch.int16))
    assert torch.equal(g["gb"]["material"], material)
    res.destroy()


def test_withheld_last_tile_needs_no_wait(cuda, pkg, orc):
    # nobody waits on the last tile of a scan: withholding it changes nothing
    # (800x600 and 3,000 splats: both scans have 2 scan tiles)
    scene = pkg.workloads.plain_scene(3_000, seed=6)
    g = render_gpu(pkg, scene, pkg.camera.look_from((0.0, 0.1, 4.0)), 800, 600)
    res = g["res"]
    res.set_scan_wait(spin_limit=1000, withheld_tile=1)
    pkg.encode_full_compute_compositor_pipeline(None, res)
    st = res.query_status()
    assert st["status"] == 0 and not (st["device_flags"] & pkg._lib.DEV_TIMEOUT), st
    assert_frame_parity(orc, g)
    res.destroy()
