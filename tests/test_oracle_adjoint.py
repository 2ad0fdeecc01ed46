"""The oracle's FP64 reference gradient (oracle/adjoint.py) pinned against
FP64 central differences of the oracle's FP64 forward, on the CPU.

The reference gradient is the checker of the CUDA adjoint (see
test_gpu_backward.py), so it is itself checked here: forward-mode dual
numbers through the projection and a reverse sweep through the composite
must agree with difference quotients of orc_render_frame_f64 over the same
entry lists. A parameter counts when its quotient at h and 4h agrees
(no threshold crossed); tolerance 1e-4 relative (floored at 1e-2 of the RMS
gradient), far inside the 1e-3 the CUDA adjoint is held to.
"""
import copy

import numpy as np
import pytest

GROUPS = [("positions", "positions", 3), ("log_scales", "scales", 3), ("rotations", "rotations", 4),
          ("opacities", "opacities", 1), ("sh", "sh_data", None)]


@pytest.mark.parametrize("deg", [0, 1, 3])
def test_reference_gradient_matches_fp64_central_differences(pkg, orc, deg):
    from oracle import adjoint

    n, W, H = 300, 48, 40
    sc = pkg.workloads.hot_scene(n, 5, sh_degree=deg)
    cam = pkg.camera.OrbitCamera(azimuth=0.4, elevation=0.2, distance=3.0)
    packed = pkg.splats.pack_splat_attributes(sc)
    plan = pkg.plan_tile_splat_compositor(W, H, 16, n)
    u, fr = pkg.frame_uniforms_for(plan, cam, sh_degree=deg)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    frame = orc.render_frame(u, packed, order)
    rng = np.random.default_rng(deg)
    w = rng.standard_normal((H, W, 4))
    G = adjoint.reference_gradient(u, packed, order, frame, w)
    # the duals' values are the oracle's FP64 projection
    screen, vis, _ = adjoint.project_dual(u, packed, order)
    par = orc.project_f64(u, packed, order)
    for i, k in enumerate(("cx", "cy", "ia", "ib", "ic", "op", "r", "g", "b")):
        assert np.allclose(screen[k].v[vis], par[vis, i], rtol=1e-12, atol=1e-12), k
    flagged = adjoint.threshold_adjacent_ranks(u, par, frame)
    inv = np.empty(n, np.int64)
    inv[np.asarray(order, np.int64)] = np.arange(n)
    clean = [i for i in np.nonzero(np.abs(G["opacities"]) > 0)[0] if int(inv[i]) not in flagged]
    assert len(clean) > 100

    def loss(pk):
        return float((orc.render_frame_f64(u, pk, order, frame) * w).sum())

    sh_w = packed.sh_data.size // n
    rows = []
    for trial in range(100):
        gname, pname, width = GROUPS[trial % len(GROUPS)]
        width = width or sh_w
        colour_slots = width - 3 if gname == "sh" else width  # the emissive slots do not reach the image
        sid = int(rng.choice(clean))
        idx = sid * width + int(rng.integers(0, colour_slots))
        arr = getattr(packed, pname)
        flat = arr.reshape(-1)
        th = float(flat[idx])
        fds = []
        for h in (1e-6, 4e-6):
            hh = h * max(1.0, abs(th))
            tp, tm = np.float32(th + hh), np.float32(th - hh)
            a2 = flat.copy()
            pk = copy.copy(packed)
            a2[idx] = tp
            setattr(pk, pname, a2.reshape(arr.shape))
            lp = loss(pk)
            a2[idx] = tm
            setattr(pk, pname, a2.reshape(arr.shape))
            lm = loss(pk)
            fds.append((lp - lm) / (float(tp) - float(tm)))
        rows.append((trial % len(GROUPS), float(G[gname].reshape(-1)[idx]), fds[0], fds[1]))
    rows = np.array(rows)
    consistent = np.abs(rows[:, 2] - rows[:, 3]) <= 1e-4 * np.maximum(np.abs(rows[:, 2]), 1e-3)
    assert consistent.sum() >= 80, int(consistent.sum())
    r = rows[consistent]
    scale = np.sqrt(np.mean(r[:, 2] ** 2))
    rel = np.abs(r[:, 1] - r[:, 2]) / np.maximum(np.abs(r[:, 2]), 1e-2 * scale)
    assert rel.max() <= 1e-4, (float(rel.max()), r[np.argmax(rel)])
    # the emissive slots get no gradient
    assert not G["sh"][:, sh_w - 3:].any()
