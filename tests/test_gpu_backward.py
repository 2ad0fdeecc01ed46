"""The frame's adjoint (hdsr_encode_backward) and its torch.autograd binding.

Gradients are checked against central differences of the oracle's FP64
forward (same per-tile entry lists, no f16 rounding) on a 2,000-splat,
64x64, SH degree 1 sub-scene of the training distribution. Tolerance: 1e-3
relative; a gradient below 1% of the RMS gradient is held to 1e-3 of that
floor instead (absolute 1e-5 x RMS: the fp32 sums over pixels carry about that
much noise). Masked, as the threshold-adjacent entries of that comparison:
 - parameters whose FP64 difference quotient changes between steps h and 4h
   (the perturbation crosses a threshold of the composite);
 - splats with a (pixel, entry) within 1e-4 relative of a threshold of the
   composite (power -4, alpha 1/255, the 0.99 alpha cap, T 0.001) or of a
   clamp (opacity 0.99, colour 0 or 1), where fp32 and FP64 may decide
   differently.
"""
import copy

import numpy as np
import pytest

from gpu_helpers import u32

pytestmark = pytest.mark.gpu

GROUPS = [("positions", "positions", 3), ("log_scales", "scales", 3), ("rotations", "rotations", 4),
          ("opacities", "opacities", 1), ("sh", "sh_data", 15)]


def _sub_scene(pkg, n=2000, W=64, H=64, seed=5):
    sc = pkg.workloads.hot_scene(n, seed, sh_degree=1)
    cam = pkg.camera.OrbitCamera(azimuth=0.4, elevation=0.2, distance=3.0)
    packed = pkg.splats.pack_splat_attributes(sc)
    plan = pkg.plan_tile_splat_compositor(W, H, 16, sc.count)
    u, fr = pkg.frame_uniforms_for(plan, cam, sh_degree=1)
    order = pkg.splats.back_to_front_order(packed.positions, fr["view"])
    return sc, packed, plan, u, order


def _tensors(packed, order):
    import torch

    def t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    n = packed.count
    return (t(packed.positions.reshape(n, 3)), t(packed.scales.reshape(n, 3)), t(packed.rotations.reshape(n, 4)),
            t(packed.opacities.reshape(n)), t(packed.sh_data.reshape(n, -1)),
            t(np.asarray(order, np.uint32).view(np.int32)))


def _gpu_gradients(pkg, renderer, tens, u, weights):
    import torch

    pos, lsc, rot, opa, sh, srt = tens
    renderer.forward_frame(pos, lsc, rot, opa, sh, srt, u)
    grads = {"positions": torch.empty_like(pos), "log_scales": torch.empty_like(lsc),
             "rotations": torch.empty_like(rot), "opacities": torch.empty_like(opa), "sh": torch.empty_like(sh)}
    pkg.encode_backward(None, renderer.res, torch.from_numpy(weights).cuda(), grads)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in grads.items()}


def test_gradients_match_fp64_central_differences(cuda, pkg, orc):
    from oracle import adjoint

    sc, packed, plan, u, order = _sub_scene(pkg)
    renderer = pkg.differentiable.SplatFrameRenderer(plan.viewport_width, plan.viewport_height, sc.count,
                                                    sh_degree=1)
    tens = _tensors(packed, order)
    rng = np.random.default_rng(0)
    weights = rng.standard_normal((plan.viewport_height, plan.viewport_width, 4)).astype(np.float32)
    G = _gpu_gradients(pkg, renderer, tens, u, weights)
    frame = orc.render_frame(u, packed, order)
    assert np.array_equal(u32(renderer.res.buffer("tile_entries", count=frame["total_pairs"])),
                          frame["tile_entries"])
    par = orc.project_f64(u, packed, order)
    flagged = adjoint.threshold_adjacent_ranks(u, par, frame)
    inv = np.empty(sc.count, np.int64)
    inv[np.asarray(order, np.int64)] = np.arange(sc.count)
    # S per parameter: the sum of the absolute per-pixel terms of its gradient
    _, S = adjoint.reference_gradient(u, packed, order, frame, weights.astype(np.float64), with_scale=True)

    def loss(pk):
        return float((orc.render_frame_f64(u, pk, order, frame) * weights).sum())

    contributing = np.nonzero(np.abs(G["opacities"]) > 0)[0]
    clean = np.array([i for i in contributing if int(inv[i]) not in flagged])
    assert clean.size > 200, (contributing.size, clean.size)
    rows = []
    for trial in range(200):
        gname, pname, width = GROUPS[trial % len(GROUPS)]
        sid = int(rng.choice(clean))
        j = int(rng.integers(0, 12 if gname == "sh" else width))  # dc and all 9 SH1 slots, not the emissive ones
        idx = sid * width + j
        arr = getattr(packed, pname)
        flat = arr.reshape(-1)
        th = float(flat[idx])
        fds = []
        for h in (1e-6, 4e-6):
            hh = h * max(1.0, abs(th))
            tp, tm = np.float32(th + hh), np.float32(th - hh)
            pk = copy.copy(packed)
            a2 = flat.copy()
            a2[idx] = tp
            setattr(pk, pname, a2.reshape(arr.shape))
            lp = loss(pk)
            a2[idx] = tm
            setattr(pk, pname, a2.reshape(arr.shape))
            lm = loss(pk)
            fds.append((lp - lm) / (float(tp) - float(tm)))
        rows.append((trial % len(GROUPS), float(G[gname].reshape(-1)[idx]), fds[0], fds[1],
                     float(S[gname].reshape(-1)[idx])))
    rows = np.array(rows)
    consistent = np.abs(rows[:, 2] - rows[:, 3]) <= 1e-4 * np.maximum(np.abs(rows[:, 2]), 1e-3)
    # trials whose quotients at h and 4h disagree crossed a threshold of the
    # composite: dropped, and reported
    print(f"finite-difference trials: {len(rows)}, dropped as inconsistent: {int((~consistent).sum())}")
    assert consistent.sum() >= 150
    r = rows[consistent]
    # within 1e-3 relative (floored at 1e-2 of the RMS gradient), or, where
    # the gradient sums opposing pixel terms, within 2e-3 of S: the fp32
    # frame's transmittance drifts from the FP64 frame's by up to ~7e-4
    # (see test_gradients_match_the_fp64_reference_gradient)
    scale = np.sqrt(np.mean(r[:, 2] ** 2))
    err = np.abs(r[:, 1] - r[:, 2])
    ok = (err <= 1e-3 * np.maximum(np.abs(r[:, 2]), 1e-2 * scale)) | (err <= 2e-3 * r[:, 4])
    rel = err / np.maximum(np.abs(r[:, 2]), 1e-2 * scale)
    print(f"within 1e-3 relative: {int((rel <= 1e-3).sum())} of {len(r)}; the rest within 2e-3 of S: "
          f"{int((~(rel <= 1e-3) & ok).sum())}")
    for k, (gname, _, _) in enumerate(GROUPS):
        sel = r[:, 0] == k
        assert sel.sum() >= 20, gname
        assert ok[sel].all(), (gname, float(rel[sel].max()), r[sel][np.argmax(rel[sel])])
    renderer.destroy()


def test_gradients_match_the_fp64_reference_gradient(cuda, pkg, orc):
    """Every parameter of every splat of the 2,000-splat, 64x64, SH1
    sub-scene against the oracle's analytic FP64 gradient (forward-mode
    projection, reverse composite: oracle/adjoint.py, itself pinned to FP64
    central differences on the CPU), twice.

    1. The FP64 gradient of the frame as fp32 renders it: the projection's
       derivatives and the reverse sweep in FP64, the composite's alphas and
       transmittances those of the canonical f32 composite at the f32
       screen-space values. Every parameter, nothing masked: within 1e-3
       relative, the denominator floored at 1e-2 of the group's RMS gradient
       and at 1e-3 of S, the sum of the absolute per-pixel terms the gradient
       adds up (an fp32 sum of such terms is rounded against S, not against
       its result, so a gradient that cancels far below S is held to 1e-6 S).
    2. The FP64 gradient of the FP64 frame (exact screen-space values, FP64
       alphas and transmittances). An fp32 transmittance drifts from the FP64
       one (up to ~7e-4 relative after ~100 entries of a dense pixel), which a
       gradient summing opposing pixel terms magnifies: outside the
       threshold-adjacent pixels the difference stays below 2e-3 of S, and
       the per-group relative errors are reported."""
    from oracle import adjoint

    sc, packed, plan, u, order = _sub_scene(pkg)
    renderer = pkg.differentiable.SplatFrameRenderer(plan.viewport_width, plan.viewport_height, sc.count,
                                                    sh_degree=1)
    tens = _tensors(packed, order)
    rng = np.random.default_rng(2)
    weights = rng.standard_normal((plan.viewport_height, plan.viewport_width, 4)).astype(np.float32)
    G = _gpu_gradients(pkg, renderer, tens, u, weights)
    frame = orc.render_frame(u, packed, order)
    d_out = weights.astype(np.float64)
    R32, S32 = adjoint.reference_gradient(u, packed, order, frame, d_out, with_scale=True, screen_f32=True,
                                          trajectory="f32")
    R64, S64 = adjoint.reference_gradient(u, packed, order, frame, d_out, with_scale=True)
    par = orc.project_f64(u, packed, order)
    flagged = adjoint.threshold_adjacent_ranks(u, par, frame)
    ids = np.asarray(order, np.int64)
    clean = np.ones(sc.count, bool)
    clean[ids[sorted(flagged)]] = False
    assert clean.sum() >= 0.8 * sc.count, int(clean.sum())
    report32, report64 = {}, {}
    for gname, width in (("positions", 3), ("log_scales", 3), ("rotations", 4), ("opacities", 1), ("sh", 12)):
        g = G[gname].reshape(sc.count, -1)[:, :width].astype(np.float64)
        r, s = R32[gname].reshape(sc.count, -1)[:, :width], S32[gname].reshape(sc.count, -1)[:, :width]
        rel = np.abs(g - r) / np.maximum(np.maximum(np.abs(r), 1e-2 * np.sqrt(np.mean(r ** 2))), 1e-3 * s)
        report32[gname] = (int(rel.size), float(rel.max()))
        gc = g[clean]
        r, s = R64[gname].reshape(sc.count, -1)[clean][:, :width], S64[gname].reshape(sc.count, -1)[clean][:, :width]
        rel = np.abs(gc - r) / np.maximum(np.maximum(np.abs(r), 1e-2 * np.sqrt(np.mean(r ** 2))), 1e-3 * s)
        drift = np.abs(gc - r) / np.maximum(s, 1e-300)
        nz = np.abs(r) > 0
        report64[gname] = (int(rel.size), float(np.median(rel[nz])), float(np.percentile(rel, 99.9)),
                           float(rel.max()), float(drift.max()))
    print("GPU adjoint vs the FP64 gradient along the f32 trajectory (parameters, max rel):", report32)
    print("GPU adjoint vs the FP64 gradient of the FP64 frame, clean splats "
          "(parameters, median rel of the non-zero ones, 99.9th percentile, max rel, max |g - r| / S):", report64)
    for gname, (cnt, worst) in report32.items():
        assert worst <= 1e-3, (gname, worst)
    for gname, (cnt, med, p999, worst, drift) in report64.items():
        assert med <= 1e-5 and drift <= 2e-3, (gname, med, drift)
    # the emissive slots of the SH rows get exactly 0 from both
    assert not G["sh"][:, 12:].any() and not R32["sh"][:, 12:].any()
    renderer.destroy()


def test_autograd_matches_the_c_abi_and_trains(cuda, pkg):
    import torch

    sc, packed, plan, u, order = _sub_scene(pkg, n=3000, W=96, H=80, seed=8)
    renderer = pkg.differentiable.SplatFrameRenderer(plan.viewport_width, plan.viewport_height, sc.count,
                                                    sh_degree=1)
    pos, lsc, rot, opa, sh, srt = _tensors(packed, order)
    target = renderer.render(pos, lsc, rot, opa, sh, srt, u).detach().clone()
    g = torch.Generator(device="cuda").manual_seed(3)
    params = [pos + 0.01 * torch.randn(pos.shape, device="cuda", generator=g), lsc.clone(), rot.clone(),
              torch.logit(opa.clamp(1e-4, 1 - 1e-4)), sh.clone()]
    for p in params:
        p.requires_grad_(True)
    img = renderer.render(params[0], params[1], params[2], torch.sigmoid(params[3]), params[4], srt, u)
    loss = ((img - target) ** 2).mean()
    loss.backward()
    # the same frame's gradients straight through the C ABI
    d_color = (2.0 * (img.detach() - target) / img.numel()).contiguous()
    direct = {k: torch.empty_like(v) for k, v in (("positions", pos), ("log_scales", lsc), ("rotations", rot),
                                                  ("opacities", opa), ("sh", sh))}
    renderer.forward_frame(params[0].detach(), params[1].detach(), params[2].detach(),
                           torch.sigmoid(params[3]).detach(), params[4].detach(), srt, u)
    pkg.encode_backward(None, renderer.res, d_color, direct)
    torch.cuda.synchronize()
    # float atomics add in a different order from run to run: equal up to
    # that rounding, measured against each gradient array's scale (a
    # gradient that cancels to near zero, such as the radial component of a
    # quaternion's, is all rounding)
    def close(a, b):
        return torch.allclose(a, b, rtol=1e-4, atol=1e-5 * float(b.abs().max()))

    for p, k in zip(params[:3], ("positions", "log_scales", "rotations")):
        assert torch.isfinite(p.grad).all()
        assert close(p.grad, direct[k]), k
    s = torch.sigmoid(params[3]).detach()
    assert close(params[3].grad, direct["opacities"] * s * (1 - s))
    assert close(params[4].grad, direct["sh"])
    assert float(params[0].grad.abs().sum()) > 0
    # the gradient is a descent direction: normalised steps on the positions
    # (at most 5e-4 per coordinate) lower the loss
    first = float(loss.detach())
    cur = params[0].detach().clone()
    grad = params[0].grad.detach()
    for _ in range(5):
        cur = cur - 5e-4 * grad / grad.abs().max()
        p0 = cur.clone().requires_grad_(True)
        img = renderer.render(p0, params[1].detach(), params[2].detach(), torch.sigmoid(params[3]).detach(),
                              params[4].detach(), srt, u)
        loss = ((img - target) ** 2).mean()
        loss.backward()
        grad = p0.grad.detach()
    assert float(loss.detach()) < first
    renderer.destroy()


def test_backward_is_repeatable_and_validated(cuda, pkg):
    import torch

    sc, packed, plan, u, order = _sub_scene(pkg, n=1500, W=64, H=48, seed=9)
    renderer = pkg.differentiable.SplatFrameRenderer(plan.viewport_width, plan.viewport_height, sc.count,
                                                    sh_degree=1)
    tens = _tensors(packed, order)
    w = np.random.default_rng(1).standard_normal((plan.viewport_height, plan.viewport_width, 4)).astype(np.float32)
    a = _gpu_gradients(pkg, renderer, tens, u, w)
    b = _gpu_gradients(pkg, renderer, tens, u, w)
    # float atomics land in a different order from run to run: equal up to
    # that rounding, measured against each gradient array's scale
    for k in a:
        assert np.abs(a[k] - b[k]).max() <= 1e-5 * np.abs(a[k]).max(), k
    # a handle without the adjoint buffers refuses; so does one with no frame
    res = pkg.create_tile_splat_compositor(plan)
    grads = {k: torch.zeros(1, device="cuda") for k in ("positions", "log_scales", "rotations", "opacities", "sh")}
    d = torch.zeros((plan.viewport_height, plan.viewport_width, 4), device="cuda")
    with pytest.raises(pkg._lib.HdsrError) as e:
        pkg.encode_backward(None, res, d, grads)
    assert e.value.status == 6
    res.destroy()
    fresh = pkg.create_tile_splat_compositor(plan, backward=True)
    with pytest.raises(pkg._lib.HdsrError) as e:
        pkg.encode_backward(None, fresh, d, grads)
    assert e.value.status == 7
    fresh.destroy()
    renderer.destroy()
