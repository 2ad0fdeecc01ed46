"""FP64 reference gradient of one frame: TEST INFRASTRUCTURE ONLY.

The checker for hdsr_encode_backward. Only the test suite imports it; the
product never does. It differentiates the oracle's FP64 forward
(orc_render_frame_f64 over orc_project_f64 in hdsr_oracle.c: the projection
of gpu_project_splats.wgsl:112-358 and the composite of
gpu_tile_splat_composite.wgsl:162-370, in double, no f16 rounding) with the
per-tile entry lists held fixed and the composite's thresholds held fixed
(power > -4, alpha > 1/255, T >= 0.001): the function the adjoint
differentiates. It is written from that forward, not from the CUDA adjoint:

  - projection: forward-mode dual numbers (value + derivative with respect
    to every parameter of the splat) through the same steps as
    project_one_f64: the perspective centre, the quaternion normalisation,
    exp of the log-scales, the Jacobian with the vz clamp, the 0.3 low-pass,
    the anti-aliasing factor, the opacity clamp [0, 0.99], the SH colour with
    its view direction (degrees 1-3, the shader's basis and signs) clamped to
    [0, 1]. A clamp passes no derivative where it is active. The two
    determinants use |b0 x b1|^2 for b0.b0 b1.b1 - (b0.b1)^2 (the same value,
    without cancellation);
  - composite: reverse mode per pixel over the tile's entries, vectorised
    over the tile's 256 pixels and its entries (exclusive products for the
    transmittance, suffix sums for the light behind each entry);
  - chain: dL/d(splat parameters) = sum over the splat's screen-space
    gradient (centre, conic, opacity, colour) times the dual derivatives.

Parameters, per splat id (the layouts of hdsr_scene_views): positions 3,
log-scales 3, rotations 4 (wxyz, before normalisation), activated opacity 1,
the SH row (dc 3, higher bands 3K; the 3 emissive slots get 0).
"""
from __future__ import annotations

import numpy as np


class Dual:
    """Value (n,) and derivatives (n, m), float64."""

    __slots__ = ("v", "d")

    def __init__(self, v, d):
        self.v = v
        self.d = d

    @staticmethod
    def const(v, n, m):
        v = np.broadcast_to(np.asarray(v, np.float64), (n,)).astype(np.float64)
        return Dual(v, np.zeros((n, m)))

    def _lift(self, o):
        if isinstance(o, Dual):
            return o
        return Dual(np.broadcast_to(np.asarray(o, np.float64), self.v.shape), np.zeros_like(self.d))

    def __add__(self, o):
        o = self._lift(o)
        return Dual(self.v + o.v, self.d + o.d)

    __radd__ = __add__

    def __sub__(self, o):
        o = self._lift(o)
        return Dual(self.v - o.v, self.d - o.d)

    def __rsub__(self, o):
        return self._lift(o) - self

    def __neg__(self):
        return Dual(-self.v, -self.d)

    def __mul__(self, o):
        o = self._lift(o)
        return Dual(self.v * o.v, self.d * o.v[:, None] + o.d * self.v[:, None])

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = self._lift(o)
        q = self.v / o.v
        return Dual(q, (self.d - o.d * q[:, None]) / o.v[:, None])

    def __rtruediv__(self, o):
        return self._lift(o) / self


def dsqrt(x: Dual) -> Dual:
    s = np.sqrt(x.v)
    g = np.where(s > 0, 0.5 / np.where(s > 0, s, 1.0), 0.0)
    return Dual(s, x.d * g[:, None])


def dexp(x: Dual) -> Dual:
    e = np.exp(x.v)
    return Dual(e, x.d * e[:, None])


def dmax_const(x: Dual, c: float) -> Dual:
    """max(x, c): the constant (no derivative) where it wins."""
    keep = x.v > c
    return Dual(np.where(keep, x.v, c), x.d * keep[:, None])


def dmin_const(x: Dual, c: float) -> Dual:
    keep = x.v < c
    return Dual(np.where(keep, x.v, c), x.d * keep[:, None])


def dclamp(x: Dual, lo: float, hi: float) -> Dual:
    return dmin_const(dmax_const(x, lo), hi)


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def param_layout(sh_degree: int) -> dict:
    """Slices of the per-splat parameter vector."""
    k = (sh_degree + 1) ** 2 - 1
    sh_w = 6 + 3 * k
    return {"positions": slice(0, 3), "log_scales": slice(3, 6), "rotations": slice(6, 10),
            "opacities": slice(10, 11), "sh": slice(11, 11 + sh_w), "m": 11 + sh_w, "sh_width": sh_w}


def project_dual(U, packed, order):
    """Screen-space parameters per sortRank as duals over the splat's own
    parameters: dict of Dual (cx, cy, ia, ib, ic, op, r, g, b) and the
    visibility mask (project_one_f64 of hdsr_oracle.c)."""
    U = np.asarray(U, np.float32).astype(np.float64)
    deg = int(packed.sh_degree)
    lay = param_layout(deg)
    n, m = int(packed.count), lay["m"]
    ids = np.asarray(order, np.int64)
    pos = np.asarray(packed.positions, np.float32).reshape(n, 3).astype(np.float64)[ids]
    scl = np.asarray(packed.scales, np.float32).reshape(n, 3).astype(np.float64)[ids]
    rot = np.asarray(packed.rotations, np.float32).reshape(n, 4).astype(np.float64)[ids]
    opa = np.asarray(packed.opacities, np.float32).reshape(n).astype(np.float64)[ids]
    sh = np.asarray(packed.sh_data, np.float32).reshape(n, -1).astype(np.float64)[ids]

    def var(values, col):
        d = np.zeros((n, m))
        d[:, col] = 1.0
        return Dual(values, d)

    P = [var(pos[:, i], i) for i in range(3)]
    S = [var(scl[:, i], 3 + i) for i in range(3)]
    Q = [var(rot[:, i], 6 + i) for i in range(4)]
    O = var(opa, 10)
    SH = [var(sh[:, i], 11 + i) for i in range(lay["sh_width"])]

    clip = [P[0] * U[r] + P[1] * U[4 + r] + P[2] * U[8 + r] + U[12 + r] for r in range(4)]
    visible = clip[3].v > 0.0
    sw = dmax_const(clip[3], 1e-4)
    cx = (clip[0] / sw * 0.5 + 0.5) * U[16]
    cy = (1.0 - (clip[1] / sw * 0.5 + 0.5)) * U[17]
    ql = dmax_const(dsqrt(Q[0] * Q[0] + Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]), 1e-6)
    qx = Q[0] / ql
    u = (Q[1] / ql, Q[2] / ql, Q[3] / ql)
    axes = []
    for i in range(3):
        e = [1.0 if j == i else 0.0 for j in range(3)]
        c_in = _cross(u, e)
        inn = tuple(c_in[j] + qx * e[j] for j in range(3))
        c = _cross(u, inn)
        sc = dexp(S[i]) * U[24]
        axes.append(tuple((c[j] * 2.0 + e[j]) * sc for j in range(3)))
    w0, w1, w2 = (U[32], U[36], U[40]), (U[33], U[37], U[41]), (U[34], U[38], U[42])
    vc = [P[0] * U[32 + r] + P[1] * U[36 + r] + P[2] * U[40 + r] + U[44 + r] for r in range(3)]
    vz = dmin_const(vc[2], -0.001)
    J1x, J1y = U[48] / vz, U[49] / vz
    J2x, J2y = -J1x / vz * vc[0], -J1y / vz * vc[1]
    t0 = tuple(J1x * w0[j] + J2x * w2[j] for j in range(3))
    t1 = tuple(J1y * w1[j] + J2y * w2[j] for j in range(3))
    b0 = tuple(_dot(axes[i], t0) for i in range(3))
    b1 = tuple(_dot(axes[i], t1) for i in range(3))
    xx, xy, yy = _dot(b0, b0), _dot(b0, b1), _dot(b1, b1)
    cr = _cross(b0, b1)
    det_o = _dot(cr, cr)                     # = xx yy - xy^2
    XX, YY = xx + 0.3, yy + 0.3
    det_b = det_o + (xx + yy) * 0.3 + 0.09   # = XX YY - xy^2
    dbm = dmax_const(det_b, 1e-6)
    aa = dsqrt(dmax_const(det_o / dbm, 0.0))
    ia, ib, ic = YY / dbm, -xy / dbm, XX / dbm
    op = dclamp(O * aa, 0.0, 0.99)
    col = [SH[0], SH[1], SH[2]]
    if deg >= 1:
        d = (U[28] - P[0], U[29] - P[1], U[30] - P[2])
        ln = dsqrt(_dot(d, d))
        vx, vy, vw = d[0] / ln, d[1] / ln, d[2] / ln
        b = SH[3:]
        xx2, yy2, zz2 = vx * vx, vy * vy, vw * vw
        e2 = [vx * vy * 1.0925484305920792, vy * vw * 1.0925484305920792,
              (zz2 * 2.0 - xx2 - yy2) * 0.31539156525252005, vx * vw * 1.0925484305920792,
              (xx2 - yy2) * 0.5462742152960396]
        e3 = [vy * (xx2 * 3.0 - yy2) * 0.5900435899266435, vx * vy * vw * 2.890611442640554,
              vy * (zz2 * 4.0 - xx2 - yy2) * 0.4570457994644658,
              vw * (zz2 * 2.0 - xx2 * 3.0 - yy2 * 3.0) * 0.3731763325901154,
              vx * (zz2 * 4.0 - xx2 - yy2) * 0.4570457994644658, vw * (xx2 - yy2) * 1.445305721320277,
              vx * (xx2 - yy2 * 3.0) * 0.5900435899266435]
        for ch in range(3):
            acc = (b[ch] * vy + b[3 + ch] * vw + b[6 + ch] * vx) * 0.4886025119029199
            if deg >= 2:
                for k in range(5):
                    acc = acc + b[9 + 3 * k + ch] * e2[k]
            if deg >= 3:
                for k in range(7):
                    acc = acc + b[24 + 3 * k + ch] * e3[k]
            col[ch] = col[ch] + acc
    col = [dclamp(c, 0.0, 1.0) for c in col]
    screen = {"cx": cx, "cy": cy, "ia": ia, "ib": ib, "ic": ic, "op": op, "r": col[0], "g": col[1], "b": col[2]}
    return screen, visible, lay


def _f32_trajectory(p, px, py):
    """The canonical f32 composite of one tile's entries over its pixels (the
    oracle's composite arithmetic, hdsr_oracle.c: fused power, its own exp,
    f32 alpha and transmittance products), at the f32 values of the screen
    parameters p (K, 9): per entry and pixel the alpha, the exp factor, the
    capped flag, the validity and the transmittance before the entry."""
    from . import splat_expf  # the oracle's composite exp

    f32 = np.float32
    fma32 = lambda a, b, c: (np.asarray(a, np.float64) * b + c).astype(f32)  # noqa: E731
    K, n = p.shape[0], px.size
    px32, py32 = px.astype(f32), py.astype(f32)
    al, ex, cap, val, tin = (np.zeros((K, n)), np.zeros((K, n)), np.zeros((K, n), bool), np.zeros((K, n), bool),
                             np.zeros((K, n)))
    T = np.ones(n, f32)
    for k in range(K):
        cx, cy, ia, ib, ic, op = (f32(v) for v in p[k, :6])
        ka, kb, kc = f32(ia * f32(-0.5)), f32(-ib), f32(ic * f32(-0.5))
        dx, dy = (px32 - cx).astype(f32), (py32 - cy).astype(f32)
        pw = fma32((kc * dy).astype(f32), dy, fma32((kb * dx).astype(f32), dy, ((ka * dx).astype(f32) * dx).astype(f32)))
        g = splat_expf(pw).reshape(n)
        raw = (op * g).astype(f32)
        a = np.minimum(f32(0.99), raw)
        v = (pw > f32(-4.0)) & (a > f32(1.0) / f32(255.0)) & (T >= f32(0.001))
        # entries a pixel does not take contribute nothing (far entries may
        # even overflow the power to inf or nan there)
        al[k], ex[k], cap[k], val[k], tin[k] = np.where(v, a, 0), np.where(v, g, 0), v & (raw > f32(0.99)), v, T
        T = np.where(v, (T * (f32(1.0) - a).astype(f32)).astype(f32), T)
    return al, ex, cap, val, tin, T.astype(np.float64)


def composite_adjoint(U, screen: dict, frame: dict, d_out: np.ndarray, with_abs: bool = False,
                      trajectory: str = "f64"):
    """dL/d(cx, cy, ia, ib, ic, op, r, g, b) per sortRank for dL/d(output
    rgba) = d_out (H, W, 4), over the frame's entry lists; FP64 values of
    the screen parameters come from `screen`. With `with_abs`, also the sums
    of the absolute per-pixel terms (the magnitude an fp32 sum of those terms
    is rounded against).

    `trajectory` "f64": the composite's alphas and transmittances are FP64.
    "f32": they are those of the canonical f32 composite (_f32_trajectory),
    the reverse sweep staying FP64: the exact gradient of the frame as fp32
    renders it. An fp32 transmittance drifts from the FP64 one (each
    1 - alpha carries the rounding of alpha, relatively larger as alpha
    nears 1: measured up to 7e-4 after ~100 entries of a dense pixel), and a
    gradient that sums many opposing pixel terms magnifies that drift; this
    mode takes the drift out of the comparison with an fp32 adjoint."""
    U = np.asarray(U, np.float32)
    Uu = U.view(np.uint32)
    cols, rows = int(Uu[20]), int(Uu[21])
    W, H = int(U[16]), int(U[17])
    par = np.stack([screen[k].v for k in ("cx", "cy", "ia", "ib", "ic", "op", "r", "g", "b")], 1)
    g2d = np.zeros_like(par)
    gabs = np.zeros_like(par)
    counts, offs, ents = frame["tile_counts"], frame["tile_offsets"], frame["tile_entries"]
    bg = np.array([0.02, 0.02, 0.04])
    gy, gx = np.mgrid[0:16, 0:16]
    for ty in range(rows):
        for tx in range(cols):
            t = _morton(tx, ty)
            K = int(counts[t])
            if K == 0:
                continue
            X = (tx * 16 + gx).reshape(-1)
            Y = (ty * 16 + gy).reshape(-1)
            inside = (X < W) & (Y < H)
            X, Y = X[inside], Y[inside]
            px, py = X + 0.5, Y + 0.5
            e = np.asarray(ents[int(offs[t]): int(offs[t]) + K], np.int64)
            p = par[e]                                               # (K, 9)
            dx = px[None, :] - p[:, 0:1]
            dy = py[None, :] - p[:, 1:2]
            ia, ib, ic, op = p[:, 2:3], p[:, 3:4], p[:, 4:5], p[:, 5:6]
            if trajectory == "f32":
                a, ex, capped, valid, Tin, Tf = _f32_trajectory(p, px, py)
            else:
                pw = -0.5 * ia * dx * dx - 0.5 * ic * dy * dy - ib * dx * dy
                ex = np.exp(pw)
                raw = op * ex
                capped = raw > 0.99
                a = np.where(capped, 0.99, raw)
                cond = (pw > -4.0) & (a > 1.0 / 255.0)
                fac = np.where(cond, 1.0 - a, 1.0)
                G = np.vstack([np.ones((1, fac.shape[1])), np.cumprod(fac, axis=0)[:-1]])   # exclusive products
                valid = cond & (G >= 0.001)
                fac_v = np.where(valid, 1.0 - a, 1.0)
                Tin = np.vstack([np.ones((1, fac.shape[1])), np.cumprod(fac_v, axis=0)[:-1]])  # T before entry k
                Tf = Tin[-1] * fac_v[-1]
            wgt = np.where(valid, a * Tin, 0.0)                      # colour weight of entry k
            dC = d_out[Y, X, :3]                                     # (px, 3)
            dA = d_out[Y, X, 3]
            colr = p[:, 6:9]                                         # (K, 3)
            contrib = wgt[:, :, None] * colr[:, None, :]             # (K, px, 3)
            behind = np.cumsum(contrib[::-1], axis=0)[::-1] - contrib + (Tf[None, :, None] * bg[None, None, :])
            one_m = np.where(valid, 1.0 - a, 1.0)
            dL_da = (dC[None, :, :] * (colr[:, None, :] * Tin[:, :, None] - behind / one_m[:, :, None])).sum(2)
            dL_da += dA[None, :] * Tf[None, :] / one_m
            dL_da = np.where(valid & ~capped, dL_da, 0.0)
            dL_dcol = (wgt[:, :, None] * dC[None, :, :]).sum(1)      # (K, 3)
            dL_dpw = dL_da * a
            terms = [dL_dpw * (ia * dx + ib * dy), dL_dpw * (ic * dy + ib * dx), dL_dpw * (-0.5 * dx * dx),
                     dL_dpw * (-dx * dy), dL_dpw * (-0.5 * dy * dy), dL_da * ex]
            g = np.zeros((K, 9))
            for j, tm in enumerate(terms):
                g[:, j] = tm.sum(1)
            g[:, 6:9] = dL_dcol
            np.add.at(g2d, e, g)
            if with_abs:
                ga = np.zeros((K, 9))
                for j, tm in enumerate(terms):
                    ga[:, j] = np.abs(tm).sum(1)
                ga[:, 6:9] = (wgt[:, :, None] * np.abs(dC)[None, :, :]).sum(1)
                np.add.at(gabs, e, ga)
    return (g2d, gabs) if with_abs else g2d


def reference_gradient(U, packed, order, frame: dict, d_out: np.ndarray, with_scale: bool = False,
                       screen_f32: bool = False, trajectory: str = "f64"):
    """dL/d(parameters) per splat id in the layouts of hdsr_scene_views, for
    dL/d(output rgba) = d_out, in FP64. With `with_scale`, also (second
    value) per parameter the sum over pixels of the absolute value of each
    pixel's contribution (through the same chain rule, term by term): the
    magnitude against which an fp32 evaluation of the gradient's sums is
    rounded, used to bound the error such an evaluation may carry.

    With `screen_f32`, the composite reads the screen-space parameters
    (centre, conic, opacity, colour) rounded to f32, as the projection cache
    holds them (its centre and conic words are f32), the derivatives of the
    projection staying FP64: the FP64 gradient of the frame as the fp32
    cache defines it. Splat centres lie hundreds to thousands of pixels from
    the origin, where an f32 centre is good to ~1e-4 px, which alone moves
    some gradients by up to ~1e-2 relative (where a gradient sums many
    opposing pixel terms). `trajectory`: see composite_adjoint."""
    screen, visible, lay = project_dual(U, packed, order)
    if screen_f32:
        screen = {k: Dual(v.v.astype(np.float32).astype(np.float64), v.d) for k, v in screen.items()}
    res = composite_adjoint(U, screen, frame, np.asarray(d_out, np.float64), with_abs=with_scale,
                            trajectory=trajectory)
    g2d, gabs = res if with_scale else (res, None)
    keys = ("cx", "cy", "ia", "ib", "ic", "op", "r", "g", "b")
    n = int(packed.count)
    ids = np.asarray(order, np.int64)

    def per_splat(rows, absolute):
        if absolute:
            pr = sum(np.abs(screen[k].d) * rows[:, i:i + 1] for i, k in enumerate(keys))
        else:
            pr = sum(screen[k].d * rows[:, i:i + 1] for i, k in enumerate(keys))
        pr[~visible] = 0.0
        per_id = np.zeros_like(pr)
        per_id[ids] = pr
        out = {name: per_id[:, lay[name]] for name in ("positions", "log_scales", "rotations", "opacities", "sh")}
        out["opacities"] = out["opacities"].reshape(n)
        out["sh"] = out["sh"].copy()
        out["sh"][:, lay["sh_width"] - 3:] = 0.0  # emissive slots: no effect on the colour output
        return out

    grads = per_splat(g2d, False)
    return (grads, per_splat(gabs, True)) if with_scale else grads


def _morton(x: int, y: int) -> int:
    out = 0
    for i in range(16):
        out |= ((x >> i) & 1) << (2 * i) | ((y >> i) & 1) << (2 * i + 1)
    return out


def threshold_adjacent_ranks(U, par, frame, rel=1e-4) -> set:
    """sortRanks left out of exact gradient checks, traced in FP64 over the
    frame's entry lists (par: orc_project_f64's (N, 10) array): those whose
    opacity or colour sits at a clamp, and, for every pixel where some entry
    lies within `rel` of a composite threshold (power -4, alpha 1/255, the
    0.99 cap, T 0.001), every entry taken in that pixel. There fp32 and FP64
    may decide the comparison differently, and a decision that differs
    changes the transmittance of every entry behind it and the light behind
    every entry in front of it, i.e. the gradients of all of the pixel's
    entries, not only its own."""
    U = np.asarray(U, np.float32)
    Uu = U.view(np.uint32)
    cols, rows = int(Uu[20]), int(Uu[21])
    W, H = int(U[16]), int(U[17])
    counts, offs, ents = frame["tile_counts"], frame["tile_offsets"], frame["tile_entries"]
    flagged = set()
    op = par[:, 5]
    flagged.update(int(r) for r in np.nonzero((np.abs(op - 0.99) < rel) | (op == 0.0))[0])
    col = par[:, 6:9]
    flagged.update(int(r) for r in np.nonzero(((col < rel) | (col > 1 - rel)).any(1))[0])
    gy, gx = np.mgrid[0:16, 0:16]
    for ty in range(rows):
        for tx in range(cols):
            t = _morton(tx, ty)
            K = int(counts[t])
            if K == 0:
                continue
            X = (tx * 16 + gx).reshape(-1)
            Y = (ty * 16 + gy).reshape(-1)
            inside = (X < W) & (Y < H)
            px, py = X[inside] + 0.5, Y[inside] + 0.5
            e = np.asarray(ents[int(offs[t]): int(offs[t]) + K], np.int64)
            p = par[e]
            dx, dy = px[None, :] - p[:, 0:1], py[None, :] - p[:, 1:2]
            pw = -0.5 * p[:, 2:3] * dx * dx - 0.5 * p[:, 4:5] * dy * dy - p[:, 3:4] * dx * dy
            raw = p[:, 5:6] * np.exp(pw)
            a = np.minimum(raw, 0.99)
            cond = (pw > -4.0) & (a > 1.0 / 255.0)
            fac = np.where(cond, 1.0 - a, 1.0)
            G = np.vstack([np.ones((1, fac.shape[1])), np.cumprod(fac, axis=0)[:-1]])
            near = (np.abs(pw + 4.0) < 4.0 * rel) | (np.abs(a * 255.0 - 1.0) < rel) | \
                   (np.abs(raw / 0.99 - 1.0) < rel) | (np.abs(G / 0.001 - 1.0) < rel)
            # an entry after the saturation point changes nothing; a T near
            # the cutoff still matters at the entry that meets it
            sat = np.maximum.accumulate(G < 0.001 * (1 - rel), axis=0)
            near = near & ~np.vstack([np.zeros((1, sat.shape[1]), bool), sat[:-1]])
            valid = cond & (G >= 0.001)
            pix = near.any(0)
            hit = near.any(1) | (valid[:, pix].any(1) if pix.any() else np.zeros(K, bool))
            flagged.update(int(x) for x in e[hit])
    return flagged
