// hdsr_backward.cu — the adjoint of one frame: dL/d(colour image) ->
// dL/d(positions, log-scales, rotations, opacities, SH coefficients).
//
// No reference counterpart (the reference renders only). The differentiated
// function is the frame's mathematics at fp32: the cache's f16 opacity and
// colour are taken unrounded, and the 2D conic is evaluated without the
// cancellation of XX*YY - XY^2 (detOrig = |b0 x b1|^2, the Lagrange identity,
// and detBlur = detOrig + 0.3 (XX + YY) + 0.09), which for splats seen
// edge-on (a nearly singular covariance) loses several digits in fp32.
// Every threshold of the composite (power > -4, alpha > 1/255, T >= 0.001,
// the 0.99 alpha cap) and every clamp of the projection (opacity, colour,
// view depth, w) is held fixed: a clamped quantity passes no gradient. The
// forward frame's superblock lists are walked again (no per-tile lists).
//   1. k_bwd_prep: per sortRank, the screen-space parameters of the adjoint
//      (centre, conic, clamped opacity with the anti-aliasing factor, clamped
//      SH colour); zeroes the screen-space accumulators.
//   2. k_raster_bwd: one warp per half tile (rows 0-7 or 8-15, from an atomic
//      counter), each lane one 2x2 quad. Pass A recomputes the composite
//      front to back and keeps, per pixel, the final transmittance T_f and
//      output O = sum c_k w_k + bg T_f. Pass B walks the same entries again:
//      with C_k = sum_{j<=k} c_j w_j, the light behind entry k is O - C_k, so
//        dL/dalpha_k = sum_ch dL/dO_ch (c_k,ch T_k - (O_ch - C_k,ch) / (1 -
//                      alpha_k)) + dL/dA T_f / (1 - alpha_k),   A = 1 - T_f,
//      and dL/dc_k = dL/dO w_k. Per entry the warp sums its lanes' values
//      (butterfly shuffles) and one lane adds them to the entry's accumulators.
//   3. k_project_bwd: per sortRank, recompute the projection (double-float) and apply
//      the chain rule back to the scene arrays (atomic adds: a splat id may
//      appear in sortedIndices more than once).
#ifndef HDSR_BWD_REAL
#define HDSR_BWD_REAL df64
#endif
#include "hdsr_proj_adjoint.cuh"

namespace hdsr {

namespace {

constexpr float kBgR = 0.02f, kBgG = 0.02f, kBgB = 0.04f;  // composite background (T-weighted)

constexpr int kBwdWarps = 4;
// A staged entry is four float4 rows, read with broadcast 16-byte loads:
//   row 0: cx, cy, -ia/2, -ib   row 1: -ic/2, opacity, r, g
//   row 2: b, ia, ib, ic        row 3: sortRank bits, 0, 0, 0
constexpr int kBRows = 4;

// One entry's adjoint parameters as loaded (a batch ahead of its use).
struct BwdRow {
  float4 p0, p1, p2;
  uint32_t r;
};

__device__ __forceinline__ void bwd_load(const BwdArgs& b, BwdRow& w, uint32_t r) {
  w.p0 = b.par[(size_t)r * 3];
  w.p1 = b.par[(size_t)r * 3 + 1];
  w.p2 = b.par[(size_t)r * 3 + 2];
  w.r = r;
}

// Stages the loaded entry, in order, if it can reach the half tile
// [x0, x0 + 15] x [y0, y0 + 7]; returns how many of the batch were kept
// (warp-collective: every lane calls it, lanes without an entry pass
// valid = false).
__device__ __forceinline__ uint32_t bwd_stage_kept(float4 (*s)[kBRows], const BwdRow& w, bool valid, uint32_t lane,
                                                   float x0, float y0) {
  const bool keep =
      valid && reaches_rect(w.p0.x, w.p0.y, w.p0.z, w.p0.w, w.p1.x, w.p1.y, x0, x0 + 15.0f, y0, y0 + 7.0f);
  const uint32_t kept = __ballot_sync(0xFFFFFFFFu, keep);
  if (keep) {
    const uint32_t k = __popc(kept & ((1u << lane) - 1u));
    s[k][0] = make_float4(w.p0.x, w.p0.y, w.p0.z * -0.5f, -w.p0.w);
    s[k][1] = make_float4(w.p1.x * -0.5f, w.p1.y, w.p1.z, w.p1.w);
    s[k][2] = make_float4(w.p2.x, w.p0.z, w.p0.w, w.p1.x);
    s[k][3] = make_float4(u2f(w.r), 0.0f, 0.0f, 0.0f);
  }
  return __popc(kept);
}

// Warp sums of 9 values (padded to 16) by recursive halving: at each step a
// lane keeps half of its values, receives its partner's partial sums of that
// half and sends the other half (8 + 4 + 2 + 1 shuffles, then 1 to finish).
// On return lanes 2k and 2k+1 hold the sum of value k' = bits 4..1 of the
// lane; returns that index (>= 9: padding).
__device__ __forceinline__ uint32_t warp_sum9(const float (&g)[9], uint32_t lane, float& out) {
  float v[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = j < 9 ? g[j] : 0.0f;
#pragma unroll
  for (int h = 8; h >= 1; h >>= 1) {
    const bool upper = (lane & (uint32_t)(2 * h)) != 0u;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const float send = upper ? v[j] : v[j + h];
      const float keep = upper ? v[j + h] : v[j];
      v[j] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 2 * h);
    }
  }
  out = v[0] + __shfl_xor_sync(0xFFFFFFFFu, v[0], 1);
  return ((lane >> 1) & 1u) | (((lane >> 2) & 1u) << 1) | (((lane >> 3) & 1u) << 2) | (((lane >> 4) & 1u) << 3);
}

__global__ void __launch_bounds__(kBwdWarps * 32) k_raster_bwd(BwdArgs b) {
  __shared__ float4 s_pay[kBwdWarps][32][kBRows];
  __shared__ uint32_t s_queue[kBwdWarps][kWalkQueue];
  const FrameArgs& a = b.f;
  if (a.ctl[kCtlFlags] & kSkipFlags) return;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  float4 (*s)[kBRows] = s_pay[warp];
  const uint32_t items = 2u * a.tile_count;
  for (;;) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(a.ctl + kCtlBwdTile, 1u);
    item = __shfl_sync(0xFFFFFFFFu, item, 0);
    if (item >= items) break;
    const uint32_t tile = a.tile_order[item >> 1], half = item & 1u;
    const uint32_t tx = tile & 0xFFFFu, ty = tile >> 16;
    const uint32_t bx = tx * 16u + (lane & 7u) * 2u;
    const uint32_t by = ty * 16u + ((lane >> 3) + 4u * half) * 2u;
    const float p00x = (float)bx + 0.5f, p00y = (float)by + 0.5f;
    float dxv[4], dyv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      dxv[k] = p00x + (float)(k & 1);
      dyv[k] = p00y + (float)(k >> 1);
    }
    // pass A: forward recompute
    float T[4], C[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k) { T[k] = 1.0f; C[k][0] = C[k][1] = C[k][2] = 0.0f; }
    bool done = false;
    uint32_t n_end = 0;
    const float rx0 = (float)(tx * 16u) + 0.5f, ry0 = (float)(ty * 16u + 8u * half) + 0.5f;
    TileWalk walk;
    walk.start(a, tx, ty, s_queue[warp]);
    BwdRow cur;
    uint32_t rank = 0;
    uint32_t nb = walk.take(a, lane, 32u, rank);
    if (lane < nb) bwd_load(b, cur, rank);
    while (nb > 0u) {
      const uint32_t n = bwd_stage_kept(s, cur, lane < nb, lane, rx0, ry0);
      // the next batch's parameters in flight while this one is composited
      const uint32_t nb2 = walk.take(a, lane, 32u, rank);
      if (lane < nb2) bwd_load(b, cur, rank);
      __syncwarp();
      for (uint32_t i = 0; i < n && !done; ++i) {
        const float4 r0 = s[i][0], r1 = s[i][1];
        const float cx = r0.x, cy = r0.y, ka = r0.z, kb = r0.w, kc = r1.x;
        const float op = r1.y;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float dx = dxv[k] - cx, dy = dyv[k] - cy;
          const float pw = fmaf(kc * dy, dy, fmaf(kb * dx, dy, (ka * dx) * dx));
          const float al = mn(0.99f, op * splat_expf(pw));
          const bool valid = (pw > -4.0f) && (al > (1.0f / 255.0f)) && (T[k] >= 0.001f);
          if (valid) {
            const float w = al * T[k];
            C[k][0] = fmaf(r1.z, w, C[k][0]);
            C[k][1] = fmaf(r1.w, w, C[k][1]);
            C[k][2] = fmaf(s[i][2].x, w, C[k][2]);
            T[k] = T[k] * (1.0f - al);
          }
        }
        done = T[0] < 0.001f && T[1] < 0.001f && T[2] < 0.001f && T[3] < 0.001f;
      }
      __syncwarp();
      n_end += nb;
      if (__all_sync(0xFFFFFFFFu, done)) break;
      nb = nb2;
    }
    // outputs and their incoming gradients (pixels outside the image: none)
    float O[4][3], Tf[4], gO[4][3], gA[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      Tf[k] = T[k];
      O[k][0] = fmaf(T[k], kBgR, C[k][0]);
      O[k][1] = fmaf(T[k], kBgG, C[k][1]);
      O[k][2] = fmaf(T[k], kBgB, C[k][2]);
      const uint32_t px = bx + (uint32_t)(k & 1), py = by + (uint32_t)(k >> 1);
      float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (px < a.W && py < a.H)
        g = reinterpret_cast<const float4*>(reinterpret_cast<const char*>(b.d_color) + (size_t)py * b.d_color_pitch)[px];
      gO[k][0] = g.x; gO[k][1] = g.y; gO[k][2] = g.z; gA[k] = g.w;
      T[k] = 1.0f;
      C[k][0] = C[k][1] = C[k][2] = 0.0f;
    }
    // pass B: gradients, the same n_end entries in the same order
    walk.start(a, tx, ty, s_queue[warp]);
    nb = walk.take(a, lane, n_end < 32u ? n_end : 32u, rank);
    uint32_t b0 = nb;
    if (lane < nb) bwd_load(b, cur, rank);
    while (nb > 0u) {
      const uint32_t n = bwd_stage_kept(s, cur, lane < nb, lane, rx0, ry0);
      const uint32_t nb2 = walk.take(a, lane, n_end - b0 < 32u ? n_end - b0 : 32u, rank);
      b0 += nb2;
      if (lane < nb2) bwd_load(b, cur, rank);
      __syncwarp();
      for (uint32_t i = 0; i < n; ++i) {
        const float4 r0 = s[i][0], r1 = s[i][1], r2 = s[i][2];
        const float cx = r0.x, cy = r0.y, ka = r0.z, kb = r0.w, kc = r1.x;
        const float op = r1.y, cr = r1.z, cg = r1.w, cb = r2.x;
        const float ia = r2.y, ib = r2.z, ic = r2.w;
        float g[9] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        bool any = false;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float dx = dxv[k] - cx, dy = dyv[k] - cy;
          const float pw = fmaf(kc * dy, dy, fmaf(kb * dx, dy, (ka * dx) * dx));
          const float ge = splat_expf(pw);
          const float raw = op * ge;
          const float al = mn(0.99f, raw);
          const bool valid = (pw > -4.0f) && (al > (1.0f / 255.0f)) && (T[k] >= 0.001f);
          if (!valid) continue;
          any = true;
          const float w = al * T[k];
          C[k][0] = fmaf(cr, w, C[k][0]);
          C[k][1] = fmaf(cg, w, C[k][1]);
          C[k][2] = fmaf(cb, w, C[k][2]);
          // 1 - alpha is in [0.01, 1]: the approximate reciprocal (2 ulp)
          // is far inside the gradient's tolerance
          const float inv1m = __fdividef(1.0f, 1.0f - al);
          float dal = gO[k][0] * (cr * T[k] - (O[k][0] - C[k][0]) * inv1m) +
                      gO[k][1] * (cg * T[k] - (O[k][1] - C[k][1]) * inv1m) +
                      gO[k][2] * (cb * T[k] - (O[k][2] - C[k][2]) * inv1m) + gA[k] * Tf[k] * inv1m;
          g[6] += gO[k][0] * w;
          g[7] += gO[k][1] * w;
          g[8] += gO[k][2] * w;
          if (raw < 0.99f) {
            g[5] += dal * ge;
            const float dpw = dal * raw;
            g[0] += dpw * (ia * dx + ib * dy);
            g[1] += dpw * (ib * dx + ic * dy);
            g[2] += dpw * (-0.5f * dx * dx);
            g[3] += dpw * (-dx * dy);
            g[4] += dpw * (-0.5f * dy * dy);
          }
          T[k] = T[k] * (1.0f - al);
        }
        if (__any_sync(0xFFFFFFFFu, any)) {
          float v;
          const uint32_t j = warp_sum9(g, lane, v);
          if (!(lane & 1u) && j < 9u && v != 0.0f) atomicAdd(b.g2d + (size_t)f2u(s[i][3].x) * kG2d + j, v);
        }
      }
      __syncwarp();
      nb = nb2;
    }
  }
}

__global__ void __launch_bounds__(128) k_project_bwd(BwdArgs b) {
  const FrameArgs& a = b.f;
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.N) return;
  if (a.aux[r].x == kSentinel) return;
  const float* gr = b.g2d + (size_t)r * kG2d;
  const real g_cx = gr[0], g_cy = gr[1], g_ia = gr[2], g_ib = gr[3], g_ic = gr[4];
  const real g_op = gr[5];
  const real g_col[3] = {gr[6], gr[7], gr[8]};
  if (g_cx == 0.0f && g_cy == 0.0f && g_ia == 0.0f && g_ib == 0.0f && g_ic == 0.0f && g_op == 0.0f &&
      g_col[0] == 0.0f && g_col[1] == 0.0f && g_col[2] == 0.0f)
    return;
  const uint32_t id = __ldg(a.sorted + r);
  Proj P;
  proj_recompute(a, id, P);
  const float* U = a.U;
  F3 g_p = f3(0.0f, 0.0f, 0.0f);

  // opacity = clamp(op * aa, 0, 0.99)
  real g_aa = 0.0f;
  if (P.op_aa > 0.0f && P.op_aa < 0.99f) {
    atomicAdd(b.d_opa + id, g_op * P.aa);
    g_aa = g_op * P.op_in;
  }
  // inverse conic: ia = cYY/D, ib = -XY/D, ic = cXX/D
  const real Di = 1.0f / P.D;
  real g_cXX = g_ic * Di, g_cYY = g_ia * Di, g_XY = -g_ib * Di;
  real g_D = -(g_ia * P.cYY - g_ib * P.XY + g_ic * P.cXX) * Di * Di;
  // aa = sqrt(detOrig / D)
  real g_detOrig = 0.0f;
  if (P.aa > 0.0f) {
    const real g_ratio = g_aa * 0.5f / P.aa;
    g_detOrig += g_ratio * Di;
    g_D -= g_ratio * P.detOrig * Di * Di;
  }
  // D = detOrig + 0.3 (XXr + YYr) + 0.09; cXX = XXr + 0.3, cYY = YYr + 0.3
  g_detOrig += g_D;
  const real g_XXr = g_cXX + 0.3f * g_D;
  const real g_YYr = g_cYY + 0.3f * g_D;
  // XXr = |b0|^2, XY = b0.b1, YYr = |b1|^2, detOrig = |b0 x b1|^2
  const F3 gb0 = add(add(mul(P.b0, 2.0f * g_XXr), mul(P.b1, g_XY)), mul(cross(P.b1, P.cr), 2.0f * g_detOrig));
  const F3 gb1 = add(add(mul(P.b1, 2.0f * g_YYr), mul(P.b0, g_XY)), mul(cross(P.cr, P.b0), 2.0f * g_detOrig));
  // b0_i = ax_i . tt0, b1_i = ax_i . tt1
  const real gb0v[3] = {gb0.x, gb0.y, gb0.z}, gb1v[3] = {gb1.x, gb1.y, gb1.z};
  F3 g_tt0 = f3(0.0f, 0.0f, 0.0f), g_tt1 = f3(0.0f, 0.0f, 0.0f);
  F3 g_ax[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    g_ax[i] = add(mul(P.tt0, gb0v[i]), mul(P.tt1, gb1v[i]));
    g_tt0 = add(g_tt0, mul(P.ax[i], gb0v[i]));
    g_tt1 = add(g_tt1, mul(P.ax[i], gb1v[i]));
  }
  // tt0 = J1x w0 + J2x w2, tt1 = J1y w1 + J2y w2
  const real g_J1x = dot(g_tt0, P.w0), g_J2x = dot(g_tt0, P.w2);
  const real g_J1y = dot(g_tt1, P.w1), g_J2y = dot(g_tt1, P.w2);
  // J1 = f / vz, J2 = -f vc / vz^2
  const real vz = P.vz, vz2 = vz * vz, vz3 = vz2 * vz;
  real g_vc[3];
  g_vc[0] = -g_J2x * P.fx / vz2;
  g_vc[1] = -g_J2y * P.fy / vz2;
  const real g_vz = -g_J1x * P.fx / vz2 - g_J1y * P.fy / vz2 + g_J2x * 2.0f * P.fx * P.vc[0] / vz3 +
                     g_J2y * 2.0f * P.fy * P.vc[1] / vz3;
  g_vc[2] = P.vz_free ? g_vz : 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) g_p = add(g_p, mul(f3(ld(U + 32 + k), ld(U + 36 + k), ld(U + 40 + k)), g_vc[k]));
  // axes: ax_i = R_i s_i, s_i = exp(logScale_i) * splatScale
  real gR[3][3];  // gR[i] = dL/d(column i)
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    atomicAdd(b.d_lsc + (size_t)id * 3 + i, dot(g_ax[i], P.R[i]) * P.s[i]);
    const F3 gc = mul(g_ax[i], P.s[i]);
    gR[i][0] = gc.x; gR[i][1] = gc.y; gR[i][2] = gc.z;
  }
  // R from (w, x, y, z); column i holds R[row][i] = gR[i][row]
  {
    const real w = P.qn[0], x = P.qn[1], y = P.qn[2], z = P.qn[3];
    // dL/dR_rc with r = row, c = column
    const real g00 = gR[0][0], g10 = gR[0][1], g20 = gR[0][2];
    const real g01 = gR[1][0], g11 = gR[1][1], g21 = gR[1][2];
    const real g02 = gR[2][0], g12 = gR[2][1], g22 = gR[2][2];
    const real gw = 2.0f * (-z * g01 + y * g02 + z * g10 - x * g12 - y * g20 + x * g21);
    const real gx = 2.0f * (y * g01 + z * g02 + y * g10 - 2.0f * x * g11 - w * g12 + z * g20 + w * g21 - 2.0f * x * g22);
    const real gy = 2.0f * (-2.0f * y * g00 + x * g01 + w * g02 + x * g10 + z * g12 - w * g20 + z * g21 - 2.0f * y * g22);
    const real gz = 2.0f * (-2.0f * z * g00 - w * g01 + x * g02 + w * g10 - 2.0f * z * g11 + y * g12 + x * g20 + y * g21);
    // q_hat = q / max(|q|, 1e-6)
    const real gq[4] = {gw, gx, gy, gz};
    const real qd = gw * w + gx * x + gy * y + gz * z;
    const real dn = rmax_(P.qlen, 0.000001f);
    const bool norm_free = P.qlen > 0.000001f;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      atomicAdd(b.d_rot + (size_t)id * 4 + k, (gq[k] - (norm_free ? P.qn[k] * qd : 0.0f)) / dn);
  }
  // centre: cpx = (clip0/safeW * 0.5 + 0.5) W, cpy = (1 - (clip1/safeW * 0.5 + 0.5)) H
  {
    const real vpW = ld(U + 16), vpH = ld(U + 17);
    const real g_nx = g_cx * 0.5f * vpW, g_ny = -g_cy * 0.5f * vpH;
    real g_clip[4];
    g_clip[0] = g_nx / P.safeW;
    g_clip[1] = g_ny / P.safeW;
    g_clip[2] = 0.0f;
    g_clip[3] = P.w_free ? -(g_nx * P.clip[0] + g_ny * P.clip[1]) / (P.safeW * P.safeW) : 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) g_p = add(g_p, mul(f3(ld(U + k), ld(U + 4 + k), ld(U + 8 + k)), g_clip[k]));
  }
  // colour = clamp(SH(dir), 0, 1), dir = normalize(cam - p)
  {
    const uint32_t deg = f2u(__ldg(U + 25));
    const uint32_t nb = (deg + 1) * (deg + 1) - 1;
    const uint32_t shStride = nb * 3;
    const uint64_t base = (uint64_t)id * (3 + shStride + 3);
    const float* sh = a.sh + base;
    real basis[15];
    {
      const real vx = P.dir.x, vy = P.dir.y, vzz = P.dir.z;
      const real xx = vx * vx, yy = vy * vy, zz = vzz * vzz;
      basis[0] = 0.4886025119029199f * vy;
      basis[1] = 0.4886025119029199f * vzz;
      basis[2] = 0.4886025119029199f * vx;
      basis[3] = 1.0925484305920792f * vx * vy;
      basis[4] = 1.0925484305920792f * vy * vzz;
      basis[5] = 0.31539156525252005f * ((2.0f * zz - xx) - yy);
      basis[6] = 1.0925484305920792f * vx * vzz;
      basis[7] = 0.5462742152960396f * (xx - yy);
      basis[8] = 0.5900435899266435f * vy * (3.0f * xx - yy);
      basis[9] = 2.890611442640554f * vx * vy * vzz;
      basis[10] = 0.4570457994644658f * vy * ((4.0f * zz - xx) - yy);
      basis[11] = 0.3731763325901154f * vzz * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
      basis[12] = 0.4570457994644658f * vx * ((4.0f * zz - xx) - yy);
      basis[13] = 1.445305721320277f * vzz * (xx - yy);
      basis[14] = 0.5900435899266435f * vx * (xx - 3.0f * yy);
    }
    F3 g_dir = f3(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      if (!(P.craw[ch] > 0.0f && P.craw[ch] < 1.0f) || g_col[ch] == 0.0f) continue;
      const real gc = g_col[ch];
      atomicAdd(b.d_sh + base + ch, gc);
      for (uint32_t k = 0; k < nb && k < 15u; ++k) {
        atomicAdd(b.d_sh + base + 3 + 3 * k + ch, gc * basis[k]);
        g_dir = add(g_dir, mul(dbasis((int)k, P.dir), gc * ld(sh + 3 + 3 * k + ch)));
      }
    }
    if (nb) {
      const real proj = dot(g_dir, P.dir);
      const F3 g_d = mul(sub(g_dir, mul(P.dir, proj)), 1.0f / P.dlen);
      g_p = sub(g_p, g_d);
    }
  }
  atomicAdd(b.d_pos + (size_t)id * 3 + 0, g_p.x);
  atomicAdd(b.d_pos + (size_t)id * 3 + 1, g_p.y);
  atomicAdd(b.d_pos + (size_t)id * 3 + 2, g_p.z);
}

}  // namespace

cudaError_t launch_backward(const BwdArgs& b, cudaStream_t s) {
  const FrameArgs& a = b.f;
  cudaError_t e = launch_bwd_prep(b, s);
  if (e != cudaSuccess) return e;
  if (a.tile_count) {
    const uint32_t want = (2u * a.tile_count + kBwdWarps - 1) / kBwdWarps;
    const uint32_t cap = (uint32_t)a.num_sms * 8u;
    k_raster_bwd<<<want < cap ? want : cap, kBwdWarps * 32, 0, s>>>(b);
  }
  if (a.N) k_project_bwd<<<(a.N + 127) / 128, 128, 0, s>>>(b);
  return cudaGetLastError();
}

}  // namespace hdsr
