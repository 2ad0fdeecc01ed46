// hdsr_proj_adjoint.cuh — the projection of one splat recomputed with every
// intermediate its adjoint needs (gpu_project_splats.wgsl:112-358, colour and
// 2D conic), in the scalar type HDSR_BWD_REAL chosen by the including unit
// (both use double-float, df64, by default; fp64 on request: for splats seen
// nearly edge-on the conic and its adjoint combine large terms that cancel,
// and at fp32 a few gradients land 1e-3 to 1e-2 from the FP64 ones).
#pragma once
#include "hdsr_df64.cuh"
#include "hdsr_internal.cuh"

namespace hdsr {
namespace {

// Scalar type of the recompute (HDSR_BWD_REAL, set by the including unit).
#ifndef HDSR_BWD_REAL
#error "define HDSR_BWD_REAL (float, double or df64) before including hdsr_proj_adjoint.cuh"
#endif
using real = HDSR_BWD_REAL;
__device__ __forceinline__ float rsqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double rsqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ df64 rsqrt_(df64 x) { return df_sqrt(x); }
__device__ __forceinline__ float rexp_(float x) { return hx_expf(x); }
__device__ __forceinline__ double rexp_(double x) { return exp(x); }
__device__ __forceinline__ real rmax_(real a, real b) { return a > b ? a : b; }
__device__ __forceinline__ real rmin_(real a, real b) { return a < b ? a : b; }
__device__ __forceinline__ real rclamp_(real x, real lo, real hi) { return rmin_(rmax_(x, lo), hi); }

struct F3 { real x, y, z; };
__device__ __forceinline__ F3 f3(real x, real y, real z) { return F3{x, y, z}; }
__device__ __forceinline__ real dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 mul(F3 a, real s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Projection of one splat, recomputed in fp32 with every intermediate the
// adjoint needs (gpu_project_splats.wgsl:112-358, colour part and 2D conic).
struct Proj {
  F3 p;
  real clip[4], safeW;
  bool w_free;          // safeW == clip[3] (not clamped to 1e-4)
  real vc[3], vz;
  bool vz_free;         // vz == vc[2]
  real fx, fy, J1x, J1y, J2x, J2y;
  F3 w0, w1, w2, tt0, tt1;
  real qn[4], qlen;    // normalised quaternion (w, x, y, z), its length
  F3 R[3];              // rotated unit axes (columns of R)
  real s[3];           // axis scales exp(logScale) * splatScale
  F3 ax[3];
  F3 b0, b1, cr;         // b0_i = ax_i . tt0, b1_i = ax_i . tt1, cr = b0 x b1
  real XXr, XY, YYr, detOrig, cXX, cYY, D, ratio, aa;
  real cx, cy;
  real op_in, op_aa;   // input opacity, opacity * aa (before the clamp)
  F3 cam, dir;
  real dlen;
  real craw[3];        // SH colour before the clamp
};

__device__ __forceinline__ real ld(const float* p) { return (real)__ldg(p); }

__device__ void proj_recompute(const FrameArgs& a, uint32_t id, Proj& P) {
  const float* U = a.U;
  const float* pp = a.pos + (uint64_t)id * 3;
  P.p = f3(ld(pp), ld(pp + 1), ld(pp + 2));
#pragma unroll
  for (int k = 0; k < 4; ++k)
    P.clip[k] = ((ld(U + k) * P.p.x + ld(U + 4 + k) * P.p.y) + ld(U + 8 + k) * P.p.z) + ld(U + 12 + k);
  P.safeW = rmax_(P.clip[3], 0.0001f);
  P.w_free = P.clip[3] > 0.0001f;
  P.cx = (P.clip[0] / P.safeW * 0.5f + 0.5f) * ld(U + 16);
  P.cy = (1.0f - (P.clip[1] / P.safeW * 0.5f + 0.5f)) * ld(U + 17);
  // axes
  const float4 q = __ldg(reinterpret_cast<const float4*>(a.rot) + id);
  const real qx = q.x, qy = q.y, qz = q.z, qw = q.w;
  P.qlen = rsqrt_(qx * qx + qy * qy + qz * qz + qw * qw);
  const real iq = real(1) / rmax_(P.qlen, 0.000001f);
  P.qn[0] = qx * iq; P.qn[1] = qy * iq; P.qn[2] = qz * iq; P.qn[3] = qw * iq;
  const real w = P.qn[0], x = P.qn[1], y = P.qn[2], z = P.qn[3];
  P.R[0] = f3(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + w * z), 2.0f * (x * z - w * y));
  P.R[1] = f3(2.0f * (x * y - w * z), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + w * x));
  P.R[2] = f3(2.0f * (x * z + w * y), 2.0f * (y * z - w * x), 1.0f - 2.0f * (x * x + y * y));
  const float* sl = a.scl + (uint64_t)id * 3;
  const real ss = ld(U + 24);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    // exp at fp32: an error in s_i scales b0_i and b1_i alike, so the
    // near-parallel cancellation of the conic does not amplify it
    P.s[i] = (real)hx_expf(__ldg(sl + i)) * ss;
    P.ax[i] = mul(P.R[i], P.s[i]);
  }
  // Jacobian of the perspective projection in view space
#pragma unroll
  for (int k = 0; k < 3; ++k)
    P.vc[k] = ((ld(U + 32 + k) * P.p.x + ld(U + 36 + k) * P.p.y) + ld(U + 40 + k) * P.p.z) + ld(U + 44 + k);
  P.vz = rmin_(P.vc[2], -0.001f);
  P.vz_free = P.vc[2] < -0.001f;
  P.fx = ld(U + 48);
  P.fy = ld(U + 49);
  const real ivz = real(1) / P.vz;
  P.J1x = P.fx * ivz;
  P.J1y = P.fy * ivz;
  P.J2x = (-P.J1x * ivz) * P.vc[0];
  P.J2y = (-P.J1y * ivz) * P.vc[1];
  P.w0 = f3(ld(U + 32), ld(U + 36), ld(U + 40));
  P.w1 = f3(ld(U + 33), ld(U + 37), ld(U + 41));
  P.w2 = f3(ld(U + 34), ld(U + 38), ld(U + 42));
  P.tt0 = add(mul(P.w0, P.J1x), mul(P.w2, P.J2x));
  P.tt1 = add(mul(P.w1, P.J1y), mul(P.w2, P.J2y));
  P.b0 = f3(dot(P.ax[0], P.tt0), dot(P.ax[1], P.tt0), dot(P.ax[2], P.tt0));
  P.b1 = f3(dot(P.ax[0], P.tt1), dot(P.ax[1], P.tt1), dot(P.ax[2], P.tt1));
  P.XXr = dot(P.b0, P.b0);
  P.XY = dot(P.b0, P.b1);
  P.YYr = dot(P.b1, P.b1);
  P.cr = cross(P.b0, P.b1);
  P.detOrig = dot(P.cr, P.cr);
  P.cXX = P.XXr + 0.3f;
  P.cYY = P.YYr + 0.3f;
  P.D = P.detOrig + 0.3f * (P.XXr + P.YYr) + 0.09f;  // >= 0.09: never below the 1e-6 floor
  P.ratio = P.detOrig / P.D;
  P.aa = rsqrt_(P.ratio);
  P.op_in = ld(a.opa + id);
  P.op_aa = P.op_in * P.aa;
  // SH colour (WGSL basis and signs)
  P.cam = f3(ld(U + 28), ld(U + 29), ld(U + 30));
  const F3 dv = sub(P.cam, P.p);
  P.dlen = rsqrt_(dot(dv, dv));
  const real idl = real(1) / P.dlen;
  P.dir = f3(dv.x * idl, dv.y * idl, dv.z * idl);
  const uint32_t deg = f2u(__ldg(U + 25));
  const uint32_t shStride = ((deg + 1) * (deg + 1) - 1) * 3;
  const float* sh = a.sh + (uint64_t)id * (3 + shStride + 3);
  real basis[15];
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
  const uint32_t nb = (deg + 1) * (deg + 1) - 1;
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    real c = ld(sh + ch);
    for (uint32_t k = 0; k < nb && k < 15u; ++k) c += ld(sh + 3 + 3 * k + ch) * basis[k];
    P.craw[ch] = c;
  }
}

// d(basis_k)/d(dir), k < 15 (same order as proj_recompute)
__device__ __forceinline__ F3 dbasis(int k, F3 v) {
  const real vx = v.x, vy = v.y, vz = v.z, xx = vx * vx, yy = vy * vy, zz = vz * vz;
  const real C1 = 0.4886025119029199f, A = 1.0925484305920792f, B = 0.31539156525252005f;
  const real Cc = 0.5462742152960396f, Dd = 0.5900435899266435f, E = 2.890611442640554f;
  const real Ff = 0.4570457994644658f, G = 0.3731763325901154f, Hh = 1.445305721320277f;
  switch (k) {
    case 0: return f3(0.0f, C1, 0.0f);
    case 1: return f3(0.0f, 0.0f, C1);
    case 2: return f3(C1, 0.0f, 0.0f);
    case 3: return f3(A * vy, A * vx, 0.0f);
    case 4: return f3(0.0f, A * vz, A * vy);
    case 5: return f3(-2.0f * B * vx, -2.0f * B * vy, 4.0f * B * vz);
    case 6: return f3(A * vz, 0.0f, A * vx);
    case 7: return f3(2.0f * Cc * vx, -2.0f * Cc * vy, 0.0f);
    case 8: return f3(6.0f * Dd * vx * vy, Dd * (3.0f * xx - 3.0f * yy), 0.0f);
    case 9: return f3(E * vy * vz, E * vx * vz, E * vx * vy);
    case 10: return f3(-2.0f * Ff * vx * vy, Ff * (4.0f * zz - xx - 3.0f * yy), 8.0f * Ff * vy * vz);
    case 11: return f3(-6.0f * G * vx * vz, -6.0f * G * vy * vz, G * (6.0f * zz - 3.0f * xx - 3.0f * yy));
    case 12: return f3(Ff * (4.0f * zz - 3.0f * xx - yy), -2.0f * Ff * vx * vy, 8.0f * Ff * vx * vz);
    case 13: return f3(2.0f * Hh * vx * vz, -2.0f * Hh * vy * vz, Hh * (xx - yy));
    default: return f3(Dd * (3.0f * xx - 3.0f * yy), -6.0f * Dd * vx * vy, 0.0f);
  }
}

}  // namespace
}  // namespace hdsr
