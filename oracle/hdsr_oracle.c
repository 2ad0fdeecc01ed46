/*
 * hdsr_oracle.c — CPU restatement of the reference compute compositor.
 * TEST INFRASTRUCTURE ONLY (see hdsr_oracle.h for scope, canonical order and
 * parity status). Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp -fPIC
 * -shared hdsr_oracle.c -lm. The -ffp-contract=off is part of the definition:
 * every multiply-add below rounds twice unless it is an explicit fmaf().
 */
#include "hdsr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PROJ_STRIDE 14u
#define SENTINEL 0xFFFFFFFFu
#define LARGE_SPLAT_TILE_THRESHOLD 16u
#define MAX_LARGE_SPLATS 65535u
#define MAX_TILE_ENTRIES 4096u
#define NUM_BUCKETS 128u
#define MAX_CHUNKS 1024u
#define KEY20_MAX 0xFFFFFu

static inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float bitsf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline float Uf(const float* U, int i) { return U[i]; }
static inline uint32_t Uu(const float* U, int i) { return fbits(U[i]); }

/* WGSL min/max/clamp on f32 (no NaN inputs on the defined path). */
static inline float fmin_(float a, float b) { return a < b ? a : b; }
static inline float fmax_(float a, float b) { return a > b ? a : b; }
static inline float clampf_(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }
/* WGSL u32(f32): truncate toward zero, saturate, NaN -> 0. */
static inline uint32_t sat_u32(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}

/* ---------------------------------------------------------------------------
 * exp/log: own implementations, identical op sequence to the CUDA kernels.
 * exp: Cody-Waite reduction by ln2 (hi/lo split), degree-7 Taylor polynomial
 * in Horner form with fma, two-step power-of-two scaling.
 * log: x = m*2^e with m in [sqrt(1/2), sqrt(2)], s = (m-1)/(m+1),
 * log(m) = 2*atanh(s) = 2s + 2s^3/3 + 2s^5/5 + 2s^7/7 + 2s^9/9.
 * ------------------------------------------------------------------------- */
#define EXP_HI 88.72283935546875f
#define EXP_LO (-103.97208404541015625f)
#define LOG2E_F 1.44269502162933349609375f
#define LN2_HI 0.693145751953125f
#define LN2_LO 1.428606765330187045e-06f

static inline float pow2i(int k) { return bitsf((uint32_t)(k + 127) << 23); } /* k in [-126,127] */

float orc_expf(float x) {
  if (x != x) return x;
  if (x > EXP_HI) return INFINITY;
  if (x < EXP_LO) return 0.0f;
  float k = rintf(x * LOG2E_F);
  float r = fmaf(k, -LN2_HI, x);
  r = fmaf(k, -LN2_LO, r);
  float p = 1.98412701e-04f;         /* 1/7! */
  p = fmaf(p, r, 1.38888892e-03f);   /* 1/6! */
  p = fmaf(p, r, 8.33333377e-03f);   /* 1/5! */
  p = fmaf(p, r, 4.16666679e-02f);   /* 1/4! */
  p = fmaf(p, r, 1.66666672e-01f);   /* 1/3! */
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int ki = (int)k;
  int k1 = ki / 2;
  int k2 = ki - k1;
  return (p * pow2i(k1)) * pow2i(k2);
}

float orc_logf(float x) {
  if (x != x) return x;
  if (x < 0.0f) return NAN;
  if (x == 0.0f) return -INFINITY;
  if (x == INFINITY) return x;
  uint32_t b = fbits(x);
  int e = 0;
  if (b < 0x00800000u) { x = x * 8388608.0f; b = fbits(x); e = -23; }
  e += (int)(b >> 23) - 127;
  float m = bitsf((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421353816986083984375f) { m = m * 0.5f; e += 1; }
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  float q = 2.22222224e-01f;         /* 2/9 */
  q = fmaf(q, z, 2.85714298e-01f);   /* 2/7 */
  q = fmaf(q, z, 4.00000006e-01f);   /* 2/5 */
  q = fmaf(q, z, 6.66666687e-01f);   /* 2/3 */
  float lm = fmaf(s * z, q, 2.0f * s);
  float fe = (float)e;
  return fmaf(fe, LN2_HI, fmaf(fe, LN2_LO, lm));
}

/* exp of the deferred passes' weights, the same steps as the kernels' composite_expf:
 * k = the integer nearest the exact x log2(e) (an fma with 1.5 * 2^23, whose
 * rounding rounds to an integer), Cody-Waite reduction (ln2 in two parts),
 * degree-5 polynomial fitted for least maximum relative error on |r| <= ln2/2
 * (own Remez fit), scale 2^k from the sum's low bits (a normal float for
 * k >= -126: the weights call it for x > -86). */
float orc_composite_expf(float x) {
  const float t = fmaf(x, 1.44269502162933349609375f, 12582912.0f);
  const float k = t - 12582912.0f;
  float r = fmaf(k, -0.693145751953125f, x);
  r = fmaf(k, -1.428606765330187045e-06f, r);
  float p = 0x1.0fe5c6p-7f;
  p = fmaf(p, r, 0x1.575eeep-5f);
  p = fmaf(p, r, 0x1.555a18p-3f);
  p = fmaf(p, r, 0x1.fffd1ap-2f);
  p = fmaf(p, r, 0x1.fffff6p-1f);
  p = fmaf(p, r, 0x1.000002p+0f);
  return p * bitsf((fbits(t) << 23) + 0x3F800000u);
}

/* exp of a splat's power in the composites (the kernels' splat_expf): the
 * steps above with one reduction constant, ln 2 rounded to f32, which is
 * accurate for the powers whose exp is used (k in [-6, 0]). exp(x) = p * 2^k;
 * *kb = k << 23 (mod 2^32), the exponent-field bits of 2^k. */
float orc_splat_exp_parts(float x, uint32_t* kb) {
  const float t = fmaf(x, 1.44269502162933349609375f, 12582912.0f);
  const float k = t - 12582912.0f;
  const float r = fmaf(k, -0.693147182464599609375f, x);
  float p = 0x1.0fe5c6p-7f;
  p = fmaf(p, r, 0x1.575eeep-5f);
  p = fmaf(p, r, 0x1.555a18p-3f);
  p = fmaf(p, r, 0x1.fffd1ap-2f);
  p = fmaf(p, r, 0x1.fffff6p-1f);
  p = fmaf(p, r, 0x1.000002p+0f);
  *kb = fbits(t) << 23;
  return p;
}

float orc_splat_expf(float x) {
  uint32_t kb;
  const float p = orc_splat_exp_parts(x, &kb);
  return p * bitsf(kb + 0x3F800000u);
}

/* pack2x16float conversion: IEEE round-to-nearest-even, overflow -> inf,
 * NaN -> 0x7E00 (WGSL leaves NaN undefined; this fixes it). */
uint16_t orc_f32_to_f16_rne(float f) {
  uint32_t x = fbits(f);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ax = x & 0x7FFFFFFFu;
  if (ax > 0x7F800000u) return (uint16_t)0x7E00u;
  if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);
  if (ax < 0x38800000u) {
    float m = rintf(bitsf(ax) * 16777216.0f);
    return (uint16_t)(sign | (uint32_t)m);
  }
  uint32_t e = (ax >> 23) - 112u;
  uint32_t mant = ax & 0x7FFFFFu;
  uint32_t h = (e << 10) | (mant >> 13);
  uint32_t rem = mant & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1u;
  return (uint16_t)(sign | h);
}

float orc_f16_to_f32(uint16_t h) {
  uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
  uint32_t e = ((uint32_t)h >> 10) & 0x1Fu;
  uint32_t m = (uint32_t)h & 0x3FFu;
  if (e == 0) {
    float v = (float)m * 5.9604644775390625e-08f; /* m * 2^-24, exact */
    return sign ? -v : v;
  }
  if (e == 31) return bitsf(sign | 0x7F800000u | (m << 13));
  return bitsf(sign | ((e + 112u) << 23) | (m << 13));
}

/* IEEE binary16 round-to-nearest-even of a double (overflow -> inf, NaN ->
 * 0x7E00, subnormals kept). The f16 composite's arithmetic is exact in
 * double and then rounded here once, which is what a correctly rounded f16
 * multiply, subtract or fused multiply-add returns. */
uint16_t orc_f64_to_f16_rne(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  const uint16_t sign = (uint16_t)((b >> 48) & 0x8000u);
  const uint64_t ab = b & 0x7FFFFFFFFFFFFFFFull;
  if (ab > 0x7FF0000000000000ull) return (uint16_t)0x7E00u;
  if (ab >= 0x40EFFE0000000000ull) return (uint16_t)(sign | 0x7C00u); /* >= 65520 */
  if ((ab >> 52) == 0) return sign;                                    /* double subnormal: rounds to 0 */
  const int e = (int)(ab >> 52) - 1023;
  const uint64_t m = (ab & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int shift = e >= -14 ? 42 : 28 - e;  /* keep 11 bits (normal) or value / 2^-24 (subnormal) */
  if (shift > 63) return sign;
  uint64_t q = m >> shift;
  const uint64_t rem = m & ((1ull << shift) - 1ull), half = 1ull << (shift - 1);
  if (rem > half || (rem == half && (q & 1ull))) q += 1ull;
  if (e < -14) return (uint16_t)(sign | (uint16_t)q);  /* q == 0x400 is the smallest normal */
  return (uint16_t)(sign | (uint16_t)((((uint32_t)(e + 15)) << 10) + (uint32_t)(q - 0x400ull)));
}

/* splats.ts:431-442 — truncating f32ToF16 used by the host packers. */
uint16_t orc_f32_to_f16_trunc(float value) {
  uint32_t bits = fbits(value);
  uint32_t sign = (bits >> 16) & 0x8000u;
  int exp = (int)((bits >> 23) & 0xFFu) - 127 + 15;
  uint32_t frac = bits & 0x7FFFFFu;
  if (exp <= 0) return (uint16_t)sign;
  if (exp >= 31) return (uint16_t)(sign | 0x7C00u);
  return (uint16_t)(sign | ((uint32_t)exp << 10) | (frac >> 13));
}

static inline uint32_t pack2x16(float a, float b) {
  return (uint32_t)orc_f32_to_f16_rne(a) | ((uint32_t)orc_f32_to_f16_rne(b) << 16);
}
static inline float unpack_lo(uint32_t w) { return orc_f16_to_f32((uint16_t)(w & 0xFFFFu)); }
static inline float unpack_hi(uint32_t w) { return orc_f16_to_f32((uint16_t)(w >> 16)); }

/* gpu_tile_splat_composite.wgsl:33-47 */
uint32_t orc_morton(uint32_t x, uint32_t y) {
  uint32_t mx = x & 0xFFFFu;
  mx = (mx | (mx << 8)) & 0x00FF00FFu;
  mx = (mx | (mx << 4)) & 0x0F0F0F0Fu;
  mx = (mx | (mx << 2)) & 0x33333333u;
  mx = (mx | (mx << 1)) & 0x55555555u;
  uint32_t my = y & 0xFFFFu;
  my = (my | (my << 8)) & 0x00FF00FFu;
  my = (my | (my << 4)) & 0x0F0F0F0Fu;
  my = (my | (my << 2)) & 0x33333333u;
  my = (my | (my << 1)) & 0x55555555u;
  return mx | (my << 1);
}

/* gpuTileSplatCompositor.ts:109-139 */
void orc_plan(uint32_t W, uint32_t H, uint32_t tile, uint32_t N, double mult, uint32_t out[9]) {
  uint32_t cols = (W + tile - 1) / tile;
  uint32_t rows = (H + tile - 1) / tile;
  double want = ceil((double)N * mult);
  double cap = 65535.0 * 256.0;
  out[0] = W; out[1] = H; out[2] = tile; out[3] = cols; out[4] = rows;
  out[5] = cols * rows;
  out[6] = orc_morton(cols - 1, rows - 1) + 1;
  out[7] = N;
  out[8] = (uint32_t)(want < cap ? want : cap);
}

/* ---------------------------------------------------------------------------
 * small vector helpers (WGSL semantics, evaluation order left to right)
 * ------------------------------------------------------------------------- */
typedef struct { float x, y, z; } v3;
static inline v3 V3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 add3(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3s(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
/* Quotients that share a denominator take one correctly rounded reciprocal
 * and products (the kernels' canonical form of WGSL's '/' and normalize,
 * which allow 2.5 ulp), in the projection and the composites alike. */
static inline v3 div3s(v3 a, float s) { return mul3s(a, 1.0f / s); }
static inline float len3(v3 a) { return sqrtf(dot3(a, a)); }
static inline v3 norm3(v3 a) { return div3s(a, len3(a)); }

/* gpu_project_splats.wgsl:75-79 */
static inline v3 rotate_axis(const float q4[4], v3 axis) {
  float ql = sqrtf(q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
  float d = fmax_(ql, 0.000001f);
  float rd = 1.0f / d;
  float qx = q4[0] * rd, qy = q4[1] * rd, qz = q4[2] * rd, qw = q4[3] * rd;
  v3 u = V3(qy, qz, qw);
  v3 inner = add3(cross3(u, axis), mul3s(axis, qx));
  v3 c = cross3(u, inner);
  return add3(axis, mul3s(c, 2.0f));
}

/* gpu_project_splats.wgsl:82-89 */
static inline void oct_encode(v3 n, float* ox, float* oy) {
  float rs = 1.0f / (fabsf(n.x) + fabsf(n.y) + fabsf(n.z));
  float px = n.x * rs, py = n.y * rs;
  if (n.z < 0.0f) {
    float sx = px >= 0.0f ? 1.0f : -1.0f;
    float sy = py >= 0.0f ? 1.0f : -1.0f;
    float nx = (1.0f - fabsf(py)) * sx;
    float ny = (1.0f - fabsf(px)) * sy;
    px = nx; py = ny;
  }
  *ox = px; *oy = py;
}

/* gpu_tile_splat_composite.wgsl:143-149 */
static inline v3 oct_decode(float ex, float ey) {
  v3 n = V3(ex, ey, (1.0f - fabsf(ex)) - fabsf(ey));
  if (n.z < 0.0f) {
    float sx = n.x >= 0.0f ? 1.0f : -1.0f;
    float sy = n.y >= 0.0f ? 1.0f : -1.0f;
    float nx = (1.0f - fabsf(n.y)) * sx;
    float ny = (1.0f - fabsf(n.x)) * sy;
    n.x = nx; n.y = ny;
  }
  return norm3(n);
}

/* SH constants, gpu_project_splats.wgsl:59-71 (abstract floats -> f32) */
#define SH_C1 0.4886025119029199f
#define SH_C2_0 1.0925484305920792f
#define SH_C2_1 1.0925484305920792f
#define SH_C2_2 0.31539156525252005f
#define SH_C2_3 1.0925484305920792f
#define SH_C2_4 0.5462742152960396f
#define SH_C3_0 0.5900435899266435f
#define SH_C3_1 2.890611442640554f
#define SH_C3_2 0.4570457994644658f
#define SH_C3_3 0.3731763325901154f
#define SH_C3_4 0.4570457994644658f
#define SH_C3_5 1.445305721320277f
#define SH_C3_6 0.5900435899266435f

/* ---------------------------------------------------------------------------
 * project_splats — gpu_project_splats.wgsl:112-358, one sortRank.
 * ------------------------------------------------------------------------- */
static void project_one(const float* U, const orc_scene* s, uint32_t sortRank, uint32_t* pc,
                        uint32_t* depth) {
  const uint32_t N = Uu(U, 22);
  uint32_t* c = pc + (uint64_t)sortRank * PROJ_STRIDE;
  uint32_t splatId = s->sorted_indices[sortRank];
  if (splatId >= N) {
    /* The reference returns without writing (stale cache); canonical: invisible. */
    c[7] = SENTINEL;
    depth[sortRank] = SENTINEL;
    return;
  }
  const float* p = s->positions + (uint64_t)splatId * 3;
  v3 center = V3(p[0], p[1], p[2]);
  /* clip = viewProj * (center, 1): column-major, columns accumulated in order */
  float clip[4];
  for (int r = 0; r < 4; ++r)
    clip[r] = ((U[0 + r] * center.x + U[4 + r] * center.y) + U[8 + r] * center.z) + U[12 + r] * 1.0f;
  if (clip[3] <= 0.0f) {
    c[7] = SENTINEL;
    depth[sortRank] = SENTINEL;
    return;
  }
  float rW = 1.0f / fmax_(clip[3], 0.0001f);
  float ndcx = clip[0] * rW, ndcy = clip[1] * rW;
  float vpW = Uf(U, 16), vpH = Uf(U, 17);
  float cpx = (ndcx * 0.5f + 0.5f) * vpW;
  float cpy = (1.0f - (ndcy * 0.5f + 0.5f)) * vpH;
  float depthNdc = clip[2] * rW;

  const float* sl = s->scales + (uint64_t)splatId * 3;
  const float* q = s->rotations + (uint64_t)splatId * 4;
  float splatScale = Uf(U, 24);
  float scx = orc_expf(sl[0]) * splatScale;
  float scy = orc_expf(sl[1]) * splatScale;
  float scz = orc_expf(sl[2]) * splatScale;
  v3 axis0 = mul3s(rotate_axis(q, V3(1.0f, 0.0f, 0.0f)), scx);
  v3 axis1 = mul3s(rotate_axis(q, V3(0.0f, 1.0f, 0.0f)), scy);
  v3 axis2 = mul3s(rotate_axis(q, V3(0.0f, 0.0f, 1.0f)), scz);
  float len0 = dot3(axis0, axis0), len1 = dot3(axis1, axis1), len2 = dot3(axis2, axis2);
  float minLen = fmin_(len0, fmin_(len1, len2));
  v3 normalAxis = (len0 == minLen) ? axis0 : ((len1 == minLen) ? axis1 : axis2);
  v3 localNormal = norm3(normalAxis);

  v3 w0 = V3(U[32], U[36], U[40]);
  v3 w1 = V3(U[33], U[37], U[41]);
  v3 w2 = V3(U[34], U[38], U[42]);
  float vc[3];
  for (int r = 0; r < 3; ++r)
    vc[r] = ((U[32 + r] * center.x + U[36 + r] * center.y) + U[40 + r] * center.z) + U[44 + r] * 1.0f;
  float vz = fmin_(vc[2], -0.001f);
  float focx = U[48], focy = U[49];
  float rvz = 1.0f / vz;
  float J1x = focx * rvz, J1y = focy * rvz;
  float J2x = (-J1x * rvz) * vc[0];
  float J2y = (-J1y * rvz) * vc[1];
  v3 tt0 = V3(J1x * w0.x + J2x * w2.x, J1x * w0.y + J2x * w2.y, J1x * w0.z + J2x * w2.z);
  v3 tt1 = V3(J1y * w1.x + J2y * w2.x, J1y * w1.y + J2y * w2.y, J1y * w1.z + J2y * w2.z);
  v3 b0 = V3(dot3(axis0, tt0), dot3(axis1, tt0), dot3(axis2, tt0));
  v3 b1 = V3(dot3(axis0, tt1), dot3(axis1, tt1), dot3(axis2, tt1));
  float covXXraw = dot3(b0, b0), covXY = dot3(b0, b1), covYYraw = dot3(b1, b1);
  float detOrig = covXXraw * covYYraw - covXY * covXY;
  float covXX = covXXraw + 0.3f;
  float covYY = covYYraw + 0.3f;
  float detBlur = covXX * covYY - covXY * covXY;
  float detInv = 1.0f / fmax_(detBlur, 0.000001f);
  float aaFactor = sqrtf(fmax_(detOrig * detInv, 0.0f));
  float mid = 0.5f * (covXX + covYY);
  float det = fmax_(detBlur, 0.1f);
  float lambda = mid + sqrtf(fmax_(mid * mid - det, 0.1f));
  float radius = ceilf(3.0f * sqrtf(lambda));
  if (radius <= 0.0f) {
    c[7] = SENTINEL;
    depth[sortRank] = SENTINEL;
    return;
  }
  float icx = covYY * detInv, icy = -covXY * detInv, icz = covXX * detInv;
  float sourceOpacity = clampf_(s->opacities[splatId] * aaFactor, 0.0f, 0.99f);

  float tileSize = fmax_(Uf(U, 18), 1.0f);
  uint32_t gx = Uu(U, 20), gy = Uu(U, 21);
  uint32_t maxTx = (gx > 1u ? gx : 1u) - 1u, maxTy = (gy > 1u ? gy : 1u) - 1u;
  float clampedRadius = fmin_(radius, tileSize * 8.0f);
  float minPx = fmax_(cpx - clampedRadius, 0.0f), minPy = fmax_(cpy - clampedRadius, 0.0f);
  float maxPx = fmin_(cpx + clampedRadius, vpW), maxPy = fmin_(cpy + clampedRadius, vpH);
  float rTile = 1.0f / tileSize;
  uint32_t t0x = sat_u32(floorf(minPx * rTile)); if (t0x > maxTx) t0x = maxTx;
  uint32_t t0y = sat_u32(floorf(minPy * rTile)); if (t0y > maxTy) t0y = maxTy;
  uint32_t t1x = sat_u32(floorf(fmax_((maxPx - 0.000000001f) * rTile, 0.0f))); if (t1x > maxTx) t1x = maxTx;
  uint32_t t1y = sat_u32(floorf(fmax_((maxPy - 0.000000001f) * rTile, 0.0f))); if (t1y > maxTy) t1y = maxTy;

  c[0] = fbits(cpx); c[1] = fbits(cpy);
  c[2] = fbits(icx); c[3] = fbits(icy); c[4] = fbits(icz);
  c[5] = s->material[splatId];
  c[6] = pack2x16(radius, sourceOpacity);
  depth[sortRank] = fbits(depthNdc);
  c[7] = (t0x & 0xFFu) | ((t0y & 0xFFu) << 8) | ((t1x & 0xFFu) << 16) | ((t1y & 0xFFu) << 24);

  /* normals (gpu_project_splats.wgsl:234-291) */
  v3 splatNormal = localNormal;
  uint64_t nlen = s->normals ? s->normals_len : 0;
  uint64_t nb = (uint64_t)splatId * 3;
  if (nb + 2 < nlen) {
    v3 baked = V3(s->normals[nb], s->normals[nb + 1], s->normals[nb + 2]);
    float bl = len3(baked);
    if (bl > 0.001f) splatNormal = div3s(baked, bl);
  }
  uint64_t db = (uint64_t)N * 3 + (uint64_t)splatId * 3;
  if (db + 2 < nlen) {
    v3 detail = V3(s->normals[db], s->normals[db + 1], s->normals[db + 2]);
    float dl = len3(detail);
    if (dl > 0.001f) {
      v3 tc;
      if (len0 >= len1 && len0 >= len2) tc = axis0;
      else if (len1 >= len2) tc = axis1;
      else tc = axis2;
      v3 tp = sub3(tc, mul3s(splatNormal, dot3(tc, splatNormal)));
      float tl = len3(tp);
      if (tl > 0.001f) {
        v3 T = div3s(tp, tl);
        v3 B = cross3(splatNormal, T);
        v3 dn = div3s(detail, dl);
        v3 m = V3((T.x * dn.x + B.x * dn.y) + splatNormal.x * dn.z,
                  (T.y * dn.x + B.y * dn.y) + splatNormal.y * dn.z,
                  (T.z * dn.x + B.z * dn.y) + splatNormal.z * dn.z);
        splatNormal = norm3(m);
      }
    }
  }
  v3 cam = V3(U[28], U[29], U[30]);
  v3 nvd = norm3(sub3(cam, center));
  v3 fn = norm3(splatNormal);
  v3 fv = norm3(nvd);
  v3 faced = dot3(fn, fv) < 0.0f ? V3(-fn.x, -fn.y, -fn.z) : fn;
  float conf = clampf_(dot3(faced, nvd), 0.0f, 1.0f);
  v3 wn = V3((U[52] * faced.x + U[56] * faced.y) + U[60] * faced.z,
             (U[53] * faced.x + U[57] * faced.y) + U[61] * faced.z,
             (U[54] * faced.x + U[58] * faced.y) + U[62] * faced.z);
  wn = norm3(wn);
  float ox, oy;
  oct_encode(wn, &ox, &oy);
  c[8] = pack2x16(ox, oy);
  c[13] = pack2x16(conf, 0.0f);

  /* SH color (gpu_project_splats.wgsl:293-351), WGSL basis and signs */
  uint32_t deg = Uu(U, 25);
  uint32_t shCoeff = (deg + 1) * (deg + 1) - 1;
  uint32_t shStride = shCoeff * 3;
  const float* sh = s->sh_data + (uint64_t)splatId * (3 + shStride + 3);
  float cr = sh[0], cg = sh[1], cb = sh[2];
  if (deg >= 1) {
    v3 vd = norm3(sub3(cam, center));
    float vx = vd.x, vy = vd.y, vzz = vd.z;
    const float* b1 = sh + 3;
    cr = cr + SH_C1 * ((b1[0] * vy + b1[3] * vzz) + b1[6] * vx);
    cg = cg + SH_C1 * ((b1[1] * vy + b1[4] * vzz) + b1[7] * vx);
    cb = cb + SH_C1 * ((b1[2] * vy + b1[5] * vzz) + b1[8] * vx);
    if (deg >= 2) {
      float xx = vx * vx, yy = vy * vy, zz = vzz * vzz;
      float xy = vx * vy, yz = vy * vzz, xz = vx * vzz;
      float e0 = SH_C2_0 * xy, e1 = SH_C2_1 * yz, e2 = SH_C2_2 * ((2.0f * zz - xx) - yy);
      float e3 = SH_C2_3 * xz, e4 = SH_C2_4 * (xx - yy);
      const float* b2 = b1 + 9;
      cr = cr + ((((b2[0] * e0 + b2[3] * e1) + b2[6] * e2) + b2[9] * e3) + b2[12] * e4);
      cg = cg + ((((b2[1] * e0 + b2[4] * e1) + b2[7] * e2) + b2[10] * e3) + b2[13] * e4);
      cb = cb + ((((b2[2] * e0 + b2[5] * e1) + b2[8] * e2) + b2[11] * e3) + b2[14] * e4);
      if (deg >= 3) {
        float f0 = SH_C3_0 * vy * (3.0f * xx - yy);
        float f1 = SH_C3_1 * vx * vy * vzz;
        float f2 = SH_C3_2 * vy * ((4.0f * zz - xx) - yy);
        float f3 = SH_C3_3 * vzz * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
        float f4 = SH_C3_4 * vx * ((4.0f * zz - xx) - yy);
        float f5 = SH_C3_5 * vzz * (xx - yy);
        float f6 = SH_C3_6 * vx * (xx - 3.0f * yy);
        const float* b3 = b2 + 15;
        cr = cr + ((((((b3[0] * f0 + b3[3] * f1) + b3[6] * f2) + b3[9] * f3) + b3[12] * f4) + b3[15] * f5) + b3[18] * f6);
        cg = cg + ((((((b3[1] * f0 + b3[4] * f1) + b3[7] * f2) + b3[10] * f3) + b3[13] * f4) + b3[16] * f5) + b3[19] * f6);
        cb = cb + ((((((b3[2] * f0 + b3[5] * f1) + b3[8] * f2) + b3[11] * f3) + b3[14] * f4) + b3[17] * f5) + b3[20] * f6);
      }
    }
  }
  cr = clampf_(cr, 0.0f, 1.0f); cg = clampf_(cg, 0.0f, 1.0f); cb = clampf_(cb, 0.0f, 1.0f);
  c[9] = pack2x16(cr, cg);
  c[10] = pack2x16(cb, 0.0f);
  const float* em = sh + 3 + shStride;
  c[11] = pack2x16(em[0], em[1]);
  c[12] = pack2x16(em[2], 0.0f);
}

void orc_project(const float* U, const orc_scene* s, uint32_t* proj_cache, uint32_t* depth,
                 int threads) {
  const uint32_t N = Uu(U, 22);
  (void)threads;
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1)
  for (int64_t r = 0; r < (int64_t)N; ++r) project_one(U, s, (uint32_t)r, proj_cache, depth);
}

static inline void unpack_box(uint32_t packed, uint32_t* x0, uint32_t* y0, uint32_t* x1, uint32_t* y1) {
  *x0 = packed & 0xFFu; *y0 = (packed >> 8) & 0xFFu;
  *x1 = (packed >> 16) & 0xFFu; *y1 = (packed >> 24) & 0xFFu;
}

/* count_tile_refs, gpu_tile_splat_composite.wgsl:65-84 (M-bounds checked). */
void orc_count_tile_refs(const float* U, uint32_t N, const uint32_t* pc, uint32_t M,
                         uint32_t* counts) {
  (void)U;
  memset(counts, 0, sizeof(uint32_t) * M);
  for (uint32_t r = 0; r < N; ++r) {
    uint32_t packed = pc[(uint64_t)r * PROJ_STRIDE + 7];
    if (packed == SENTINEL) continue;
    uint32_t x0, y0, x1, y1;
    unpack_box(packed, &x0, &y0, &x1, &y1);
    for (uint32_t ty = y0; ty <= y1; ++ty)
      for (uint32_t tx = x0; tx <= x1; ++tx) {
        uint32_t t = orc_morton(tx, ty);
        if (t < M) counts[t] += 1u;
      }
  }
}

/* gpu_prefix_sum.wgsl: three-pass Hillis-Steele = exclusive scan (mod 2^32). */
void orc_exclusive_scan(const uint32_t* in, uint32_t n, uint32_t* out) {
  uint32_t acc = 0;
  for (uint32_t i = 0; i < n; ++i) { out[i] = acc; acc += in[i]; }
}

/* ---------------------------------------------------------------------------
 * sorting helpers
 * ------------------------------------------------------------------------- */
static int cmp_u64(const void* a, const void* b) {
  uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* Sort entries[0..n) by (depth bits, sortRank) — the canonical total order
 * that the reference's key-only bitonic network (gpu_tile_depth_sort.wgsl:
 * 141-157) produces up to ties. */
static void sort_depth_rank(uint32_t* entries, uint32_t n, const uint32_t* depth, uint64_t* tmp) {
  if (n <= 1) return;
  for (uint32_t i = 0; i < n; ++i) tmp[i] = ((uint64_t)depth[entries[i]] << 32) | entries[i];
  qsort(tmp, n, sizeof(uint64_t), cmp_u64);
  for (uint32_t i = 0; i < n; ++i) entries[i] = (uint32_t)tmp[i];
}

typedef struct { uint32_t bucket; uint64_t key; } bucket_entry;
static int cmp_bucket_entry(const void* a, const void* b) {
  const bucket_entry* x = (const bucket_entry*)a; const bucket_entry* y = (const bucket_entry*)b;
  if (x->bucket != y->bucket) return x->bucket < y->bucket ? -1 : 1;
  return x->key < y->key ? -1 : (x->key > y->key ? 1 : 0);
}

/* Per-tile log-depth mapping shared by the bucket cascade and the k20 keys
 * (gpu_tile_bucket_sort.wgsl:75-79, bucket :85). */
typedef struct { float logMin; float bucketScale; float keyScale; } tile_log;

static tile_log tile_log_params(uint32_t dminBits, uint32_t dmaxBits) {
  tile_log t;
  float depthMin = bitsf(dminBits), depthMax = bitsf(dmaxBits);
  t.logMin = orc_logf(fmax_(depthMin, 1e-6f));
  float logRange = orc_logf(fmax_(depthMax, 1e-6f)) - t.logMin;
  int degenerate = logRange < 1e-10f;
  t.bucketScale = degenerate ? 0.0f : 128.0f / logRange;
  t.keyScale = degenerate ? 0.0f : 1048576.0f / logRange;
  return t;
}

static inline uint32_t bucket_of(float logd, tile_log t) {
  uint32_t b = sat_u32((logd - t.logMin) * t.bucketScale);
  return b < NUM_BUCKETS - 1 ? b : NUM_BUCKETS - 1;
}
static inline uint32_t key20_of(float logd, tile_log t) {
  uint32_t k = sat_u32((logd - t.logMin) * t.keyScale);
  return k < KEY20_MAX ? k : KEY20_MAX;
}
static inline float log_depth(uint32_t dbits) { return orc_logf(fmax_(bitsf(dbits), 1e-6f)); }

/* ---------------------------------------------------------------------------
 * full canonical frame
 * ------------------------------------------------------------------------- */
static void composite_tile(const float* U, const uint32_t* pc, const uint32_t* depth,
                           const uint32_t* counts, const uint32_t* offsets,
                           const uint32_t* entries, uint32_t tileX, uint32_t tileY, orc_frame* f);

int orc_render_frame(const float* U, const orc_scene* s, orc_frame* f, int threads) {
  const uint32_t N = Uu(U, 22);
  const uint32_t cols = Uu(U, 20), rows = Uu(U, 21);
  const uint32_t budget = Uu(U, 23);
  const uint32_t M = orc_morton(cols - 1, rows - 1) + 1;
  int nt = threads > 0 ? threads : 1;
  f->flags = 0;

  orc_project(U, s, f->proj_cache, f->depth, nt);
  orc_count_tile_refs(U, N, f->proj_cache, M, f->tile_counts);
  orc_exclusive_scan(f->tile_counts, M, f->tile_offsets);
  uint64_t P = 0;
  for (uint32_t t = 0; t < M; ++t) P += f->tile_counts[t];
  f->total_pairs = P;
  /* chunk count (canonical) */
  uint32_t small = 0, hot = 0, chunks = 0;
  for (uint32_t t = 0; t < M; ++t) {
    uint32_t c = f->tile_counts[t];
    if (c == 0) continue;
    if (c <= MAX_TILE_ENTRIES) small++;
    else { hot++; chunks += (c + MAX_TILE_ENTRIES - 1) / MAX_TILE_ENTRIES; }
  }
  f->small_tiles = small; f->hot_tiles = hot; f->total_chunks = chunks;
  if (P > f->entries_cap || chunks > f->chunk_cap) return -2;
  if (P > budget) f->flags |= ORC_FLAG_REF_BUDGET_DROP;
  if (chunks > MAX_CHUNKS) f->flags |= ORC_FLAG_CHUNK_CAP;

  /* scatter: small splats first (scatter_tile_refs), then large splats
   * (large_splat_scatter), each in ascending sortRank — the canonical form
   * of the atomic slot order. */
  uint32_t* cursor = (uint32_t*)calloc(M, sizeof(uint32_t));
  if (!cursor) return -1;
  uint32_t large = 0;
  for (int pass = 0; pass < 2; ++pass) {
    for (uint32_t r = 0; r < N; ++r) {
      uint32_t packed = f->proj_cache[(uint64_t)r * PROJ_STRIDE + 7];
      if (packed == SENTINEL) continue;
      uint32_t x0, y0, x1, y1;
      unpack_box(packed, &x0, &y0, &x1, &y1);
      uint32_t spanX = x1 - x0 + 1, spanY = y1 - y0 + 1;
      int isLarge = spanX * spanY > LARGE_SPLAT_TILE_THRESHOLD;
      if (isLarge != pass) continue;
      if (pass == 1) large++;
      for (uint32_t ty = y0; ty <= y1; ++ty)
        for (uint32_t tx = x0; tx <= x1; ++tx) {
          uint32_t t = orc_morton(tx, ty);
          if (t >= M) continue;
          uint32_t slot = cursor[t]++;
          f->tile_entries[(uint64_t)f->tile_offsets[t] + slot] = r;
        }
    }
  }
  free(cursor);
  f->large_splats = large;
  if (large > MAX_LARGE_SPLATS) f->flags |= ORC_FLAG_LARGE_SPLAT_CAP;

  /* classify_tiles + tile_depth_sort + bucket_sort + chunk_sort */
  uint32_t* hotList = (uint32_t*)malloc(sizeof(uint32_t) * (hot + 1));
  uint32_t* hotBase = (uint32_t*)malloc(sizeof(uint32_t) * (hot + 1));
  uint32_t* smallList = (uint32_t*)malloc(sizeof(uint32_t) * (small + 1));
  if (!hotList || !hotBase || !smallList) return -1;
  uint32_t ns = 0, nh = 0;
  uint64_t overflow = 0;
  for (uint32_t t = 0; t < M; ++t) {
    uint32_t c = f->tile_counts[t];
    if (c == 0) continue;
    if (c <= MAX_TILE_ENTRIES) smallList[ns++] = t;
    else {
      hotBase[nh] = (uint32_t)((uint64_t)budget + overflow);
      if ((uint64_t)budget + overflow + c > (uint64_t)budget * 2u) f->flags |= ORC_FLAG_OVERFLOW_SKIP;
      overflow += c;
      hotList[nh++] = t;
    }
  }

#pragma omp parallel num_threads(nt)
  {
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * MAX_TILE_ENTRIES);
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < (int64_t)ns; ++i) {
      uint32_t t = smallList[i];
      sort_depth_rank(f->tile_entries + f->tile_offsets[t], f->tile_counts[t], f->depth, tmp);
    }
    free(tmp);
  }

  /* hot tiles, one at a time (chunk order is ascending Morton) */
  uint32_t chunkIdx = 0;
  uint32_t flags = 0;
  for (uint32_t h = 0; h < nh; ++h) {
    uint32_t t = hotList[h];
    uint32_t start = f->tile_offsets[t], count = f->tile_counts[t];
    uint32_t* e = f->tile_entries + start;
    /* phase 1: min/max of depth bits */
    uint32_t dmin = 0xFFFFFFFFu, dmax = 0u;
    for (uint32_t i = 0; i < count; ++i) {
      uint32_t d = f->depth[e[i]];
      if (d < dmin) dmin = d;
      if (d > dmax) dmax = d;
    }
    tile_log tl = tile_log_params(dmin, dmax);
    /* phases 2-4: bucket histogram, prefix, scatter in bucket order;
     * within a bucket ascending (depth bits, sortRank). */
    bucket_entry* tmp = (bucket_entry*)malloc(sizeof(bucket_entry) * count);
    uint32_t bucketCounts[NUM_BUCKETS];
    memset(bucketCounts, 0, sizeof(bucketCounts));
    for (uint32_t i = 0; i < count; ++i) {
      float ld = log_depth(f->depth[e[i]]);
      uint32_t b = bucket_of(ld, tl);
      uint32_t k = key20_of(ld, tl);
      if ((k >> 13) != b) flags |= ORC_FLAG_BUCKET_KEY_MISMATCH;
      bucketCounts[b]++;
      tmp[i].bucket = b;
      tmp[i].key = ((uint64_t)f->depth[e[i]] << 32) | e[i];
    }
    qsort(tmp, count, sizeof(bucket_entry), cmp_bucket_entry);
    uint32_t bucketOffsets[NUM_BUCKETS + 1];
    bucketOffsets[0] = 0;
    for (uint32_t b = 0; b < NUM_BUCKETS; ++b) bucketOffsets[b + 1] = bucketOffsets[b] + bucketCounts[b];
    for (uint32_t i = 0; i < count; ++i) e[i] = (uint32_t)tmp[i].key;
    free(tmp);
    /* phase 5: greedy chunk pack (gpu_tile_bucket_sort.wgsl:110-143) */
    uint32_t chunkStart = 0, cur = 0;
    for (uint32_t b = 0; b < NUM_BUCKETS; ++b) {
      uint32_t rem = bucketOffsets[b + 1] - bucketOffsets[b];
      while (rem > 0) {
        uint32_t space = MAX_TILE_ENTRIES - cur;
        uint32_t take = rem < space ? rem : space;
        cur += take; rem -= take;
        if (cur == MAX_TILE_ENTRIES) {
          f->chunk_ranges[2 * chunkIdx] = start + chunkStart;
          f->chunk_ranges[2 * chunkIdx + 1] = cur;
          chunkIdx++;
          chunkStart += cur;
          cur = 0;
        }
      }
    }
    if (cur > 0) {
      f->chunk_ranges[2 * chunkIdx] = start + chunkStart;
      f->chunk_ranges[2 * chunkIdx + 1] = cur;
      chunkIdx++;
    }
  }
  f->flags |= flags;
  f->total_chunks = chunkIdx;
  free(hotList); free(hotBase); free(smallList);

#pragma omp parallel num_threads(nt)
  {
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * MAX_TILE_ENTRIES);
#pragma omp for schedule(dynamic, 4)
    for (int64_t c = 0; c < (int64_t)chunkIdx; ++c) {
      uint32_t st = f->chunk_ranges[2 * c], n = f->chunk_ranges[2 * c + 1];
      sort_depth_rank(f->tile_entries + st, n, f->depth, tmp);
    }
    free(tmp);
  }

  if (f->out_color) orc_composite(U, f->proj_cache, f->depth, f->tile_counts, f->tile_offsets,
                                  f->tile_entries, f, nt);
  return 0;
}

int orc_sorted_keys20(const float* U, uint32_t N, const uint32_t* pc, const uint32_t* depth,
                      uint64_t* keys, uint32_t* values, uint64_t cap, uint64_t* total) {
  const uint32_t cols = Uu(U, 20), rows = Uu(U, 21);
  const uint32_t M = orc_morton(cols - 1, rows - 1) + 1;
  uint32_t* counts = (uint32_t*)calloc(M, sizeof(uint32_t));
  uint32_t* offs = (uint32_t*)calloc(M + 1, sizeof(uint32_t));
  uint32_t* dmin = (uint32_t*)malloc(sizeof(uint32_t) * M);
  uint32_t* dmax = (uint32_t*)calloc(M, sizeof(uint32_t));
  if (!counts || !offs || !dmin || !dmax) return -1;
  for (uint32_t t = 0; t < M; ++t) dmin[t] = 0xFFFFFFFFu;
  orc_count_tile_refs(U, N, pc, M, counts);
  uint64_t P = 0;
  for (uint32_t t = 0; t < M; ++t) { offs[t] = (uint32_t)P; P += counts[t]; }
  *total = P;
  if (P > cap) { free(counts); free(offs); free(dmin); free(dmax); return -2; }
  for (uint32_t r = 0; r < N; ++r) {
    uint32_t packed = pc[(uint64_t)r * PROJ_STRIDE + 7];
    if (packed == SENTINEL) continue;
    uint32_t x0, y0, x1, y1;
    unpack_box(packed, &x0, &y0, &x1, &y1);
    for (uint32_t ty = y0; ty <= y1; ++ty)
      for (uint32_t tx = x0; tx <= x1; ++tx) {
        uint32_t t = orc_morton(tx, ty);
        if (t >= M) continue;
        if (depth[r] < dmin[t]) dmin[t] = depth[r];
        if (depth[r] > dmax[t]) dmax[t] = depth[r];
      }
  }
  memset(counts, 0, sizeof(uint32_t) * M);
  for (uint32_t r = 0; r < N; ++r) {
    uint32_t packed = pc[(uint64_t)r * PROJ_STRIDE + 7];
    if (packed == SENTINEL) continue;
    uint32_t x0, y0, x1, y1;
    unpack_box(packed, &x0, &y0, &x1, &y1);
    float ld = log_depth(depth[r]);
    for (uint32_t ty = y0; ty <= y1; ++ty)
      for (uint32_t tx = x0; tx <= x1; ++tx) {
        uint32_t t = orc_morton(tx, ty);
        if (t >= M) continue;
        tile_log tl = tile_log_params(dmin[t], dmax[t]);
        uint64_t pos = (uint64_t)offs[t] + counts[t]++;
        keys[pos] = ((uint64_t)t << 20) | key20_of(ld, tl);
        values[pos] = r;
      }
  }
  /* within each tile ascending (k20, sortRank) */
  for (uint32_t t = 0; t < M; ++t) {
    uint32_t n = counts[t];
    if (n <= 1) continue;
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * n);
    for (uint32_t i = 0; i < n; ++i)
      tmp[i] = ((keys[offs[t] + i] & KEY20_MAX) << 32) | values[offs[t] + i];
    qsort(tmp, n, sizeof(uint64_t), cmp_u64);
    for (uint32_t i = 0; i < n; ++i) {
      keys[offs[t] + i] = ((uint64_t)t << 20) | (tmp[i] >> 32);
      values[offs[t] + i] = (uint32_t)tmp[i];
    }
    free(tmp);
  }
  free(counts); free(offs); free(dmin); free(dmax);
  return 0;
}

/* ---------------------------------------------------------------------------
 * composite — gpu_tile_splat_composite.wgsl:162-370.
 * The per-pixel arithmetic below is the canonical form shared with the CUDA
 * rasteriser: power = fma(cy*dy, dy, fma(cz*dx, dy, (cx*dx)*dx)) and every
 * accumulation "acc += v * w" is fma(v, w, acc).
 * ------------------------------------------------------------------------- */
static void composite_tile(const float* U, const uint32_t* pc, const uint32_t* depth,
                           const uint32_t* counts, const uint32_t* offsets,
                           const uint32_t* entries, uint32_t tileX, uint32_t tileY, orc_frame* f) {
  const uint32_t W = (uint32_t)Uf(U, 16), H = (uint32_t)Uf(U, 17);
  const uint32_t tileId = orc_morton(tileX, tileY);
  const uint32_t refStart = offsets[tileId], refCount = counts[tileId];
  const float bg[3] = {0.02f, 0.02f, 0.04f};
  for (uint32_t ly = 0; ly < 8; ++ly)
    for (uint32_t lx = 0; lx < 8; ++lx) {
      uint32_t bx = tileX * 16 + lx * 2, by = tileY * 16 + ly * 2;
      float p00x = (float)bx + 0.5f, p00y = (float)by + 0.5f;
      float T[4] = {1.0f, 1.0f, 1.0f, 1.0f};
      float col[4][3] = {{0}}, em[4][3] = {{0}}, nrm[4][3] = {{0}}, mat[4][2] = {{0}};
      float gbD[4] = {0}, gbW[4] = {0}, gbC[4] = {0};
      for (uint32_t k = 0; k < refCount; ++k) {
        uint32_t r = entries[(uint64_t)refStart + k];
        const uint32_t* c = pc + (uint64_t)r * PROJ_STRIDE;
        float cx = bitsf(c[0]), cy = bitsf(c[1]);
        float ka = bitsf(c[2]) * -0.5f, kc = bitsf(c[4]) * -0.5f, kb = -bitsf(c[3]);
        float op = unpack_hi(c[6]);
        float sr = unpack_lo(c[9]), sg = unpack_hi(c[9]), sb = unpack_lo(c[10]);
        float dx0 = p00x - cx, dy0 = p00y - cy;
        float dxv[4] = {dx0, dx0 + 1.0f, dx0, dx0 + 1.0f};
        float dyv[4] = {dy0, dy0, dy0 + 1.0f, dy0 + 1.0f};
        float pw[4];
        for (int i = 0; i < 4; ++i)
          pw[i] = fmaf(kc * dyv[i], dyv[i], fmaf(kb * dxv[i], dyv[i], (ka * dxv[i]) * dxv[i]));
        if (pw[0] <= -4.0f && pw[1] <= -4.0f && pw[2] <= -4.0f && pw[3] <= -4.0f) continue;
        float sd = bitsf(depth[r]);
        float mr = unpack_lo(c[5]), mm = unpack_hi(c[5]);
        v3 sn = oct_decode(unpack_lo(c[8]), unpack_hi(c[8]));
        float sc = unpack_lo(c[13]);
        float er = unpack_lo(c[11]), eg = unpack_hi(c[11]), eb = unpack_lo(c[12]);
        for (int i = 0; i < 4; ++i) {
          float g = orc_splat_expf(pw[i]);
          float a = fmin_(0.99f, op * g);
          float nT = T[i] * (1.0f - a);
          int valid = (pw[i] > -4.0f) && (a > (1.0f / 255.0f)) && (T[i] >= 0.001f);
          float w = valid ? a * T[i] : 0.0f;
          col[i][0] = fmaf(sr, w, col[i][0]);
          col[i][1] = fmaf(sg, w, col[i][1]);
          col[i][2] = fmaf(sb, w, col[i][2]);
          if (valid) T[i] = nT;
          float gw = w > 0.01f ? w : 0.0f;
          gbD[i] = fmaf(gw, sd, gbD[i]);
          gbW[i] = gbW[i] + gw;
          mat[i][0] = fmaf(mr, gw, mat[i][0]);
          mat[i][1] = fmaf(mm, gw, mat[i][1]);
          nrm[i][0] = fmaf(sn.x, gw, nrm[i][0]);
          nrm[i][1] = fmaf(sn.y, gw, nrm[i][1]);
          nrm[i][2] = fmaf(sn.z, gw, nrm[i][2]);
          gbC[i] = fmaf(sc, gw, gbC[i]);
          em[i][0] = fmaf(er, w, em[i][0]);
          em[i][1] = fmaf(eg, w, em[i][1]);
          em[i][2] = fmaf(eb, w, em[i][2]);
        }
        if (T[0] < 0.001f && T[1] < 0.001f && T[2] < 0.001f && T[3] < 0.001f) break;
      }
      for (int i = 0; i < 4; ++i) {
        uint32_t px = bx + (uint32_t)(i & 1), py = by + (uint32_t)(i >> 1);
        if (px >= W || py >= H) continue;
        uint64_t o = (uint64_t)py * W + px;
        float rsw = 1.0f / fmax_(gbW[i], 0.0001f);
        float ox, oy;
        oct_encode(norm3(V3(nrm[i][0], nrm[i][1] + 0.0001f, nrm[i][2])), &ox, &oy);
        f->out_color[o * 4 + 0] = orc_f32_to_f16_rne(fmaf(T[i], bg[0], col[i][0]));
        f->out_color[o * 4 + 1] = orc_f32_to_f16_rne(fmaf(T[i], bg[1], col[i][1]));
        f->out_color[o * 4 + 2] = orc_f32_to_f16_rne(fmaf(T[i], bg[2], col[i][2]));
        f->out_color[o * 4 + 3] = orc_f32_to_f16_rne(1.0f - T[i]);
        f->out_depth[o] = gbD[i] * rsw;
        f->out_normal[o] = pack2x16(ox, oy);
        f->out_material[o * 4 + 0] = pack2x16(mat[i][0] * rsw, mat[i][1] * rsw);
        f->out_material[o * 4 + 1] = pack2x16(em[i][0], em[i][1]);
        f->out_material[o * 4 + 2] = pack2x16(em[i][2], 0.0f);
        f->out_material[o * 4 + 3] = pack2x16(gbC[i] * rsw, 0.0f);
      }
    }
}

/* ---------------------------------------------------------------------------
 * composite, f16 variant — gpu_tile_splat_composite_f16.wgsl:86-285 (the
 * reference selects it when the adapter has shader-f16, splatRenderer.ts:907).
 * The Gaussian, alpha and the G-buffer votes stay f32 as in composite_tile;
 * transmittance and colour are f16: alpha is rounded to f16 (:193),
 * T' = T * (1 - alpha) rounds twice (:194), the weight is f16(alpha * T)
 * (:197), colour accumulates with one f16 fused multiply-add per channel
 * (:199, the canonical form, like the f32 path's fmaf), the thresholds are
 * the f16 constants 1/255 and 0.001 (:53-54), and the output colour is
 * fma16(T, bg16, c) (:254-259). Every f16 operation here is computed exactly
 * in double (the operands are multiples of 2^-48 below 2^5) and rounded once.
 * ------------------------------------------------------------------------- */
static inline float h16(double x) { return orc_f16_to_f32(orc_f64_to_f16_rne(x)); }

static void composite_tile_f16(const float* U, const uint32_t* pc, const uint32_t* depth,
                               const uint32_t* counts, const uint32_t* offsets,
                               const uint32_t* entries, uint32_t tileX, uint32_t tileY, orc_frame* f) {
  const uint32_t W = (uint32_t)Uf(U, 16), H = (uint32_t)Uf(U, 17);
  const uint32_t tileId = orc_morton(tileX, tileY);
  const uint32_t refStart = offsets[tileId], refCount = counts[tileId];
  const float bg[3] = {h16(0.02), h16(0.02), h16(0.04)};
  const float alphaTh = h16(1.0 / 255.0), cutoff = h16(0.001);
  for (uint32_t ly = 0; ly < 8; ++ly)
    for (uint32_t lx = 0; lx < 8; ++lx) {
      uint32_t bx = tileX * 16 + lx * 2, by = tileY * 16 + ly * 2;
      float p00x = (float)bx + 0.5f, p00y = (float)by + 0.5f;
      float T[4] = {1.0f, 1.0f, 1.0f, 1.0f};
      float col[4][3] = {{0}}, em[4][3] = {{0}}, nrm[4][3] = {{0}}, mat[4][2] = {{0}};
      float gbD[4] = {0}, gbW[4] = {0}, gbC[4] = {0};
      for (uint32_t k = 0; k < refCount; ++k) {
        uint32_t r = entries[(uint64_t)refStart + k];
        const uint32_t* c = pc + (uint64_t)r * PROJ_STRIDE;
        float cx = bitsf(c[0]), cy = bitsf(c[1]);
        float ka = bitsf(c[2]) * -0.5f, kc = bitsf(c[4]) * -0.5f, kb = -bitsf(c[3]);
        float op = unpack_hi(c[6]);
        float sr = unpack_lo(c[9]), sg = unpack_hi(c[9]), sb = unpack_lo(c[10]);
        float dx0 = p00x - cx, dy0 = p00y - cy;
        float dxv[4] = {dx0, dx0 + 1.0f, dx0, dx0 + 1.0f};
        float dyv[4] = {dy0, dy0, dy0 + 1.0f, dy0 + 1.0f};
        float pw[4];
        for (int i = 0; i < 4; ++i)
          pw[i] = fmaf(kc * dyv[i], dyv[i], fmaf(kb * dxv[i], dyv[i], (ka * dxv[i]) * dxv[i]));
        if (pw[0] <= -4.0f && pw[1] <= -4.0f && pw[2] <= -4.0f && pw[3] <= -4.0f) continue;
        float sd = bitsf(depth[r]);
        float mr = unpack_lo(c[5]), mm = unpack_hi(c[5]);
        v3 sn = oct_decode(unpack_lo(c[8]), unpack_hi(c[8]));
        float sc = unpack_lo(c[13]);
        float er = unpack_lo(c[11]), eg = unpack_hi(c[11]), eb = unpack_lo(c[12]);
        for (int i = 0; i < 4; ++i) {
          float g = orc_splat_expf(pw[i]);
          float a32 = fmin_(0.99f, op * g);
          float a16 = orc_f16_to_f32(orc_f32_to_f16_rne(a32));
          float nT = h16((double)T[i] * (double)h16(1.0 - (double)a16));
          int valid = (pw[i] > -4.0f) && (a32 > alphaTh) && (T[i] >= cutoff);
          float w = valid ? h16((double)a16 * (double)T[i]) : 0.0f;
          col[i][0] = h16((double)sr * w + col[i][0]);
          col[i][1] = h16((double)sg * w + col[i][1]);
          col[i][2] = h16((double)sb * w + col[i][2]);
          if (valid) T[i] = nT;
          float gw = w > 0.01f ? w : 0.0f;
          gbD[i] = fmaf(gw, sd, gbD[i]);
          gbW[i] = gbW[i] + gw;
          mat[i][0] = fmaf(mr, gw, mat[i][0]);
          mat[i][1] = fmaf(mm, gw, mat[i][1]);
          nrm[i][0] = fmaf(sn.x, gw, nrm[i][0]);
          nrm[i][1] = fmaf(sn.y, gw, nrm[i][1]);
          nrm[i][2] = fmaf(sn.z, gw, nrm[i][2]);
          gbC[i] = fmaf(sc, gw, gbC[i]);
          em[i][0] = fmaf(er, w, em[i][0]);
          em[i][1] = fmaf(eg, w, em[i][1]);
          em[i][2] = fmaf(eb, w, em[i][2]);
        }
        if (T[0] < cutoff && T[1] < cutoff && T[2] < cutoff && T[3] < cutoff) break;
      }
      for (int i = 0; i < 4; ++i) {
        uint32_t px = bx + (uint32_t)(i & 1), py = by + (uint32_t)(i >> 1);
        if (px >= W || py >= H) continue;
        uint64_t o = (uint64_t)py * W + px;
        float rsw = 1.0f / fmax_(gbW[i], 0.0001f);
        float ox, oy;
        oct_encode(norm3(V3(nrm[i][0], nrm[i][1] + 0.0001f, nrm[i][2])), &ox, &oy);
        for (int ch = 0; ch < 3; ++ch)
          f->out_color[o * 4 + ch] = orc_f64_to_f16_rne((double)T[i] * bg[ch] + col[i][ch]);
        f->out_color[o * 4 + 3] = orc_f32_to_f16_rne(1.0f - T[i]);
        f->out_depth[o] = gbD[i] * rsw;
        f->out_normal[o] = pack2x16(ox, oy);
        f->out_material[o * 4 + 0] = pack2x16(mat[i][0] * rsw, mat[i][1] * rsw);
        f->out_material[o * 4 + 1] = pack2x16(em[i][0], em[i][1]);
        f->out_material[o * 4 + 2] = pack2x16(em[i][2], 0.0f);
        f->out_material[o * 4 + 3] = pack2x16(gbC[i] * rsw, 0.0f);
      }
    }
}

void orc_composite(const float* U, const uint32_t* pc, const uint32_t* depth,
                   const uint32_t* counts, const uint32_t* offsets, const uint32_t* entries,
                   orc_frame* f, int threads) {
  const uint32_t cols = Uu(U, 20), rows = Uu(U, 21);
  int nt = threads > 0 ? threads : 1;
  (void)nt;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
  for (int64_t i = 0; i < (int64_t)cols * rows; ++i)
    (f->composite_f16 ? composite_tile_f16 : composite_tile)(U, pc, depth, counts, offsets, entries,
                                                            (uint32_t)(i % cols), (uint32_t)(i / cols), f);
}

/* ---------------------------------------------------------------------------
 * FP64 twin: projection + composite in double without f16 quantisation, over
 * the canonical entry order of the f32 frame. Used only as an accuracy judge.
 * ------------------------------------------------------------------------- */
typedef struct { double x, y, z; } d3;
static inline d3 D3(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 dcross(d3 a, d3 b) { return D3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline d3 dnorm(d3 a) { double l = sqrt(ddot(a, a)); return D3(a.x / l, a.y / l, a.z / l); }

typedef struct { double cx, cy, ia, ib, ic, op, r, g, b; int visible; } proj64;

static proj64 project_one_f64(const float* U, const orc_scene* s, uint32_t sortRank) {
  proj64 o; memset(&o, 0, sizeof(o));
  const uint32_t N = Uu(U, 22);
  uint32_t id = s->sorted_indices[sortRank];
  if (id >= N) return o;
  const float* p = s->positions + (uint64_t)id * 3;
  double cx = p[0], cy = p[1], cz = p[2];
  double clip[4];
  for (int r = 0; r < 4; ++r) clip[r] = U[r] * cx + U[4 + r] * cy + U[8 + r] * cz + U[12 + r];
  if (clip[3] <= 0.0) return o;
  double sw = clip[3] > 1e-4 ? clip[3] : 1e-4;
  o.cx = (clip[0] / sw * 0.5 + 0.5) * U[16];
  o.cy = (1.0 - (clip[1] / sw * 0.5 + 0.5)) * U[17];
  const float* sl = s->scales + (uint64_t)id * 3;
  const float* q = s->rotations + (uint64_t)id * 4;
  double ql = sqrt((double)q[0] * q[0] + (double)q[1] * q[1] + (double)q[2] * q[2] + (double)q[3] * q[3]);
  if (ql < 1e-6) ql = 1e-6;
  double qx = q[0] / ql;
  d3 u = D3(q[1] / ql, q[2] / ql, q[3] / ql);
  d3 ax[3];
  for (int i = 0; i < 3; ++i) {
    d3 e = D3(i == 0, i == 1, i == 2);
    d3 in = dcross(u, e); in.x += qx * e.x; in.y += qx * e.y; in.z += qx * e.z;
    d3 c = dcross(u, in);
    double sc = exp((double)sl[i]) * U[24];
    ax[i] = D3((e.x + 2 * c.x) * sc, (e.y + 2 * c.y) * sc, (e.z + 2 * c.z) * sc);
  }
  d3 w0 = D3(U[32], U[36], U[40]), w1 = D3(U[33], U[37], U[41]), w2 = D3(U[34], U[38], U[42]);
  double vc[3];
  for (int r = 0; r < 3; ++r) vc[r] = U[32 + r] * cx + U[36 + r] * cy + U[40 + r] * cz + U[44 + r];
  double vz = vc[2] < -0.001 ? vc[2] : -0.001;
  double J1x = U[48] / vz, J1y = U[49] / vz;
  double J2x = -J1x / vz * vc[0], J2y = -J1y / vz * vc[1];
  d3 t0 = D3(J1x * w0.x + J2x * w2.x, J1x * w0.y + J2x * w2.y, J1x * w0.z + J2x * w2.z);
  d3 t1 = D3(J1y * w1.x + J2y * w2.x, J1y * w1.y + J2y * w2.y, J1y * w1.z + J2y * w2.z);
  d3 b0 = D3(ddot(ax[0], t0), ddot(ax[1], t0), ddot(ax[2], t0));
  d3 b1 = D3(ddot(ax[0], t1), ddot(ax[1], t1), ddot(ax[2], t1));
  double xx = ddot(b0, b0), xy = ddot(b0, b1), yy = ddot(b1, b1);
  double detO = xx * yy - xy * xy;
  double XX = xx + 0.3, YY = yy + 0.3;
  double detB = XX * YY - xy * xy;
  double dbm = detB > 1e-6 ? detB : 1e-6;
  double aa = detO / dbm; aa = sqrt(aa > 0 ? aa : 0);
  o.ia = YY / dbm; o.ib = -xy / dbm; o.ic = XX / dbm;
  double op = s->opacities[id] * aa;
  o.op = op < 0 ? 0 : (op > 0.99 ? 0.99 : op);
  uint32_t deg = Uu(U, 25);
  uint32_t stride = ((deg + 1) * (deg + 1) - 1) * 3;
  const float* sh = s->sh_data + (uint64_t)id * (3 + stride + 3);
  double col[3] = {sh[0], sh[1], sh[2]};
  if (deg >= 1) {
    d3 vd = dnorm(D3(U[28] - cx, U[29] - cy, U[30] - cz));
    double vx = vd.x, vy = vd.y, vw = vd.z;
    const float* b1c = sh + 3;
    double xx2 = vx * vx, yy2 = vy * vy, zz2 = vw * vw;
    double e2[5] = {1.0925484305920792 * vx * vy, 1.0925484305920792 * vy * vw,
                    0.31539156525252005 * (2 * zz2 - xx2 - yy2), 1.0925484305920792 * vx * vw,
                    0.5462742152960396 * (xx2 - yy2)};
    double e3[7] = {0.5900435899266435 * vy * (3 * xx2 - yy2), 2.890611442640554 * vx * vy * vw,
                    0.4570457994644658 * vy * (4 * zz2 - xx2 - yy2),
                    0.3731763325901154 * vw * (2 * zz2 - 3 * xx2 - 3 * yy2),
                    0.4570457994644658 * vx * (4 * zz2 - xx2 - yy2), 1.445305721320277 * vw * (xx2 - yy2),
                    0.5900435899266435 * vx * (xx2 - 3 * yy2)};
    for (int ch = 0; ch < 3; ++ch) {
      col[ch] += 0.4886025119029199 * (b1c[ch] * vy + b1c[3 + ch] * vw + b1c[6 + ch] * vx);
      if (deg >= 2) for (int k = 0; k < 5; ++k) col[ch] += b1c[9 + 3 * k + ch] * e2[k];
      if (deg >= 3) for (int k = 0; k < 7; ++k) col[ch] += b1c[24 + 3 * k + ch] * e3[k];
    }
  }
  o.r = col[0] < 0 ? 0 : (col[0] > 1 ? 1 : col[0]);
  o.g = col[1] < 0 ? 0 : (col[1] > 1 ? 1 : col[1]);
  o.b = col[2] < 0 ? 0 : (col[2] > 1 ? 1 : col[2]);
  o.visible = 1;
  return o;
}

void orc_project_f64(const float* U, const orc_scene* s, double* out, int threads) {
  const uint32_t N = Uu(U, 22);
  int nt = threads > 0 ? threads : 1;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t r = 0; r < (int64_t)N; ++r) {
    proj64 p = project_one_f64(U, s, (uint32_t)r);
    double* o = out + r * 10;
    o[0] = p.cx; o[1] = p.cy; o[2] = p.ia; o[3] = p.ib; o[4] = p.ic;
    o[5] = p.op; o[6] = p.r; o[7] = p.g; o[8] = p.b; o[9] = p.visible;
  }
}

int orc_render_frame_f64(const float* U, const orc_scene* s, const uint32_t* counts,
                         const uint32_t* offsets, const uint32_t* entries, double* out,
                         int threads) {
  const uint32_t N = Uu(U, 22);
  const uint32_t cols = Uu(U, 20), rows = Uu(U, 21);
  const uint32_t W = (uint32_t)U[16], H = (uint32_t)U[17];
  int nt = threads > 0 ? threads : 1;
  proj64* pj = (proj64*)malloc(sizeof(proj64) * (N ? N : 1));
  if (!pj) return -1;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t r = 0; r < (int64_t)N; ++r) pj[r] = project_one_f64(U, s, (uint32_t)r);
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
  for (int64_t ti = 0; ti < (int64_t)cols * rows; ++ti) {
    uint32_t tx = (uint32_t)(ti % cols), ty = (uint32_t)(ti / cols);
    uint32_t t = orc_morton(tx, ty);
    for (uint32_t py = ty * 16; py < ty * 16 + 16 && py < H; ++py)
      for (uint32_t px = tx * 16; px < tx * 16 + 16 && px < W; ++px) {
        double T = 1.0, c[3] = {0, 0, 0};
        for (uint32_t k = 0; k < counts[t]; ++k) {
          /* T never grows, so once below the cutoff no later entry is valid:
           * stopping here changes nothing */
          if (!(T >= 0.001)) break;
          const proj64* g = &pj[entries[(uint64_t)offsets[t] + k]];
          double dx = px + 0.5 - g->cx, dy = py + 0.5 - g->cy;
          double pw = -0.5 * g->ia * dx * dx - 0.5 * g->ic * dy * dy - g->ib * dx * dy;
          if (!(pw > -4.0)) continue;
          double a = g->op * exp(pw);
          if (a > 0.99) a = 0.99;
          if (!(a > 1.0 / 255.0) || !(T >= 0.001)) continue;
          c[0] += g->r * a * T; c[1] += g->g * a * T; c[2] += g->b * a * T;
          T *= 1.0 - a;
        }
        uint64_t o = (uint64_t)py * W + px;
        out[o * 4 + 0] = c[0] + T * 0.02;
        out[o * 4 + 1] = c[1] + T * 0.02;
        out[o * 4 + 2] = c[2] + T * 0.04;
        out[o * 4 + 3] = 1.0 - T;
      }
  }
  free(pj);
  return 0;
}

/* ---------------------------------------------------------------------------
 * CPU depth-sort baseline — splatSort.ts:32-55 (keys.sort by depth asc, id
 * asc; depth = view[2]x + view[6]y + view[10]z + view[14] in double).
 * ------------------------------------------------------------------------- */
typedef struct { double depth; uint32_t id; } dkey;
static int cmp_dkey(const void* a, const void* b) {
  const dkey* x = (const dkey*)a; const dkey* y = (const dkey*)b;
  if (x->depth < y->depth) return -1;
  if (x->depth > y->depth) return 1;
  return x->id < y->id ? -1 : (x->id > y->id ? 1 : 0);
}

static void merge_dkeys(dkey* a, uint32_t n1, uint32_t n2, dkey* tmp) {
  uint32_t i = 0, j = n1, k = 0;
  while (i < n1 && j < n1 + n2) tmp[k++] = cmp_dkey(&a[i], &a[j]) <= 0 ? a[i++] : a[j++];
  while (i < n1) tmp[k++] = a[i++];
  while (j < n1 + n2) tmp[k++] = a[j++];
  memcpy(a, tmp, sizeof(dkey) * (n1 + n2));
}

int orc_sort_back_to_front(const float* positions, uint32_t n, const float* view,
                           uint32_t* order_out, int threads) {
  dkey* keys = (dkey*)malloc(sizeof(dkey) * (n ? n : 1));
  if (!keys) return -2;
  int bad = 0;
  for (uint32_t id = 0; id < n; ++id) {
    double x = positions[(uint64_t)id * 3], y = positions[(uint64_t)id * 3 + 1], z = positions[(uint64_t)id * 3 + 2];
    double d = (double)view[2] * x + (double)view[6] * y + (double)view[10] * z + (double)view[14];
    if (!isfinite(d)) bad = 1;
    keys[id].depth = d; keys[id].id = id;
  }
  if (bad) { free(keys); return -1; }
  int nt = threads > 0 ? threads : 1;
  if (nt <= 1 || n < 4096) {
    qsort(keys, n, sizeof(dkey), cmp_dkey);
  } else {
    /* parallel: sort nt slices, then merge pairwise (same total order) */
    uint32_t slice = (n + (uint32_t)nt - 1) / (uint32_t)nt;
#pragma omp parallel for num_threads(nt)
    for (int t = 0; t < nt; ++t) {
      uint32_t lo = (uint32_t)t * slice;
      if (lo >= n) continue;
      uint32_t hi = lo + slice < n ? lo + slice : n;
      qsort(keys + lo, hi - lo, sizeof(dkey), cmp_dkey);
    }
    dkey* tmp = (dkey*)malloc(sizeof(dkey) * n);
    for (uint32_t width = slice; width < n; width *= 2) {
#pragma omp parallel for num_threads(nt)
      for (int64_t lo = 0; lo < (int64_t)n; lo += 2 * (int64_t)width) {
        uint32_t mid = (uint32_t)lo + width;
        if (mid >= n) continue;
        uint32_t hi = mid + width < n ? mid + width : n;
        merge_dkeys(keys + lo, width, hi - mid, tmp + lo);
      }
    }
    free(tmp);
  }
  for (uint32_t i = 0; i < n; ++i) order_out[i] = keys[i].id;
  free(keys);
  return 0;
}

/* gpuSortPrototype.ts:120-163: keys = f32(-viewZ), sorted descending with
 * ties by ascending index (the bitonic comparator's total order). */
typedef struct { float key; uint32_t id; } fkey;
static int cmp_fkey_desc(const void* a, const void* b) {
  const fkey* x = (const fkey*)a; const fkey* y = (const fkey*)b;
  if (x->key > y->key) return -1;
  if (x->key < y->key) return 1;
  return x->id < y->id ? -1 : (x->id > y->id ? 1 : 0);
}

int orc_gpu_sort_prototype_order(const float* positions, uint32_t n, const float* view,
                                 uint32_t* order_out) {
  fkey* k = (fkey*)malloc(sizeof(fkey) * (n ? n : 1));
  if (!k) return -2;
  for (uint32_t i = 0; i < n; ++i) {
    double x = positions[(uint64_t)i * 3], y = positions[(uint64_t)i * 3 + 1], z = positions[(uint64_t)i * 3 + 2];
    double d = (double)view[2] * x + (double)view[6] * y + (double)view[10] * z + (double)view[14];
    k[i].key = (float)(-d);
    k[i].id = i;
  }
  qsort(k, n, sizeof(fkey), cmp_fkey_desc);
  for (uint32_t i = 0; i < n; ++i) order_out[i] = k[i].id;
  free(k);
  return 0;
}

/* ---------------------------------------------------------------------------
 * array forms of the scalar helpers (test convenience)
 * ------------------------------------------------------------------------- */
void orc_expf_n(const float* in, float* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_expf(in[i]); }
void orc_logf_n(const float* in, float* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_logf(in[i]); }
void orc_f16_rne_n(const float* in, uint16_t* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_f32_to_f16_rne(in[i]); }
void orc_f16_trunc_n(const float* in, uint16_t* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_f32_to_f16_trunc(in[i]); }
void orc_f16_to_f32_n(const uint16_t* in, float* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_f16_to_f32(in[i]); }
void orc_f64_to_f16_n(const double* in, uint16_t* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_f64_to_f16_rne(in[i]); }
void orc_composite_expf_n(const float* in, float* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_composite_expf(in[i]); }
void orc_splat_expf_n(const float* in, float* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_splat_expf(in[i]); }
void orc_splat_exp_parts_n(const float* in, float* p, uint32_t* kb, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) p[i] = orc_splat_exp_parts(in[i], kb + i);
}
void orc_morton_n(const uint32_t* x, const uint32_t* y, uint32_t* out, uint64_t n) { for (uint64_t i = 0; i < n; ++i) out[i] = orc_morton(x[i], y[i]); }
/* bucket (gpu_tile_bucket_sort.wgsl:85) and k20 of depths against one
 * tile's (min, max) depth bits; used to check bucket == k20 >> 13. */
void orc_bucket_key20_n(const uint32_t* depth_bits, uint64_t n, uint32_t dmin, uint32_t dmax,
                        uint32_t* buckets, uint32_t* keys) {
  tile_log tl = tile_log_params(dmin, dmax);
  for (uint64_t i = 0; i < n; ++i) {
    float ld = log_depth(depth_bits[i]);
    buckets[i] = bucket_of(ld, tl);
    keys[i] = key20_of(ld, tl);
  }
}
