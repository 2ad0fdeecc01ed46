// hdsr_post_math.cuh — scalar and vector arithmetic of the deferred passes
// (screen-space normals, bilateral filter, GTAO, bloom, IBL, lighting).
//
// WGSL leaves the precision of sin/cos/atan2/asin/pow/log2/exp to the
// implementation; these are this project's own, written from textbook
// methods, so that the CPU oracle can restate the same operation sequence:
//   sin/cos: Cody-Waite reduction by pi/2 (three-part constant, the first two
//            with 12 significant bits so k*C1, k*C2 are exact for |k| < 2^11),
//            Taylor polynomials on [-pi/4, pi/4] (sin to r^9, cos to r^10).
//   atan2:   octant reduction to a = min/max in [0,1], a > tan(pi/8) mapped
//            through atan(a) = pi/4 + atan((a-1)/(a+1)), odd Taylor series to
//            t^19 on |t| <= tan(pi/8).
//   asin:    atan2(x, sqrt((1-x)(1+x))).
//   pow:     exp(y*log(x)) with the compositor's exp/log; log2 = log * log2(e).
// Every product and sum is written out; the library is compiled with
// -fmad=false, so nothing is contracted behind the source's back.
#pragma once
#include "hdsr_math.cuh"

namespace hdsr {

struct F3 { float x, y, z; };

HDSR_HD F3 f3(float x, float y, float z) { F3 r; r.x = x; r.y = y; r.z = z; return r; }
HDSR_HD F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
HDSR_HD F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
HDSR_HD F3 mul(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
HDSR_HD F3 muls(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
HDSR_HD F3 divs(F3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
HDSR_HD F3 neg(F3 a) { return f3(-a.x, -a.y, -a.z); }
HDSR_HD float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HDSR_HD F3 cross(F3 a, F3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
HDSR_HD float length(F3 a) { return sqrtf(dot(a, a)); }
HDSR_HD F3 normalize(F3 a) { return divs(a, length(a)); }
HDSR_HD float sat(float x) { return clampf(x, 0.0f, 1.0f); }
// WGSL mix(a, b, t) = a * (1 - t) + b * t
HDSR_HD float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
HDSR_HD F3 mix3(F3 a, F3 b, float t) { return f3(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)); }
HDSR_HD float smoothstepf(float e0, float e1, float x) {
  float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
HDSR_HD float fractf(float x) { return x - floorf(x); }
// WGSL i32(f32): truncation toward zero, saturating, NaN -> 0.
HDSR_HD int to_i32(float x) {
  if (!(x == x)) return 0;
  if (x >= 2147483520.0f) return 2147483647;
  if (x <= -2147483648.0f) return -2147483647 - 1;
  return (int)x;
}
HDSR_HD int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// column-major mat4 * vec4(x, y, z, w): ((c0*x + c1*y) + c2*z) + c3*w
HDSR_HD void mat4_mul(const float* m, float x, float y, float z, float w, float out[4]) {
  for (int r = 0; r < 4; ++r) out[r] = m[r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}

HDSR_HD void px_sincos(float x, float* s, float* c) {
  float k = rintf(x * 0.636619746685028076171875f);
  float r = x - k * 1.5703125f;
  r = r - k * 4.837512969970703125e-4f;
  r = r - k * 7.549790126404332e-08f;
  float z = r * r;
  float ps = 2.75573192e-06f;            // 1/9!
  ps = ps * z + -1.98412698e-04f;        // -1/7!
  ps = ps * z + 8.33333333e-03f;         // 1/5!
  ps = ps * z + -1.66666667e-01f;        // -1/3!
  float sr = r + (r * z) * ps;
  float pc = -2.75573192e-07f;           // -1/10!
  pc = pc * z + 2.48015873e-05f;         // 1/8!
  pc = pc * z + -1.38888889e-03f;        // -1/6!
  pc = pc * z + 4.16666667e-02f;         // 1/4!
  pc = pc * z + -0.5f;
  float cr = 1.0f + z * pc;
  int q = ((int)k) & 3;
  if (q == 0) { *s = sr; *c = cr; }
  else if (q == 1) { *s = cr; *c = -sr; }
  else if (q == 2) { *s = -sr; *c = -cr; }
  else { *s = -cr; *c = sr; }
}
HDSR_HD float px_sin(float x) { float s, c; px_sincos(x, &s, &c); return s; }
HDSR_HD float px_cos(float x) { float s, c; px_sincos(x, &s, &c); return c; }

// atan on [0, 1]
HDSR_HD float px_atan01(float a) {
  float base = 0.0f, t = a;
  if (a > 0.414213567972183227539f) { t = (a - 1.0f) / (a + 1.0f); base = 0.785398185253143310547f; }
  float z = t * t;
  float p = -0.0526315789f;              // -1/19
  p = p * z + 0.0588235294f;             // 1/17
  p = p * z + -0.0666666667f;            // -1/15
  p = p * z + 0.0769230769f;             // 1/13
  p = p * z + -0.0909090909f;            // -1/11
  p = p * z + 0.111111111f;              // 1/9
  p = p * z + -0.142857143f;             // -1/7
  p = p * z + 0.2f;                      // 1/5
  p = p * z + -0.333333333f;             // -1/3
  return base + (t + (t * z) * p);
}

HDSR_HD float px_atan2(float y, float x) {
  if (!(x == x) || !(y == y)) return x + y;
  float ax = fabsf(x), ay = fabsf(y);
  bool swap = ay > ax;
  float num = swap ? ax : ay, den = swap ? ay : ax;
  float a;
  if (den == 0.0f) a = 0.0f;
  else if (den == u2f(0x7F800000u)) a = (num == den) ? 1.0f : 0.0f;
  else a = num / den;
  float r = px_atan01(a);
  if (swap) r = 1.57079637050628662109f - r;
  if (x < 0.0f || (x == 0.0f && (f2u(x) >> 31))) r = 3.14159274101257324219f - r;
  return (f2u(y) >> 31) ? -r : r;
}

HDSR_HD float px_asin(float x) { return px_atan2(x, sqrtf((1.0f - x) * (1.0f + x))); }

HDSR_HD float px_log2(float x) { return hx_logf(x) * 1.44269502162933349609f; }

// exp and pow where the exponent stays below a few units (the bilateral
// filter's weights; the lighting's sRGB transfer of values in [0, ~1] and
// Schlick's (1 - cos)^5): exp as the composite's (fma-rounded k, Cody-Waite,
// degree-5 fit; the 2^k scale is exact for the k >= -126 that x > -86
// gives), 0 below -86, where the value would be denormal.
HDSR_HD float weight_expf(float x) { return x > -86.0f ? composite_expf(x) : 0.0f; }
HDSR_HD float weight_pow(float x, float y) {
  if (x == 1.0f || y == 0.0f) return 1.0f;
  if (!(x == x) || !(y == y)) return u2f(0x7FC00000u);
  if (x == 0.0f) return y > 0.0f ? 0.0f : u2f(0x7F800000u);
  if (x < 0.0f) return u2f(0x7FC00000u);
  return weight_expf(y * hx_logf(x));
}

HDSR_HD float px_pow(float x, float y) {
  if (x == 1.0f || y == 0.0f) return 1.0f;
  if (!(x == x) || !(y == y)) return u2f(0x7FC00000u);
  if (x == 0.0f) return y > 0.0f ? 0.0f : u2f(0x7F800000u);
  if (x < 0.0f) return u2f(0x7FC00000u);
  return hx_expf(y * hx_logf(x));
}

// Octahedral normal coding (gpu_screen_space_normals.wgsl:36-53)
HDSR_HD void oct_enc(F3 n, float* ox, float* oy) {
  float sum = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
  float px = n.x / sum, py = n.y / sum;
  if (n.z < 0.0f) {
    float qx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
    float qy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
    px = qx; py = qy;
  }
  *ox = px; *oy = py;
}
HDSR_HD F3 oct_dec(float ex, float ey) {
  F3 n = f3(ex, ey, 1.0f - fabsf(ex) - fabsf(ey));
  if (n.z < 0.0f) {
    float nx = (1.0f - fabsf(n.y)) * (n.x >= 0.0f ? 1.0f : -1.0f);
    float ny = (1.0f - fabsf(n.x)) * (n.y >= 0.0f ? 1.0f : -1.0f);
    n.x = nx; n.y = ny;
  }
  return normalize(n);
}
HDSR_HD F3 oct_dec_word(uint32_t w) { return oct_dec(lo16(w), hi16(w)); }
HDSR_HD uint32_t oct_word(F3 n) { float ox, oy; oct_enc(n, &ox, &oy); return pack2x16(ox, oy); }
HDSR_HD F3 face_forward(F3 normal, F3 view_dir) {
  F3 n = normalize(normal);
  F3 v = normalize(view_dir);
  return dot(n, v) < 0.0f ? neg(n) : n;
}

}  // namespace hdsr
