// hdsr_math.cuh — scalar arithmetic shared by every kernel of the compositor.
//
// All translation units are compiled with -fmad=false: a product followed by
// a sum rounds twice unless the code calls fmaf() explicitly. exp/log are
// this project's own, because WGSL (the reference's shading language) leaves
// their precision to the implementation; the same op sequence defines the
// canonical frame on the CPU side.
//   exp: Cody-Waite reduction by ln2 (hi/lo split), degree-7 Taylor
//        polynomial (Horner, fma), two-step power-of-two scaling.
//   log: x = m*2^e, m in [sqrt(1/2), sqrt(2)], s = (m-1)/(m+1),
//        log(m) = 2 atanh(s) = 2s + 2s^3/3 + 2s^5/5 + 2s^7/7 + 2s^9/9.
#pragma once
#include <cuda_fp16.h>

#include <cstdint>

#ifndef HDSR_HD
#define HDSR_HD __host__ __device__ __forceinline__
#endif

namespace hdsr {

constexpr uint32_t kSentinel = 0xFFFFFFFFu;
constexpr uint32_t kLargeSplatTiles = 16u;     // gpu_classify_large_splats.wgsl:23
constexpr uint32_t kMaxTileEntries = 4096u;    // gpu_tile_classify.wgsl:11
constexpr uint32_t kKey20Max = 0xFFFFFu;
constexpr uint32_t kTilePx = 16u;

HDSR_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u; __builtin_memcpy(&u, &f, 4); return u;
#endif
}
HDSR_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f; __builtin_memcpy(&f, &u, 4); return f;
#endif
}

// WGSL min/max on f32 for the defined (non-NaN) path.
HDSR_HD float mn(float a, float b) { return a < b ? a : b; }
HDSR_HD float mx(float a, float b) { return a > b ? a : b; }
HDSR_HD float clampf(float x, float lo, float hi) { return mn(mx(x, lo), hi); }

// WGSL u32(f32): truncation toward zero, saturating, NaN -> 0.
HDSR_HD uint32_t sat_u32(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}

HDSR_HD float pow2i(int k) { return u2f((uint32_t)(k + 127) << 23); }

HDSR_HD float hx_expf(float x) {
  if (x != x) return x;
  if (x > 88.72283935546875f) return u2f(0x7F800000u);
  if (x < -103.97208404541015625f) return 0.0f;
  float k = rintf(x * 1.44269502162933349609375f);
  float r = fmaf(k, -0.693145751953125f, x);
  r = fmaf(k, -1.428606765330187045e-06f, r);
  float p = 1.98412701e-04f;
  p = fmaf(p, r, 1.38888892e-03f);
  p = fmaf(p, r, 8.33333377e-03f);
  p = fmaf(p, r, 4.16666679e-02f);
  p = fmaf(p, r, 1.66666672e-01f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int ki = (int)k;
  int k1 = ki / 2;
  int k2 = ki - k1;
  return (p * pow2i(k1)) * pow2i(k2);
}

HDSR_HD float hx_logf(float x) {
  if (x != x) return x;
  if (x < 0.0f) return u2f(0x7FC00000u);
  if (x == 0.0f) return u2f(0xFF800000u);
  if (x == u2f(0x7F800000u)) return x;
  uint32_t b = f2u(x);
  int e = 0;
  if (b < 0x00800000u) { x = x * 8388608.0f; b = f2u(x); e = -23; }
  e += (int)(b >> 23) - 127;
  float m = u2f((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421353816986083984375f) { m = m * 0.5f; e += 1; }
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  float q = 2.22222224e-01f;
  q = fmaf(q, z, 2.85714298e-01f);
  q = fmaf(q, z, 4.00000006e-01f);
  q = fmaf(q, z, 6.66666687e-01f);
  float lm = fmaf(s * z, q, 2.0f * s);
  float fe = (float)e;
  return fmaf(fe, 0.693145751953125f, fmaf(fe, 1.428606765330187045e-06f, lm));
}

// pack2x16float rounding: round-to-nearest-even, overflow -> inf, NaN -> 0x7E00.
// On the device the conversion instruction rounds the same way (cvt.rn.f16.f32);
// only its NaN encoding differs, so NaN is mapped first.
HDSR_HD uint32_t f32_to_f16(float f) {
#ifdef __CUDA_ARCH__
  if (f != f) return 0x7E00u;
  return (uint32_t)__half_as_ushort(__float2half_rn(f));
#else
  uint32_t x = f2u(f);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ax = x & 0x7FFFFFFFu;
  if (ax > 0x7F800000u) return 0x7E00u;
  if (ax >= 0x477FF000u) return sign | 0x7C00u;
  if (ax < 0x38800000u) {
    float m = rintf(u2f(ax) * 16777216.0f);
    return sign | (uint32_t)m;
  }
  uint32_t e = (ax >> 23) - 112u;
  uint32_t mant = ax & 0x7FFFFFu;
  uint32_t h = (e << 10) | (mant >> 13);
  uint32_t rem = mant & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1u;
  return sign | h;
#endif
}

// f16 -> f32 is exact; the device instruction keeps every value, NaNs are
// rebuilt with their payload as the host path does.
HDSR_HD float f16_to_f32(uint32_t h) {
#ifdef __CUDA_ARCH__
  if ((h & 0x7C00u) == 0x7C00u && (h & 0x3FFu) != 0u)
    return u2f(((h & 0x8000u) << 16) | 0x7F800000u | ((h & 0x3FFu) << 13));
  return __half2float(__ushort_as_half((unsigned short)(h & 0xFFFFu)));
#else
  uint32_t sign = (h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1Fu;
  uint32_t m = h & 0x3FFu;
  if (e == 0) {
    float v = (float)m * 5.9604644775390625e-08f;
    return sign ? -v : v;
  }
  if (e == 31) return u2f(sign | 0x7F800000u | (m << 13));
  return u2f(sign | ((e + 112u) << 23) | (m << 13));
#endif
}

HDSR_HD uint32_t pack2x16(float a, float b) { return f32_to_f16(a) | (f32_to_f16(b) << 16); }
HDSR_HD float lo16(uint32_t w) { return f16_to_f32(w & 0xFFFFu); }
HDSR_HD float hi16(uint32_t w) { return f16_to_f32(w >> 16); }

// exp on a wide range (the deferred passes' weights, x > -86: weight_expf;
// the rasterisers use splat_expf below): Cody-Waite reduction r = x - k ln2
// (|r| <= ln2/2, ln2 split in two), then a degree-5 polynomial in r fitted
// for least maximum relative error on that interval (this project's own Remez
// fit: 7.5e-8 in exact arithmetic, at most 3 ulp in f32 Horner steps against
// the true exp down to -86). The scale 2^k is a normal float for k >= -126.
// k is the integer nearest the exact x log2(e): the fma adds 1.5 * 2^23, where
// the float spacing is 1, so its rounding rounds the product to an integer
// and leaves k + 2^22 in the low mantissa bits (no conversion instructions);
// shifted into the exponent field those bits give 2^k.
HDSR_HD float composite_expf(float x) {
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
  return p * u2f((f2u(t) << 23) + 0x3F800000u);
}

// The rasterisers' exp of a splat's power, whose value is used only for a
// power in (-4, 0] (k in [-6, 0]): the steps of composite_expf with one
// reduction constant, ln 2 rounded to f32 (1.9e-9 above ln 2, so k * ln2f is
// off by at most 1.2e-8 for |k| <= 6, below the polynomial's own error).
// exp(x) = p * 2^k, returned as p and kb = k << 23 (mod 2^32), the bits that
// put 2^k into a float's exponent field: the rasterisers scale the opacity by
// 2^k with one integer add instead of forming 2^k and multiplying by it
// (exact for a normal or zero opacity with a normal product, so the alpha
// keeps the bits of opacity * splat_expf(x)).
struct SplatExp {
  float p;
  uint32_t kb;
};
HDSR_HD SplatExp splat_exp_parts(float x) {
  const float t = fmaf(x, 1.44269502162933349609375f, 12582912.0f);
  const float k = t - 12582912.0f;
  const float r = fmaf(k, -0.693147182464599609375f, x);
  float p = 0x1.0fe5c6p-7f;
  p = fmaf(p, r, 0x1.575eeep-5f);
  p = fmaf(p, r, 0x1.555a18p-3f);
  p = fmaf(p, r, 0x1.fffd1ap-2f);
  p = fmaf(p, r, 0x1.fffff6p-1f);
  p = fmaf(p, r, 0x1.000002p+0f);
  return SplatExp{p, f2u(t) << 23};
}
HDSR_HD float splat_expf(float x) {
  const SplatExp e = splat_exp_parts(x);
  return e.p * u2f(e.kb + 0x3F800000u);
}

// 16-bit x/y interleave, x on even bits (gpu_tile_splat_composite.wgsl:33-47).
HDSR_HD uint32_t morton(uint32_t x, uint32_t y) {
  uint32_t a = x & 0xFFFFu;
  a = (a | (a << 8)) & 0x00FF00FFu;
  a = (a | (a << 4)) & 0x0F0F0F0Fu;
  a = (a | (a << 2)) & 0x33333333u;
  a = (a | (a << 1)) & 0x55555555u;
  uint32_t b = y & 0xFFFFu;
  b = (b | (b << 8)) & 0x00FF00FFu;
  b = (b | (b << 4)) & 0x0F0F0F0Fu;
  b = (b | (b << 2)) & 0x33333333u;
  b = (b | (b << 1)) & 0x55555555u;
  return a | (b << 1);
}

// The even bits of m, compacted (inverse of the interleave above).
HDSR_HD uint32_t morton_even(uint32_t m) {
  m &= 0x55555555u;
  m = (m | (m >> 1)) & 0x33333333u;
  m = (m | (m >> 2)) & 0x0F0F0F0Fu;
  m = (m | (m >> 4)) & 0x00FF00FFu;
  m = (m | (m >> 8)) & 0x0000FFFFu;
  return m;
}

// Per-tile log-depth mapping of the hot-tile bucket cascade
// (gpu_tile_bucket_sort.wgsl:75-85), scaled to 2^20 keys instead of 128
// buckets: keyScale = 1048576/R = 8192 * (128/R) exactly, so a key's top
// seven bits are the reference bucket.
HDSR_HD float2 tile_log_params(uint32_t dmin_bits, uint32_t dmax_bits) {
  float logMin = hx_logf(mx(u2f(dmin_bits), 1e-6f));
  float logRange = hx_logf(mx(u2f(dmax_bits), 1e-6f)) - logMin;
  float keyScale = logRange < 1e-10f ? 0.0f : 1048576.0f / logRange;
  return make_float2(logMin, keyScale);
}

HDSR_HD float log_depth(uint32_t dbits) { return hx_logf(mx(u2f(dbits), 1e-6f)); }

HDSR_HD uint32_t key20(float logd, float2 tl) {
  uint32_t k = sat_u32((logd - tl.x) * tl.y);
  return k < kKey20Max ? k : kKey20Max;
}

}  // namespace hdsr
