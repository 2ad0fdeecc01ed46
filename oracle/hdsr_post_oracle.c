/*
 * hdsr_post_oracle.c — CPU restatement of the reference's deferred frame
 * tail (the passes splatRenderer.ts:1042-1139 encodes after the compositor).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA passes in
 * hdsr_post.cu; only the test suite and the smoke check call it.
 *
 * Restated (paths inside the reference):
 *   src/shaders/gpu_screen_space_normals.wgsl:55-119   orp_ss_normals
 *   src/shaders/bilateral_normal_filter.wgsl:39-86     orp_bilateral
 *   src/shaders/gtao_depth_prefilter.wgsl:27-72        orp_gtao_prefilter
 *   src/shaders/gtao_main.wgsl:29-222                  orp_gtao_main
 *   src/shaders/gtao_denoise.wgsl:17-95                orp_gtao_denoise
 *   src/shaders/bloom_threshold.wgsl:16-42             orp_bloom_threshold
 *   src/shaders/bloom_blur.wgsl:19-37                  orp_bloom_blur
 *   src/shaders/gpu_deferred_lighting.wgsl:32-269      orp_lighting
 *   src/shaders/ibl_brdf_lut.wgsl:20-97                orp_brdf_lut
 *   src/shaders/ibl_mipgen.wgsl:7-19                   orp_env_mip
 *   src/materialCurves.ts:26-55                        orp_curve_lut
 * with the uniform values of their encode() functions (splatRenderer.ts
 * :350-365, :414-420, :505-523; gtao.ts:143-168; bloom.ts:120-170).
 *
 * Parity status: "parity unpinned". The reference runs these passes in a
 * browser's WebGPU and has no test that fixes their outputs; this file is a
 * transcription checked by review and by property tests.
 *
 * Canonical choices where WGSL leaves room: sin/cos/atan2/asin/pow/log2/exp
 * are this project's own (below; exp/log are orc_expf/orc_logf); textureLoad
 * outside an image clamps to the edge (Tint's robustness transform); a
 * filtering sampler is bilinear in f32, rows mixed as t0*(1-a) + t1*a and
 * then by (1-b), b, trilinear as s0*(1-f) + s1*f; rgba16float stores round to
 * nearest even. Compiled with -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "hdsr_oracle.h"

typedef struct { float x, y, z; } f3;

static inline f3 F3(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f3 add(f3 a, f3 b) { return F3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 sub(f3 a, f3 b) { return F3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 muls(f3 a, float s) { return F3(a.x * s, a.y * s, a.z * s); }
static inline f3 divs(f3 a, float s) { return F3(a.x / s, a.y / s, a.z / s); }
static inline f3 neg(f3 a) { return F3(-a.x, -a.y, -a.z); }
static inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 cross(f3 a, f3 b) { return F3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float len(f3 a) { return sqrtf(dot(a, a)); }
static inline f3 nrm(f3 a) { return divs(a, len(a)); }
static inline float fmn(float a, float b) { return a < b ? a : b; }
static inline float fmx(float a, float b) { return a > b ? a : b; }
static inline float clampf(float x, float lo, float hi) { return fmn(fmx(x, lo), hi); }
static inline float sat(float x) { return clampf(x, 0.0f, 1.0f); }
static inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static inline f3 mix3(f3 a, f3 b, float t) { return F3(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)); }
static inline float smoothstep_(float e0, float e1, float x) {
  float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline uint32_t fb(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float bf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline int i32_of(float x) {
  if (!(x == x)) return 0;
  if (x >= 2147483520.0f) return 2147483647;
  if (x <= -2147483648.0f) return -2147483647 - 1;
  return (int)x;
}
static inline uint32_t pk(float a, float b) {
  return (uint32_t)orc_f32_to_f16_rne(a) | ((uint32_t)orc_f32_to_f16_rne(b) << 16);
}
static inline float lo(uint32_t w) { return orc_f16_to_f32((uint16_t)(w & 0xFFFFu)); }
static inline float hi(uint32_t w) { return orc_f16_to_f32((uint16_t)(w >> 16)); }
static inline void store4(uint16_t* p, float r, float g, float b, float a) {
  p[0] = orc_f32_to_f16_rne(r); p[1] = orc_f32_to_f16_rne(g);
  p[2] = orc_f32_to_f16_rne(b); p[3] = orc_f32_to_f16_rne(a);
}
static inline void load4(const uint16_t* p, float o[4]) {
  for (int i = 0; i < 4; ++i) o[i] = orc_f16_to_f32(p[i]);
}
/* column-major mat4 * vec4 */
static inline void mat4v(const float* m, float x, float y, float z, float w, float o[4]) {
  for (int r = 0; r < 4; ++r) o[r] = m[r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}

/* ---- elementary functions (methods named in hdsr_post_math.cuh) ---- */
static void orp_sincos(float x, float* s, float* c) {
  float k = rintf(x * 0.636619746685028076171875f);     /* 2/pi */
  float r = x - k * 1.5703125f;                          /* pi/2 in three parts */
  r = r - k * 4.837512969970703125e-4f;
  r = r - k * 7.549790126404332e-08f;
  float z = r * r;
  float ps = 2.75573192e-06f;
  ps = ps * z + -1.98412698e-04f;
  ps = ps * z + 8.33333333e-03f;
  ps = ps * z + -1.66666667e-01f;
  float sr = r + (r * z) * ps;
  float pc = -2.75573192e-07f;
  pc = pc * z + 2.48015873e-05f;
  pc = pc * z + -1.38888889e-03f;
  pc = pc * z + 4.16666667e-02f;
  pc = pc * z + -0.5f;
  float cr = 1.0f + z * pc;
  switch (((int)k) & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}

static float orp_atan01(float a) {
  float base = 0.0f, t = a;
  if (a > 0.414213567972183227539f) { t = (a - 1.0f) / (a + 1.0f); base = 0.785398185253143310547f; }
  float z = t * t;
  float p = -0.0526315789f;
  p = p * z + 0.0588235294f;
  p = p * z + -0.0666666667f;
  p = p * z + 0.0769230769f;
  p = p * z + -0.0909090909f;
  p = p * z + 0.111111111f;
  p = p * z + -0.142857143f;
  p = p * z + 0.2f;
  p = p * z + -0.333333333f;
  return base + (t + (t * z) * p);
}

float orp_atan2(float y, float x) {
  if (!(x == x) || !(y == y)) return x + y;
  float ax = fabsf(x), ay = fabsf(y);
  int swap = ay > ax;
  float num = swap ? ax : ay, den = swap ? ay : ax;
  float a;
  if (den == 0.0f) a = 0.0f;
  else if (den == bf(0x7F800000u)) a = (num == den) ? 1.0f : 0.0f;
  else a = num / den;
  float r = orp_atan01(a);
  if (swap) r = 1.57079637050628662109f - r;
  if (x < 0.0f || (x == 0.0f && (fb(x) >> 31))) r = 3.14159274101257324219f - r;
  return (fb(y) >> 31) ? -r : r;
}
float orp_asin(float x) { return orp_atan2(x, sqrtf((1.0f - x) * (1.0f + x))); }
float orp_sin(float x) { float s, c; orp_sincos(x, &s, &c); return s; }
float orp_cos(float x) { float s, c; orp_sincos(x, &s, &c); return c; }
float orp_log2(float x) { return orc_logf(x) * 1.44269502162933349609f; }
float orp_pow(float x, float y) {
  if (x == 1.0f || y == 0.0f) return 1.0f;
  if (!(x == x) || !(y == y)) return bf(0x7FC00000u);
  if (x == 0.0f) return y > 0.0f ? 0.0f : bf(0x7F800000u);
  if (x < 0.0f) return bf(0x7FC00000u);
  return orc_expf(y * orc_logf(x));
}

/* exp and pow where the exponent stays below a few units (the bilateral
 * filter's weights, the lighting's sRGB transfer and Schlick's (1 - cos)^5):
 * the composite's exp, 0 below -86 (a denormal value); pow through it. The
 * kernels' weight_expf / weight_pow, the same steps. */
float orp_weight_expf(float x) { return x > -86.0f ? orc_composite_expf(x) : 0.0f; }
float orp_weight_pow(float x, float y) {
  if (x == 1.0f || y == 0.0f) return 1.0f;
  if (!(x == x) || !(y == y)) return bf(0x7FC00000u);
  if (x == 0.0f) return y > 0.0f ? 0.0f : bf(0x7F800000u);
  if (x < 0.0f) return bf(0x7FC00000u);
  return orp_weight_expf(y * orc_logf(x));
}

/* octEncode / octDecode / faceForwardNormal (gpu_screen_space_normals.wgsl:36-59) */
static inline void oct_xy(f3 n, float* ox, float* oy) {
  float sum = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
  float px = n.x / sum, py = n.y / sum;
  if (n.z < 0.0f) {
    float qx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
    float qy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
    px = qx; py = qy;
  }
  *ox = px; *oy = py;
}
static inline uint32_t oct_pack(f3 n) {
  float ox, oy;
  oct_xy(n, &ox, &oy);
  return pk(ox, oy);
}
static inline f3 oct_unpack2(float ex, float ey) {
  f3 n = F3(ex, ey, 1.0f - fabsf(ex) - fabsf(ey));
  if (n.z < 0.0f) {
    float nx = (1.0f - fabsf(n.y)) * (n.x >= 0.0f ? 1.0f : -1.0f);
    float ny = (1.0f - fabsf(n.x)) * (n.y >= 0.0f ? 1.0f : -1.0f);
    n.x = nx; n.y = ny;
  }
  return nrm(n);
}
static inline f3 oct_unpack(uint32_t w) { return oct_unpack2(lo(w), hi(w)); }
static inline f3 face_fwd(f3 normal, f3 view) {
  f3 n = nrm(normal), v = nrm(view);
  return dot(n, v) < 0.0f ? neg(n) : n;
}

static inline f3 recon(const orp_inputs* in, const orp_params* q, float px, float py, float d) {
  float nx = px / (float)in->W * 2.0f - 1.0f;
  float ny = 1.0f - py / (float)in->H * 2.0f;
  float w[4];
  mat4v(q->view_proj_inverse, nx, ny, d, 1.0f, w);
  return F3(w[0] / w[3], w[1] / w[3], w[2] / w[3]);
}
#define DEPTH(x, y) (in->depth[(size_t)(y) * in->W + (x)])

void orp_ss_normals(const orp_inputs* in, const orp_params* q, uint32_t* out) {
  const int W = in->W, H = in->H;
  const float mode = (float)q->normal_recovery_mode;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t i = (size_t)y * W + x;
      float d = DEPTH(x, y);
      if (d >= 0.9999f) { out[i] = mode > 0.5f ? in->normal[i] : pk(0.0f, 0.0f); continue; }
      float cx = (float)x + 0.5f, cy = (float)y + 0.5f;
      f3 pc = recon(in, q, cx, cy, d);
      float dL = DEPTH(x > 0 ? x - 1 : 0, y), dR = DEPTH(x + 1 < W ? x + 1 : W - 1, y);
      float dU = DEPTH(x, y > 0 ? y - 1 : 0), dD = DEPTH(x, y + 1 < H ? y + 1 : H - 1);
      f3 ddx = fabsf(dL - d) < fabsf(dR - d) ? sub(pc, recon(in, q, cx - 1.0f, cy - 0.0f, dL))
                                             : sub(recon(in, q, cx + 1.0f, cy + 0.0f, dR), pc);
      f3 ddy = fabsf(dU - d) < fabsf(dD - d) ? sub(pc, recon(in, q, cx - 0.0f, cy - 1.0f, dU))
                                             : sub(recon(in, q, cx + 0.0f, cy + 1.0f, dD), pc);
      f3 vd = nrm(sub(F3(q->camera_pos[0], q->camera_pos[1], q->camera_pos[2]), pc));
      f3 sn = face_fwd(nrm(cross(ddy, ddx)), vd);
      f3 src = face_fwd(oct_unpack(in->normal[i]), vd);
      f3 n = sn;
      if (mode > 1.5f) n = src;
      else if (mode > 0.5f) {
        float ndv = fmx(dot(src, vd), 0.0f);
        float blend = 1.0f - smoothstep_(q->grazing_start, q->grazing_end, ndv);
        n = nrm(mix3(src, sn, blend));
      }
      out[i] = oct_pack(n);
    }
}

void orp_bilateral(const orp_inputs* in, const orp_params* q, const uint32_t* ssn, uint32_t* out) {
  const int W = in->W, H = in->H, R = (int)q->bilateral_radius;
  const float ss = q->bilateral_spatial_sigma, sdv = q->bilateral_depth_sigma;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t i = (size_t)y * W + x;
      f3 cn = oct_unpack(ssn[i]);
      float cd = DEPTH(x, y);
      if (cd >= 0.9999f) { out[i] = ssn[i]; continue; }
      f3 acc = F3(0.0f, 0.0f, 0.0f);
      float total = 0.0f;
      for (int dy = -R; dy <= R; ++dy)
        for (int dx = -R; dx <= R; ++dx) {
          int sx = clampi(x + dx, 0, W - 1), sy = clampi(y + dy, 0, H - 1);
          f3 sn = oct_unpack(ssn[(size_t)sy * W + sx]);
          float sd = DEPTH(sx, sy);
          float dist2 = (float)(dx * dx + dy * dy);
          float spatialW = orc_expf(-dist2 / (2.0f * ss * ss));
          /* divisions by per-pixel constants as multiplications by their
           * reciprocals (within WGSL's 2.5 ulp division), as the kernel */
          float inv_dden = 1.0f / fmx(cd, 0.001f);
          float neg_inv_sd2 = -(1.0f / (2.0f * sdv * sdv));
          float depthDiff = fabsf(cd - sd) * inv_dden;
          float depthW = orp_weight_expf((depthDiff * depthDiff) * neg_inv_sd2);
          float normalW = orp_weight_pow(fmx(dot(cn, sn), 0.0f), 1.0f / fmx(q->bilateral_normal_sigma, 0.01f));
          float w = spatialW * depthW * normalW;
          acc = add(acc, muls(sn, w));
          total = total + w;
        }
      out[i] = oct_pack(nrm(divs(acc, fmx(total, 0.0001f))));
    }
}

void orp_gtao_prefilter(const orp_inputs* in, const orp_params* q, float* mip0, float* mip1, float* mip2) {
  const int W = in->W, H = in->H, m1w = (W + 1) / 2, m2w = (W + 3) / 4;
  const float n = q->near_plane, f = q->far_plane;
  /* one 16x16 workgroup at a time: its shared array holds the clamped, linearised tile */
  const int bw = (W + 15) / 16, bh = (H + 15) / 16;
#pragma omp parallel for schedule(static)
  for (int b = 0; b < bw * bh; ++b) {
    float s[256];
    int bx = (b % bw) * 16, by = (b / bw) * 16;
    for (int ly = 0; ly < 16; ++ly)
      for (int lx = 0; lx < 16; ++lx) {
        int x = bx + lx, y = by + ly;
        float raw = DEPTH(clampi(x, 0, W - 1), clampi(y, 0, H - 1));
        float lin = n * f / (f - raw * (f - n));
        if (x < W && y < H) mip0[(size_t)y * W + x] = lin;
        s[ly * 16 + lx] = lin;
      }
    for (int ly = 0; ly < 16; ly += 2)
      for (int lx = 0; lx < 16; lx += 2) {
        int li = ly * 16 + lx, x = bx + lx, y = by + ly;
        float v = fmn(fmn(s[li], s[li + 1]), fmn(s[li + 16], s[li + 17]));
        if (x < W && y < H) mip1[(size_t)(y / 2) * m1w + x / 2] = v;
        s[li] = v;
      }
    for (int ly = 0; ly < 16; ly += 4)
      for (int lx = 0; lx < 16; lx += 4) {
        int li = ly * 16 + lx, x = bx + lx, y = by + ly;
        float v = fmn(fmn(s[li], s[li + 2]), fmn(s[li + 32], s[li + 34]));
        if (x < W && y < H) mip2[(size_t)(y / 4) * m2w + x / 4] = v;
      }
  }
}

static uint32_t hilbert_index(uint32_t x, uint32_t y) {
  uint32_t rx, ry, s = 8u, d = 0u;
  for (;;) {
    if (s == 0u) break;
    s = s >> 1u;
    rx = (x & s) > 0u ? 1u : 0u;
    ry = (y & s) > 0u ? 1u : 0u;
    d += s * s * ((3u * rx) ^ ry);
    if (ry == 0u) {
      if (rx == 1u) { x = s * 2u - 1u - x; y = s * 2u - 1u - y; }
      uint32_t t = x; x = y; y = t;
    }
  }
  return d;
}

typedef struct { const float* m[3]; int w[3], h[3]; float pi[4]; const orp_params* q; } gtao_ctx;

static inline float mip_sample(const gtao_ctx* c, float u, float v, int level) {
  int w = c->w[level], h = c->h[level];
  int cx = clampi(i32_of(u * (float)w), 0, w - 1), cy = clampi(i32_of(v * (float)h), 0, h - 1);
  return c->m[level][(size_t)cy * w + cx];
}
static inline f3 vpos(const gtao_ctx* c, float u, float v, float d) {
  return F3((u * c->pi[0] + c->pi[2]) * d, (v * c->pi[1] + c->pi[3]) * d, -d);
}
/* divisions by frame constants as multiplications by reciprocals taken
 * once, as the kernel (within WGSL's 2.5 ulp division); dot / dist stays */
static inline float horizon(const gtao_ctx* c, float u, float v, int mip, f3 vp, f3 vn, float inv_thick,
                            float inv_falloff, float best) {
  if (u >= 0.0f && u <= 1.0f && v >= 0.0f && v <= 1.0f) {
    f3 diff = sub(vpos(c, u, v, mip_sample(c, u, v, mip)), vp);
    float dist = len(diff);
    if (dist > 0.001f) {
      float zr = fabsf(diff.z) * inv_thick;
      float tw = sat(1.0f - zr * zr);
      float hz = dot(diff, vn) / dist;
      float fo = sat(1.0f - dist * inv_falloff);
      best = fmx(best, hz * fo * tw);
    }
  }
  return best;
}

void orp_gtao_main(const orp_inputs* in, const orp_params* q, const float* mip0, const float* mip1, const float* mip2,
                   const uint32_t* nrm_img, uint16_t* ao_raw) {
  const int W = in->W, H = in->H;
  gtao_ctx c;
  c.m[0] = mip0; c.m[1] = mip1; c.m[2] = mip2;
  c.w[0] = W; c.h[0] = H; c.w[1] = (W + 1) / 2; c.h[1] = (H + 1) / 2; c.w[2] = (W + 3) / 4; c.h[2] = (H + 3) / 4;
  c.pi[0] = (float)(2.0 / (double)q->proj[0]);
  c.pi[1] = (float)(-2.0 / (double)q->proj[5]);
  c.pi[2] = (float)(-1.0 / (double)q->proj[0]);
  c.pi[3] = (float)(1.0 / (double)q->proj[5]);
  c.q = q;
  const float vw = (float)W, vh = (float)H;
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t i = (size_t)y * W + x;
      uint16_t* o = ao_raw + 4 * i;
      float u = ((float)x + 0.5f) / vw, v = ((float)y + 0.5f) / vh;
      float cd = mip0[i];
      if (cd <= 0.0f || cd > q->ao_falloff_end * 10.0f) { store4(o, 1.0f, 0.0f, 1.0f, 0.0f); continue; }
      f3 vp = vpos(&c, u, v, cd);
      f3 wn = oct_unpack(nrm_img[i]);
      float t4[4];
      mat4v(q->view, wn.x, wn.y, wn.z, 0.0f, t4);
      f3 vn = face_fwd(nrm(F3(t4[0], t4[1], t4[2])), nrm(neg(vp)));
      float focal = vw / fabsf(c.pi[0]);
      float pr = fmx(q->ao_radius_world * focal / cd, 1.0f);
      uint32_t ridx = hilbert_index((uint32_t)x & 15u, (uint32_t)y & 15u) + q->frame_counter * 256u;
      const float a1 = 0.754877686500549316406f, a2 = a1 * a1;
      float sox = (float)ridx * a1 + 0.5f, soy = (float)ridx * a2 + 0.5f;
      sox = sox - floorf(sox);
      soy = soy - floorf(soy);
      const float inv_vw = 1.0f / vw, inv_vh = 1.0f / vh;
      const float inv_thick = 1.0f / q->ao_thickness, inv_falloff = 1.0f / q->ao_falloff_end;
      float total = 0.0f;
      f3 bent = F3(0.0f, 0.0f, 0.0f);
      for (uint32_t sl = 0; sl < q->ao_slices; ++sl) {
        float phi = (3.14159274101257324219f / (float)q->ao_slices) * ((float)sl + sox);
        float ds, dc;
        orp_sincos(phi, &ds, &dc);
        float bp = -1.0f, bn = -1.0f;
        for (uint32_t st = 1; st <= q->ao_steps; ++st) {
          float t = ((float)st + soy * 0.5f) / (float)q->ao_steps;
          float ox = dc * pr * t * inv_vw, oy = ds * pr * t * inv_vh;
          int mip = i32_of(clampf(orp_log2(pr * t / 4.0f), 0.0f, 2.0f));
          bp = horizon(&c, u + ox, v + oy, mip, vp, vn, inv_thick, inv_falloff, bp);
          bn = horizon(&c, u - ox, v - oy, mip, vp, vn, inv_thick, inv_falloff, bn);
        }
        float nds = vn.x * dc + vn.y * ds + vn.z * 0.0f;
        float cp = fmx(bp, nds * 0.08f), cn = fmx(bn, -nds * 0.08f);
        total = total + (cp + cn);
        float vP = 1.0f - cp, vN = 1.0f - cn;
        bent = add(bent, add(muls(F3(dc, ds, 0.0f), vP - vN), muls(vn, vP + vN)));
      }
      total = total / ((float)q->ao_slices * 2.0f);
      float ao = sat(1.0f - total * q->ao_intensity);
      float bl = len(bent);
      f3 bvs = bl > 0.001f ? divs(bent, bl) : vn;
      const float* m = q->view;
      f3 bw = nrm(F3(dot(F3(m[0], m[4], m[8]), bvs), dot(F3(m[1], m[5], m[9]), bvs), dot(F3(m[2], m[6], m[10]), bvs)));
      float bx, by;
      oct_xy(bw, &bx, &by);
      store4(o, ao, bx, by, 0.0f);
    }
}

void orp_gtao_denoise(const orp_inputs* in, const orp_params* q, const uint16_t* ao_raw, const float* mip0,
                      uint16_t* ao) {
  const int W = in->W, H = in->H;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t i = (size_t)y * W + x;
      float cd = mip0[i], acc[4], na[4];
      load4(ao_raw + 4 * i, acc);
      float total = 1.0f;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          if (dx == 0 && dy == 0) continue;
          size_t ni = (size_t)clampi(y + dy, 0, H - 1) * W + clampi(x + dx, 0, W - 1);
          float dd = fabsf(cd - mip0[ni]) / fmx(cd, 0.001f);
          float w = orc_expf(-dd * q->ao_denoise_strength);
          total = total + w;
          load4(ao_raw + 4 * ni, na);
          for (int k = 0; k < 4; ++k) acc[k] = acc[k] + na[k] * w;
        }
      store4(ao + 4 * i, acc[0] / total, acc[1] / total, acc[2] / total, acc[3] / total);
    }
}

void orp_bloom_threshold(const orp_inputs* in, const orp_params* q, uint16_t* out) {
  const int W = in->W, H = in->H, hw = (W + 1) / 2, hh = (H + 1) / 2;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < hh; ++y)
    for (int x = 0; x < hw; ++x) {
      float s[3] = {0.0f, 0.0f, 0.0f};
      for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
          const uint32_t* m = in->material + 4 * ((size_t)clampi(2 * y + dy, 0, H - 1) * W + clampi(2 * x + dx, 0, W - 1));
          s[0] = s[0] + lo(m[1]); s[1] = s[1] + hi(m[1]); s[2] = s[2] + lo(m[2]);
        }
      float ei = q->emissive_intensity;
      f3 e = F3(s[0] * 0.25f * ei, s[1] * 0.25f * ei, s[2] * 0.25f * ei);
      float lum = dot(e, F3(0.2126f, 0.7152f, 0.0722f));
      float knee = q->bloom_threshold * q->bloom_soft_knee;
      float soft = lum - q->bloom_threshold + knee;
      float contrib = fmx(soft, 0.0f) / fmx(knee * 2.0f, 0.0001f);
      float wgt = fmn(contrib * contrib, 1.0f);
      store4(out + 4 * ((size_t)y * hw + x), e.x * wgt, e.y * wgt, e.z * wgt, 1.0f);
    }
}

/* bilinear sample of an rgba16f image (repeat_u: repeat on u, else clamp) */
static void bilin(const uint16_t* img, int w, int h, float u, float v, int repeat_u, float o[4]) {
  float fx = u * (float)w - 0.5f, fy = v * (float)h - 0.5f;
  float x0f = floorf(fx), y0f = floorf(fy);
  float ax = fx - x0f, ay = fy - y0f;
  long long x0 = i32_of(x0f), y0 = i32_of(y0f), x1 = x0 + 1, y1 = y0 + 1;
  if (repeat_u) { x0 = ((x0 % w) + w) % w; x1 = ((x1 % w) + w) % w; }
  else { x0 = x0 < 0 ? 0 : (x0 > w - 1 ? w - 1 : x0); x1 = x1 < 0 ? 0 : (x1 > w - 1 ? w - 1 : x1); }
  y0 = y0 < 0 ? 0 : (y0 > h - 1 ? h - 1 : y0);
  y1 = y1 < 0 ? 0 : (y1 > h - 1 ? h - 1 : y1);
  float t00[4], t10[4], t01[4], t11[4];
  load4(img + 4 * (y0 * w + x0), t00); load4(img + 4 * (y0 * w + x1), t10);
  load4(img + 4 * (y1 * w + x0), t01); load4(img + 4 * (y1 * w + x1), t11);
  float bx = 1.0f - ax, by = 1.0f - ay;
  for (int k = 0; k < 4; ++k) o[k] = (t00[k] * bx + t10[k] * ax) * by + (t01[k] * bx + t11[k] * ax) * ay;
}

static const float BLUR_W[7] = {0.1112202001f, 0.1077983143f, 0.0981514821f, 0.0839534116f,
                                0.0674584614f, 0.0509203181f, 0.0361079124f};

void orp_bloom_blur(int hw, int hh, const uint16_t* src, uint16_t* dst, float dirx, float diry, float tx, float ty) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < hh; ++y)
    for (int x = 0; x < hw; ++x) {
      float u = ((float)x + 0.5f) * tx, v = ((float)y + 0.5f) * ty, c[4], p[4];
      bilin(src, hw, hh, u, v, 0, c);
      float r = c[0] * BLUR_W[0], g = c[1] * BLUR_W[0], b = c[2] * BLUR_W[0];
      for (int i = 1; i < 7; ++i) {
        float ox = dirx * (float)i, oy = diry * (float)i;
        bilin(src, hw, hh, u + ox, v + oy, 0, p);
        r = r + p[0] * BLUR_W[i]; g = g + p[1] * BLUR_W[i]; b = b + p[2] * BLUR_W[i];
        bilin(src, hw, hh, u - ox, v - oy, 0, p);
        r = r + p[0] * BLUR_W[i]; g = g + p[1] * BLUR_W[i]; b = b + p[2] * BLUR_W[i];
      }
      store4(dst + 4 * ((size_t)y * hw + x), r, g, b, 1.0f);
    }
}

#define PI_F 3.14159274101257324219f
#define TWO_PI_F 6.28318548202514648438f

static void env_sample(const orp_env* env, const orp_params* q, f3 dir, float lod, float o[3]) {
  float s, c;
  orp_sincos(q->env_rotation, &s, &c);
  f3 rd = F3(c * dir.x + s * dir.z, dir.y, -s * dir.x + c * dir.z);
  float u = orp_atan2(rd.z, rd.x) / TWO_PI_F + 0.5f;
  float v = 0.5f - orp_asin(clampf(rd.y, -1.0f, 1.0f)) / PI_F;
  float lc = clampf(lod, 0.0f, (float)(env->levels - 1));
  int l0 = i32_of(floorf(lc));
  float f = lc - (float)l0;
  int l1 = l0 + 1 < env->levels ? l0 + 1 : env->levels - 1;
  float s0[4], s1[4];
  bilin(env->texels + 4 * (size_t)env->offset[l0], env->lw[l0], env->lh[l0], u, v, 1, s0);
  bilin(env->texels + 4 * (size_t)env->offset[l1], env->lw[l1], env->lh[l1], u, v, 1, s1);
  float g = 1.0f - f;
  for (int k = 0; k < 3; ++k) o[k] = (s0[k] * g + s1[k] * f) * q->env_intensity;
}

static inline float lut(const uint16_t* curves, int which, float x) {
  return orc_f16_to_f32(curves[which * 256 + clampi(i32_of(x * 255.0f), 0, 255)]);
}
static inline f3 to_lin(f3 c) {
  return F3(orp_weight_pow(fmx(c.x, 0.0f), 2.2f), orp_weight_pow(fmx(c.y, 0.0f), 2.2f), orp_weight_pow(fmx(c.z, 0.0f), 2.2f));
}
static inline f3 to_srgb(f3 c) {
  const float e = 0.454545468091964721680f;
  return F3(orp_weight_pow(fmx(c.x, 0.0f), e), orp_weight_pow(fmx(c.y, 0.0f), e), orp_weight_pow(fmx(c.z, 0.0f), e));
}
static inline f3 reinhard(f3 c, float exposure) {
  f3 e = muls(c, exposure);
  return F3(e.x / (e.x + 1.0f), e.y / (e.y + 1.0f), e.z / (e.z + 1.0f));
}
static inline float g_direct(float ndv, float r) {
  float r1 = r + 1.0f, k = r1 * r1 / 8.0f;
  return ndv / (ndv * (1.0f - k) + k);
}

void orp_lighting(const orp_inputs* in, const orp_params* q, const uint32_t* nrm_img, const uint16_t* ao_img,
                  const orp_env* env, const uint32_t* brdf, const uint16_t* bloom, const uint16_t* curves,
                  uint16_t* lit) {
  const int W = in->W, H = in->H, hw = (W + 1) / 2, hh = (H + 1) / 2;
  const float vw = (float)W, vh = (float)H;
  const int has_env = env->w > 1;
  const f3 lumw = F3(0.2126f, 0.7152f, 0.0722f);
  const float amb_b = (float)((double)q->ambient_intensity * 1.1);
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t i = (size_t)y * W + x;
      uint16_t* o = lit + 4 * i;
      const float* col = in->color + 4 * i;
      f3 alb_s = F3(col[0], col[1], col[2]);
      float depth = in->depth[i];
      if (depth >= 0.9999f || depth <= 0.0001f) {
        if (has_env) {
          float nx = ((float)x + 0.5f) / vw * 2.0f - 1.0f, ny = 1.0f - ((float)y + 0.5f) / vh * 2.0f;
          float wn[4], wf[4], e[3];
          mat4v(q->view_proj_inverse, nx, ny, 0.0f, 1.0f, wn);
          mat4v(q->view_proj_inverse, nx, ny, 1.0f, 1.0f, wf);
          f3 vd = nrm(sub(F3(wf[0] / wf[3], wf[1] / wf[3], wf[2] / wf[3]), F3(wn[0] / wn[3], wn[1] / wn[3], wn[2] / wn[3])));
          env_sample(env, q, vd, 0.0f, e);
          f3 m = to_srgb(reinhard(F3(e[0], e[1], e[2]), q->exposure));
          store4(o, m.x, m.y, m.z, 0.0f);
        } else {
          store4(o, alb_s.x, alb_s.y, alb_s.z, 0.0f);
        }
        continue;
      }
      float alum = dot(alb_s, lumw);
      float remap = lut(curves, 2, alum);
      float ascale = alum < 0.001f ? 1.0f : remap / fmx(alum, 0.001f);
      f3 alb = to_lin(muls(alb_s, ascale));
      f3 V = nrm(sub(F3(q->camera_pos[0], q->camera_pos[1], q->camera_pos[2]),
                     recon(in, q, (float)x + 0.5f, (float)y + 0.5f, depth)));
      f3 N = face_fwd(oct_unpack(nrm_img[i]), V);
      f3 L = nrm(neg(F3(q->light_dir[0], q->light_dir[1], q->light_dir[2])));
      f3 Hh = nrm(add(V, L));
      float NdotL = fmx(dot(N, L), 0.0f), NdotV = fmx(dot(N, V), 0.001f);
      float NdotH = fmx(dot(N, Hh), 0.0f), HdotV = fmx(dot(Hh, V), 0.0f);
      const uint32_t* mat = in->material + 4 * i;
      float rough = fmx(lut(curves, 0, lo(mat[0])), 0.04f);
      float metal = lut(curves, 1, hi(mat[0]));
      f3 F0 = mix3(F3(0.04f, 0.04f, 0.04f), alb, metal);
      float ra = rough * rough, ra2 = ra * ra;
      float dd = NdotH * NdotH * (ra2 - 1.0f) + 1.0f;
      float D = ra2 / (PI_F * dd * dd);
      float G = g_direct(NdotV, rough) * g_direct(NdotL, rough);
      float fp = orp_weight_pow(sat(1.0f - HdotV), 5.0f);
      f3 F = F3(F0.x + (1.0f - F0.x) * fp, F0.y + (1.0f - F0.y) * fp, F0.z + (1.0f - F0.z) * fp);
      float den = 4.0f * NdotV * NdotL + 0.0001f;
      f3 spec = F3(D * G * F.x / den, D * G * F.y / den, D * G * F.z / den);
      float km = 1.0f - metal;
      f3 kD = F3((1.0f - F.x) * km, (1.0f - F.y) * km, (1.0f - F.z) * km);
      float aoS[4], bs[4];
      load4(ao_img + 4 * i, aoS);
      float er = lo(mat[1]), eg = hi(mat[1]), eb = lo(mat[2]);
      float emag = fmx(er, fmx(eg, eb));
      bilin(bloom, hw, hh, ((float)x + 0.5f) / vw, ((float)y + 0.5f) / vh, 1, bs);
      float bmag = dot(F3(bs[0], bs[1], bs[2]), lumw);
      float ao = fmx(aoS[0], fmx(sat(emag * q->emissive_intensity * 0.5f), sat(bmag * 2.0f)));
      const f3 lc = F3(1.0f, 0.949999988079071044922f, 0.899999976158142089844f);
      const float li = q->light_intensity;
      f3 color;
      if (q->specular_only) {
        color = F3(spec.x * lc.x * li * NdotL, spec.y * lc.y * li * NdotL, spec.z * lc.z * li * NdotL);
      } else {
        f3 Lo = F3((kD.x * alb.x / PI_F + spec.x) * lc.x * li * NdotL, (kD.y * alb.y / PI_F + spec.y) * lc.y * li * NdotL,
                   (kD.z * alb.z / PI_F + spec.z) * lc.z * li * NdotL);
        f3 amb;
        if (has_env) {
          f3 dn = nrm(mix3(N, oct_unpack2(aoS[1], aoS[2]), 0.5f));
          float maxLod = orp_log2((float)env->w);
          float irr[3], pref[3];
          env_sample(env, q, dn, fmx(maxLod - 2.0f, 3.0f), irr);
          f3 dI = F3(kD.x * alb.x * irr[0], kD.y * alb.y * irr[1], kD.z * alb.z * irr[2]);
          f3 I = neg(V);
          float dNI = 2.0f * dot(N, I);
          f3 R = F3(I.x - dNI * N.x, I.y - dNI * N.y, I.z - dNI * N.z);
          env_sample(env, q, R, rough * maxLod, pref);
          int bxi = i32_of(clampf(NdotV * 255.0f, 0.0f, 255.0f)), byi = i32_of(clampf(rough * 255.0f, 0.0f, 255.0f));
          uint32_t bw = brdf[byi * 256 + bxi];
          float bA = lo(bw), bB = hi(bw);
          float om = 1.0f - rough, fr = orp_weight_pow(sat(1.0f - NdotV), 5.0f);
          f3 Fi = F3(F0.x + (fmx(om, F0.x) - F0.x) * fr, F0.y + (fmx(om, F0.y) - F0.y) * fr,
                     F0.z + (fmx(om, F0.z) - F0.z) * fr);
          float gz = smoothstep_(0.0f, 0.02f, NdotV);
          f3 sI = F3(pref[0] * (Fi.x * bA + bB) * gz, pref[1] * (Fi.y * bA + bB) * gz, pref[2] * (Fi.z * bA + bB) * gz);
          amb = muls(add(dI, sI), ao);
        } else {
          amb = F3(q->ambient_intensity * alb.x * ao, q->ambient_intensity * alb.y * ao, amb_b * alb.z * ao);
        }
        color = add(amb, Lo);
      }
      f3 m = to_srgb(reinhard(color, q->exposure));
      if (emag > q->emissive_threshold) {
        float ei = q->emissive_intensity;
        m = F3(m.x + er * ei, m.y + eg * ei, m.z + eb * ei);
      }
      store4(o, m.x, m.y, m.z, col[3]);
    }
}

static float radical_inverse(uint32_t b) {
  b = (b << 16u) | (b >> 16u);
  b = ((b & 0x55555555u) << 1u) | ((b & 0xAAAAAAAAu) >> 1u);
  b = ((b & 0x33333333u) << 2u) | ((b & 0xCCCCCCCCu) >> 2u);
  b = ((b & 0x0F0F0F0Fu) << 4u) | ((b & 0xF0F0F0F0u) >> 4u);
  b = ((b & 0x00FF00FFu) << 8u) | ((b & 0xFF00FF00u) >> 8u);
  return (float)b * 2.3283064365386963e-10f;
}
static inline float g_ibl(float ndv, float r) {
  float k = r * r / 2.0f;
  return ndv / (ndv * (1.0f - k) + k);
}

void orp_brdf_lut(int y0, int y1, uint32_t* out) {
  const int size = 256;
#pragma omp parallel for schedule(dynamic, 1)
  for (int y = y0; y < y1; ++y)
    for (int x = 0; x < size; ++x) {
      float NdotV = fmx((float)x / (float)(size - 1), 0.001f), rough = fmx((float)y / (float)(size - 1), 0.001f);
      f3 V = F3(sqrtf(1.0f - NdotV * NdotV), 0.0f, NdotV), N = F3(0.0f, 0.0f, 1.0f);
      float A = 0.0f, B = 0.0f, a = rough * rough;
      f3 up = fabsf(N.z) < 0.999f ? F3(0.0f, 0.0f, 1.0f) : F3(1.0f, 0.0f, 0.0f);
      f3 T = nrm(cross(up, N)), Bt = cross(N, T);
      for (uint32_t i = 0; i < 1024u; ++i) {
        float xi0 = (float)i / 1024.0f, xi1 = radical_inverse(i);
        float phi = TWO_PI_F * xi0;
        float ct = sqrtf((1.0f - xi1) / (1.0f + (a * a - 1.0f) * xi1));
        float st = sqrtf(1.0f - ct * ct);
        float sp, cp;
        orp_sincos(phi, &sp, &cp);
        f3 Hs = F3(cp * st, sp * st, ct);
        f3 H = nrm(F3(T.x * Hs.x + Bt.x * Hs.y + N.x * Hs.z, T.y * Hs.x + Bt.y * Hs.y + N.y * Hs.z,
                      T.z * Hs.x + Bt.z * Hs.y + N.z * Hs.z));
        float vh2 = 2.0f * dot(V, H);
        f3 L = nrm(F3(vh2 * H.x - V.x, vh2 * H.y - V.y, vh2 * H.z - V.z));
        float NdotL = fmx(L.z, 0.0f), NdotH = fmx(H.z, 0.0f), VdotH = fmx(dot(V, H), 0.0f);
        if (NdotL > 0.0f) {
          float G = g_ibl(fmx(dot(N, V), 0.0f), rough) * g_ibl(fmx(dot(N, L), 0.0f), rough);
          float gv = G * VdotH / (NdotH * NdotV);
          float Fc = orp_pow(1.0f - VdotH, 5.0f);
          A = A + (1.0f - Fc) * gv;
          B = B + Fc * gv;
        }
      }
      out[y * size + x] = pk(A / 1024.0f, B / 1024.0f);
    }
}

void orp_env_mip(const uint16_t* src, int sw, int sh, uint16_t* dst, int dw, int dh) {
  for (int y = 0; y < dh; ++y)
    for (int x = 0; x < dw; ++x) {
      float a[4], b[4], c[4], d[4];
      int x0 = clampi(2 * x, 0, sw - 1), x1 = clampi(2 * x + 1, 0, sw - 1);
      int yy0 = clampi(2 * y, 0, sh - 1), yy1 = clampi(2 * y + 1, 0, sh - 1);
      load4(src + 4 * (yy0 * sw + x0), a); load4(src + 4 * (yy0 * sw + x1), b);
      load4(src + 4 * (yy1 * sw + x0), c); load4(src + 4 * (yy1 * sw + x1), d);
      store4(dst + 4 * (y * dw + x), (a[0] + b[0] + c[0] + d[0]) * 0.25f, (a[1] + b[1] + c[1] + d[1]) * 0.25f,
             (a[2] + b[2] + c[2] + d[2]) * 0.25f, (a[3] + b[3] + c[3] + d[3]) * 0.25f);
    }
}

void orp_curve_lut(float contrast, float brightness, float gamma, uint16_t out[256]) {
  for (int i = 0; i < 256; ++i) {
    double v = (double)i / 255.0;
    v = (v - 0.5) * (double)contrast + 0.5;
    v += (double)brightness;
    v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
    v = pow(v, (double)gamma);
    v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
    out[i] = orc_f32_to_f16_trunc((float)v);
  }
}
