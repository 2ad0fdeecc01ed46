// hdsr_post.cu — the deferred frame tail over the compositor's G-buffer.
//
// Restates, as CUDA kernels over headless device images:
//   k_ss_normals      gpu_screen_space_normals.wgsl:55-119 (params from
//                     splatRenderer.ts:350-365)
//   k_bilateral       bilateral_normal_filter.wgsl:39-86 (params :414-420),
//                     the decoded normals and depths of a 16x16 tile plus its
//                     halo staged once in shared memory
//   k_gtao_prefilter  gtao_depth_prefilter.wgsl:27-72 (16x16 blocks: the
//                     2x2 and 4x4 min levels come from the block's own tile)
//   k_gtao_main       gtao_main.wgsl:109-222
//   k_gtao_denoise    gtao_denoise.wgsl:17-95 (edge clamping of the halo is
//                     the shared-memory tile's clamped loads)
//   k_bloom_threshold bloom_threshold.wgsl:16-42
//   k_bloom_blur      bloom_blur.wgsl:19-37, run horizontally then vertically
//   k_lighting        gpu_deferred_lighting.wgsl:123-269
//   k_brdf_lut        ibl_brdf_lut.wgsl:58-97 (at create)
//   k_env_mip         ibl_mipgen.wgsl:7-19 (at set_environment)
// Texture reads of the reference become explicit loads: textureLoad outside
// the image clamps to the edge (Tint's robustness transform); a filtering
// sampler becomes bilinear (and, for the environment, trilinear) weights in
// f32: t = t00*(1-a) + t10*a per row, then rows by (1-b), b; repeat or
// clamp-to-edge addressing as the reference's GPUSampler says.
// rgba16float images are uint2 (two pack2x16float words) stored with
// round-to-nearest-even.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "../../include/hdsr.h"
#include "hdsr_post_math.cuh"

using namespace hdsr;

namespace {

constexpr int kBrdfSize = 256;
constexpr int kMaxEnvLevels = 16;
constexpr int kPasses = 7;

struct PostArgs {
  int W, H, hw, hh, m1w, m1h, m2w, m2h;
  const unsigned char* color; uint64_t color_pitch; int color_f32;
  const unsigned char* depth; uint64_t depth_pitch;
  const unsigned char* src_normal; uint64_t normal_pitch;
  const unsigned char* material; uint64_t material_pitch;
  uint32_t* ssn; uint32_t* nrm;
  float* mip0; float* mip1; float* mip2;
  uint2* ao_raw; uint2* ao;
  uint2* bloom_a; uint2* bloom_b;
  const uint32_t* brdf;
  const uint2* env; int env_w, env_h, env_levels;
  int env_lw[kMaxEnvLevels], env_lh[kMaxEnvLevels];
  uint32_t env_off[kMaxEnvLevels];
  const uint16_t* curves;
  unsigned char* lit; uint64_t lit_pitch;
  float vw, vh;                 // viewport as f32
  float blur_dir_h, blur_dir_v, texel_x, texel_y;  // f32(1/hw), f32(1/hh)
  float ambient_b;              // f32(ambientIntensity * 1.1)
  hdsr_post_params p;
};

__device__ __forceinline__ float ld_depth(const PostArgs& a, int x, int y) {
  return *reinterpret_cast<const float*>(a.depth + (uint64_t)y * a.depth_pitch + (uint64_t)x * 4u);
}
__device__ __forceinline__ uint32_t ld_src_normal(const PostArgs& a, int x, int y) {
  return *reinterpret_cast<const uint32_t*>(a.src_normal + (uint64_t)y * a.normal_pitch + (uint64_t)x * 4u);
}
__device__ __forceinline__ uint4 ld_material(const PostArgs& a, int x, int y) {
  return *reinterpret_cast<const uint4*>(a.material + (uint64_t)y * a.material_pitch + (uint64_t)x * 16u);
}
__device__ __forceinline__ float4 ld_color(const PostArgs& a, int x, int y) {
  const unsigned char* row = a.color + (uint64_t)y * a.color_pitch;
  if (a.color_f32) return reinterpret_cast<const float4*>(row)[x];
  uint2 t = reinterpret_cast<const uint2*>(row)[x];
  return make_float4(lo16(t.x), hi16(t.x), lo16(t.y), hi16(t.y));
}
__device__ __forceinline__ float4 h4(uint2 t) { return make_float4(lo16(t.x), hi16(t.x), lo16(t.y), hi16(t.y)); }
__device__ __forceinline__ uint2 pack_h4(float r, float g, float b, float w) {
  return make_uint2(pack2x16(r, g), pack2x16(b, w));
}

// reconstructViewPos / reconstructWorldPos: pixel centre + NDC depth through viewProjInv
__device__ __forceinline__ F3 recon(const PostArgs& a, float px, float py, float d) {
  float nx = px / a.vw * 2.0f - 1.0f;
  float ny = 1.0f - py / a.vh * 2.0f;
  float w[4];
  mat4_mul(a.p.view_proj_inverse, nx, ny, d, 1.0f, w);
  return f3(w[0] / w[3], w[1] / w[3], w[2] / w[3]);
}

// ---------------------------------------------------------------------------
// screen-space normals
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_ss_normals(PostArgs a) {
  int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= a.W || y >= a.H) return;
  float mode = (float)a.p.normal_recovery_mode;
  float d = ld_depth(a, x, y);
  uint32_t* out = a.ssn + (uint64_t)y * a.W + x;
  if (d >= 0.9999f) {
    *out = mode > 0.5f ? ld_src_normal(a, x, y) : pack2x16(0.0f, 0.0f);
    return;
  }
  float cx = (float)x + 0.5f, cy = (float)y + 0.5f;
  F3 posC = recon(a, cx, cy, d);
  float dL = ld_depth(a, x > 0 ? x - 1 : 0, y);
  float dR = ld_depth(a, x + 1 < a.W ? x + 1 : a.W - 1, y);
  float dU = ld_depth(a, x, y > 0 ? y - 1 : 0);
  float dD = ld_depth(a, x, y + 1 < a.H ? y + 1 : a.H - 1);
  F3 ddx, ddy;
  if (fabsf(dL - d) < fabsf(dR - d)) ddx = sub(posC, recon(a, cx - 1.0f, cy - 0.0f, dL));
  else ddx = sub(recon(a, cx + 1.0f, cy + 0.0f, dR), posC);
  if (fabsf(dU - d) < fabsf(dD - d)) ddy = sub(posC, recon(a, cx - 0.0f, cy - 1.0f, dU));
  else ddy = sub(recon(a, cx + 0.0f, cy + 1.0f, dD), posC);
  F3 cam = f3(a.p.camera_pos[0], a.p.camera_pos[1], a.p.camera_pos[2]);
  F3 viewDir = normalize(sub(cam, posC));
  F3 screenN = face_forward(normalize(cross(ddy, ddx)), viewDir);
  F3 srcN = face_forward(oct_dec_word(ld_src_normal(a, x, y)), viewDir);
  F3 n = screenN;
  if (mode > 1.5f) {
    n = srcN;
  } else if (mode > 0.5f) {
    float ndv = mx(dot(srcN, viewDir), 0.0f);
    float blend = 1.0f - smoothstepf(a.p.grazing_start, a.p.grazing_end, ndv);
    n = normalize(mix3(srcN, screenN, blend));
  }
  *out = oct_word(n);
}

// ---------------------------------------------------------------------------
// bilateral normal filter
// ---------------------------------------------------------------------------
// The two divisions of a tap by per-pixel constants (the centre's depth and
// 2 sigma^2) are multiplications by their reciprocals, taken once per pixel
// (within the 2.5 ulp WGSL allows a division; the oracle does the same).
__device__ __forceinline__ void bilateral_tap(float4 c, F3 cn, float inv_dden, float neg_inv_sd2, float ne,
                                              float spatialW, float4 s, F3& acc, float& total) {
  F3 sn = f3(s.x, s.y, s.z);
  float depthDiff = fabsf(c.w - s.w) * inv_dden;
  float depthW = weight_expf((depthDiff * depthDiff) * neg_inv_sd2);
  float normalW = weight_pow(mx(dot(cn, sn), 0.0f), ne);
  float w = spatialW * depthW * normalW;
  acc = add(acc, muls(sn, w));
  total = total + w;
}

template <int RC>
__global__ void __launch_bounds__(256) k_bilateral(PostArgs a) {
  extern __shared__ float4 s_nd[];           // (16+2R)^2 decoded normal + depth
  __shared__ float s_spatial[17 * 17];
  const int R = RC > 0 ? RC : (int)a.p.bilateral_radius;
  const int T = 16 + 2 * R;
  const int tid = threadIdx.y * 16 + threadIdx.x;
  const int bx = blockIdx.x * 16, by = blockIdx.y * 16;
  for (int i = tid; i < T * T; i += 256) {
    int gx = clampi(bx + i % T - R, 0, a.W - 1), gy = clampi(by + i / T - R, 0, a.H - 1);
    F3 n = oct_dec_word(a.ssn[(uint64_t)gy * a.W + gx]);
    s_nd[i] = make_float4(n.x, n.y, n.z, ld_depth(a, gx, gy));
  }
  const float ss = a.p.bilateral_spatial_sigma;
  for (int i = tid; i < (2 * R + 1) * (2 * R + 1); i += 256) {
    int dx = i % (2 * R + 1) - R, dy = i / (2 * R + 1) - R;
    float dist2 = (float)(dx * dx + dy * dy);
    s_spatial[i] = hx_expf(-dist2 / (2.0f * ss * ss));
  }
  __syncthreads();
  int x = bx + threadIdx.x, y = by + threadIdx.y;
  if (x >= a.W || y >= a.H) return;
  uint64_t idx = (uint64_t)y * a.W + x;
  float4 c = s_nd[(threadIdx.y + R) * T + threadIdx.x + R];
  if (c.w >= 0.9999f) { a.nrm[idx] = a.ssn[idx]; return; }
  F3 cn = f3(c.x, c.y, c.z);
  const float sd2 = 2.0f * a.p.bilateral_depth_sigma * a.p.bilateral_depth_sigma;
  const float ne = 1.0f / mx(a.p.bilateral_normal_sigma, 0.01f);
  const float inv_dden = 1.0f / mx(c.w, 0.001f);
  const float neg_inv_sd2 = -(1.0f / sd2);
  F3 acc = f3(0.0f, 0.0f, 0.0f);
  float total = 0.0f;
#pragma unroll 1
  for (int dy = -R; dy <= R; ++dy) {
    const float4* row = s_nd + (threadIdx.y + R + dy) * T + threadIdx.x + R;
#pragma unroll
    for (int dx = -R; dx <= R; ++dx)
      bilateral_tap(c, cn, inv_dden, neg_inv_sd2, ne, s_spatial[(dy + R) * (2 * R + 1) + dx + R], row[dx], acc, total);
  }
  a.nrm[idx] = oct_word(normalize(divs(acc, mx(total, 0.0001f))));
}

// ---------------------------------------------------------------------------
// GTAO
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gtao_prefilter(PostArgs a) {
  __shared__ float s[256];
  const int lx = threadIdx.x, ly = threadIdx.y;
  const int x = blockIdx.x * 16 + lx, y = blockIdx.y * 16 + ly;
  const bool in = x < a.W && y < a.H;
  const float nearp = a.p.near_plane, farp = a.p.far_plane;
  float raw = ld_depth(a, clampi(x, 0, a.W - 1), clampi(y, 0, a.H - 1));
  float lin = nearp * farp / (farp - raw * (farp - nearp));
  if (in) a.mip0[(uint64_t)y * a.W + x] = lin;
  const int li = ly * 16 + lx;
  s[li] = lin;
  __syncthreads();
  if ((lx & 1) == 0 && (ly & 1) == 0) {
    float v = mn(mn(s[li], s[li + 1]), mn(s[li + 16], s[li + 17]));
    if (in) a.mip1[(uint64_t)(y >> 1) * a.m1w + (x >> 1)] = v;
    s[li] = v;
  }
  __syncthreads();
  if ((lx & 3) == 0 && (ly & 3) == 0) {
    float v = mn(mn(s[li], s[li + 2]), mn(s[li + 32], s[li + 34]));
    if (in) a.mip2[(uint64_t)(y >> 2) * a.m2w + (x >> 2)] = v;
  }
}

__device__ __forceinline__ uint32_t hilbert16(uint32_t x, uint32_t y) {
  uint32_t d = 0u, s = 8u;
  for (;;) {
    if (s == 0u) break;
    s >>= 1;
    uint32_t rx = (x & s) > 0u ? 1u : 0u;
    uint32_t ry = (y & s) > 0u ? 1u : 0u;
    d += s * s * ((3u * rx) ^ ry);
    if (ry == 0u) {
      if (rx == 1u) { x = s * 2u - 1u - x; y = s * 2u - 1u - y; }
      uint32_t t = x; x = y; y = t;
    }
  }
  return d;
}

__device__ __forceinline__ float sample_depth_mip(const PostArgs& a, float u, float v, int level) {
  const float* m = level == 0 ? a.mip0 : (level == 1 ? a.mip1 : a.mip2);
  int w = level == 0 ? a.W : (level == 1 ? a.m1w : a.m2w);
  int h = level == 0 ? a.H : (level == 1 ? a.m1h : a.m2h);
  int cx = clampi(to_i32(u * (float)w), 0, w - 1);
  int cy = clampi(to_i32(v * (float)h), 0, h - 1);
  return m[(uint64_t)cy * w + cx];
}

__device__ __forceinline__ F3 view_pos(const PostArgs& a, const float pi[4], float u, float v, float depth) {
  return f3((u * pi[0] + pi[2]) * depth, (v * pi[1] + pi[3]) * depth, -depth);
}

// Divisions by frame constants (thickness, falloff end, viewport size) are
// multiplications by reciprocals taken once (within the 2.5 ulp WGSL allows a
// division; the oracle does the same); dot / dist stays a division.
__device__ __forceinline__ void horizon_sample(const PostArgs& a, const float pi[4], float u, float v, int mip,
                                               F3 viewPos, F3 vn, float inv_thick, float inv_falloff, float& best) {
  if (u >= 0.0f && u <= 1.0f && v >= 0.0f && v <= 1.0f) {
    float sd = sample_depth_mip(a, u, v, mip);
    F3 diff = sub(view_pos(a, pi, u, v, sd), viewPos);
    float dist = length(diff);
    if (dist > 0.001f) {
      float zr = fabsf(diff.z) * inv_thick;
      float tw = sat(1.0f - zr * zr);
      float hz = dot(diff, vn) / dist;
      float fo = sat(1.0f - dist * inv_falloff);
      best = mx(best, hz * fo * tw);
    }
  }
}

// TC > 0: the step count known at compile time (t and the mip level of each
// step do not depend on the slice, so they are computed once per pixel).
template <int TC>
__global__ void __launch_bounds__(256) k_gtao_main(PostArgs a, float4 projInfo) {
  int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= a.W || y >= a.H) return;
  const float pi[4] = {projInfo.x, projInfo.y, projInfo.z, projInfo.w};
  uint64_t idx = (uint64_t)y * a.W + x;
  float u = ((float)x + 0.5f) / a.vw, v = ((float)y + 0.5f) / a.vh;
  float cd = a.mip0[idx];
  if (cd <= 0.0f || cd > a.p.ao_falloff_end * 10.0f) { a.ao_raw[idx] = pack_h4(1.0f, 0.0f, 1.0f, 0.0f); return; }
  F3 viewPos = view_pos(a, pi, u, v, cd);
  F3 wn = oct_dec_word(a.nrm[idx]);
  float t4[4];
  mat4_mul(a.p.view, wn.x, wn.y, wn.z, 0.0f, t4);
  F3 vnr = normalize(f3(t4[0], t4[1], t4[2]));
  F3 vn = face_forward(vnr, normalize(neg(viewPos)));
  float focalPx = a.vw / fabsf(pi[0]);
  float pixelRadius = mx(a.p.ao_radius_world * focalPx / cd, 1.0f);
  uint32_t hil = hilbert16((uint32_t)x & 15u, (uint32_t)y & 15u);
  uint32_t idxr = hil + a.p.frame_counter * 256u;
  const float a1 = 0.754877686500549316406f;   // f32(1 / 1.3247179572)
  const float a2 = a1 * a1;
  float sox = fractf((float)idxr * a1 + 0.5f), soy = fractf((float)idxr * a2 + 0.5f);
  const uint32_t S = a.p.ao_slices, T = TC > 0 ? (uint32_t)TC : a.p.ao_steps;
  float tt[TC > 0 ? TC : 1];
  int tm[TC > 0 ? TC : 1];
  if (TC > 0) {
#pragma unroll
    for (int st = 1; st <= (TC > 0 ? TC : 1); ++st) {
      float t = ((float)st + soy * 0.5f) / (float)T;
      tt[st - 1] = t;
      tm[st - 1] = to_i32(clampf(px_log2(pixelRadius * t / 4.0f), 0.0f, 2.0f));
    }
  }
  const float inv_vw = 1.0f / a.vw, inv_vh = 1.0f / a.vh;
  const float inv_thick = 1.0f / a.p.ao_thickness, inv_falloff = 1.0f / a.p.ao_falloff_end;
  float totalAO = 0.0f;
  F3 bent = f3(0.0f, 0.0f, 0.0f);
  for (uint32_t sl = 0; sl < S; ++sl) {
    float phi = (3.14159274101257324219f / (float)S) * ((float)sl + sox);
    float ds, dc;
    px_sincos(phi, &ds, &dc);
    const float dcp = dc * pixelRadius, dsp = ds * pixelRadius;
    float bestP = -1.0f, bestN = -1.0f;
    if (TC > 0) {
#pragma unroll
      for (int k = 0; k < (TC > 0 ? TC : 1); ++k) {
        float ox = dcp * tt[k] * inv_vw, oy = dsp * tt[k] * inv_vh;
        horizon_sample(a, pi, u + ox, v + oy, tm[k], viewPos, vn, inv_thick, inv_falloff, bestP);
        horizon_sample(a, pi, u - ox, v - oy, tm[k], viewPos, vn, inv_thick, inv_falloff, bestN);
      }
    } else {
      for (uint32_t st = 1; st <= T; ++st) {
        float t = ((float)st + soy * 0.5f) / (float)T;
        float ox = dcp * t * inv_vw, oy = dsp * t * inv_vh;
        int mip = to_i32(clampf(px_log2(pixelRadius * t / 4.0f), 0.0f, 2.0f));
        horizon_sample(a, pi, u + ox, v + oy, mip, viewPos, vn, inv_thick, inv_falloff, bestP);
        horizon_sample(a, pi, u - ox, v - oy, mip, viewPos, vn, inv_thick, inv_falloff, bestN);
      }
    }
    float nds = vn.x * dc + vn.y * ds + vn.z * 0.0f;
    float cP = mx(bestP, nds * 0.08f), cN = mx(bestN, -nds * 0.08f);
    totalAO = totalAO + (cP + cN);
    float vP = 1.0f - cP, vN = 1.0f - cN;
    F3 sdir = f3(dc, ds, 0.0f);
    bent = add(bent, add(muls(sdir, vP - vN), muls(vn, vP + vN)));
  }
  totalAO = totalAO / ((float)S * 2.0f);
  float ao = sat(1.0f - totalAO * a.p.ao_intensity);
  float bl = length(bent);
  F3 bvs = bl > 0.001f ? divs(bent, bl) : vn;
  const float* m = a.p.view;
  // viewMatrix is orthonormal: world = transpose(view3x3) * bent, row r = (m[r], m[4+r], m[8+r])
  F3 bw = normalize(f3(dot(f3(m[0], m[4], m[8]), bvs), dot(f3(m[1], m[5], m[9]), bvs),
                       dot(f3(m[2], m[6], m[10]), bvs)));
  float bx, by;
  oct_enc(bw, &bx, &by);
  a.ao_raw[idx] = pack_h4(ao, bx, by, 0.0f);
}

__global__ void __launch_bounds__(256) k_gtao_denoise(PostArgs a) {
  int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= a.W || y >= a.H) return;
  uint64_t idx = (uint64_t)y * a.W + x;
  float cd = a.mip0[idx];
  float4 acc = h4(a.ao_raw[idx]);
  float total = 1.0f;
  const float den = mx(cd, 0.001f);
  for (int dy = -1; dy <= 1; ++dy) {
    for (int dx = -1; dx <= 1; ++dx) {
      if (dx == 0 && dy == 0) continue;
      int nx = clampi(x + dx, 0, a.W - 1), ny = clampi(y + dy, 0, a.H - 1);
      uint64_t ni = (uint64_t)ny * a.W + nx;
      float dd = fabsf(cd - a.mip0[ni]) / den;
      float w = hx_expf(-dd * a.p.ao_denoise_strength);
      total = total + w;
      float4 na = h4(a.ao_raw[ni]);
      acc.x = acc.x + na.x * w; acc.y = acc.y + na.y * w;
      acc.z = acc.z + na.z * w; acc.w = acc.w + na.w * w;
    }
  }
  a.ao[idx] = pack_h4(acc.x / total, acc.y / total, acc.z / total, acc.w / total);
}

// ---------------------------------------------------------------------------
// bloom
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bloom_threshold(PostArgs a) {
  int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= a.hw || y >= a.hh) return;
  float er = 0.0f, eg = 0.0f, eb = 0.0f;
  for (int dy = 0; dy < 2; ++dy)
    for (int dx = 0; dx < 2; ++dx) {
      uint4 m = ld_material(a, clampi(2 * x + dx, 0, a.W - 1), clampi(2 * y + dy, 0, a.H - 1));
      er = er + lo16(m.y); eg = eg + hi16(m.y); eb = eb + lo16(m.z);
    }
  const float ei = a.p.emissive_intensity;
  F3 em = f3(er * 0.25f * ei, eg * 0.25f * ei, eb * 0.25f * ei);
  float lum = dot(em, f3(0.2126f, 0.7152f, 0.0722f));
  float knee = a.p.bloom_threshold * a.p.bloom_soft_knee;
  float soft = lum - a.p.bloom_threshold + knee;
  float contrib = mx(soft, 0.0f) / mx(knee * 2.0f, 0.0001f);
  float weight = mn(contrib * contrib, 1.0f);
  a.bloom_a[(uint64_t)y * a.hw + x] = pack_h4(em.x * weight, em.y * weight, em.z * weight, 1.0f);
}

// bilinear sample of an rgba16f image; repeat_u selects repeat on u, else clamp-to-edge.
// The corner indices equal floor(coordinate) (+1) wrapped or clamped; the
// float is bounded first so the integer arithmetic cannot overflow (a bound
// only moves indices that clamp to the same edge, or, for repeat, lie beyond
// 2^24 texels, where the weights are NaN or the coordinate is not finite).
__device__ __forceinline__ int wrap_index(int i, int w) {
  if ((unsigned)i < (unsigned)w) return i;
  int r = i % w;
  return r < 0 ? r + w : r;
}
__device__ __forceinline__ float4 bilinear(const uint2* img, int w, int h, float u, float v, bool repeat_u) {
  float fx = u * (float)w - 0.5f, fy = v * (float)h - 0.5f;
  float x0f = floorf(fx), y0f = floorf(fy);
  float ax = fx - x0f, ay = fy - y0f;
  int x0, x1;
  if (repeat_u) {
    x0 = to_i32(clampf(x0f, -16777216.0f, 16777216.0f));
    if (!(x0f == x0f)) x0 = 0;
    x1 = wrap_index(x0 + 1, w);
    x0 = wrap_index(x0, w);
  } else {
    x0 = to_i32(clampf(x0f, -1.0f, (float)w));
    x1 = clampi(x0 + 1, 0, w - 1);
    x0 = clampi(x0, 0, w - 1);
  }
  int y0 = to_i32(clampf(y0f, -1.0f, (float)h));
  int y1 = clampi(y0 + 1, 0, h - 1);
  y0 = clampi(y0, 0, h - 1);
  float4 t00 = h4(img[y0 * w + x0]), t10 = h4(img[y0 * w + x1]);
  float4 t01 = h4(img[y1 * w + x0]), t11 = h4(img[y1 * w + x1]);
  float bx = 1.0f - ax, by = 1.0f - ay;
  float4 r;
  r.x = (t00.x * bx + t10.x * ax) * by + (t01.x * bx + t11.x * ax) * ay;
  r.y = (t00.y * bx + t10.y * ax) * by + (t01.y * bx + t11.y * ax) * ay;
  r.z = (t00.z * bx + t10.z * ax) * by + (t01.z * bx + t11.z * ax) * ay;
  r.w = (t00.w * bx + t10.w * ax) * by + (t01.w * bx + t11.w * ax) * ay;
  return r;
}

__constant__ float c_blur_w[7] = {0.1112202001f, 0.1077983143f, 0.0981514821f, 0.0839534116f,
                                  0.0674584614f, 0.0509203181f, 0.0361079124f};

__global__ void __launch_bounds__(256) k_bloom_blur(PostArgs a, const uint2* src, uint2* dst, float dirx,
                                                    float diry) {
  int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= a.hw || y >= a.hh) return;
  float u = ((float)x + 0.5f) * a.texel_x, v = ((float)y + 0.5f) * a.texel_y;
  float4 c = bilinear(src, a.hw, a.hh, u, v, false);
  float rr = c.x * c_blur_w[0], rg = c.y * c_blur_w[0], rb = c.z * c_blur_w[0];
  for (int i = 1; i < 7; ++i) {
    float ox = dirx * (float)i, oy = diry * (float)i;
    float4 p = bilinear(src, a.hw, a.hh, u + ox, v + oy, false);
    rr = rr + p.x * c_blur_w[i]; rg = rg + p.y * c_blur_w[i]; rb = rb + p.z * c_blur_w[i];
    float4 q = bilinear(src, a.hw, a.hh, u - ox, v - oy, false);
    rr = rr + q.x * c_blur_w[i]; rg = rg + q.y * c_blur_w[i]; rb = rb + q.z * c_blur_w[i];
  }
  dst[(uint64_t)y * a.hw + x] = pack_h4(rr, rg, rb, 1.0f);
}

// ---------------------------------------------------------------------------
// deferred lighting
// ---------------------------------------------------------------------------
constexpr float kPI = 3.14159274101257324219f;      // f32(3.14159265359)
constexpr float kTwoPI = 6.28318548202514648438f;   // f32(2 * 3.14159265359)

__device__ __forceinline__ float4 sample_env(const PostArgs& a, float s, float c, F3 dir, float lod) {
  F3 rd = f3(c * dir.x + s * dir.z, dir.y, -s * dir.x + c * dir.z);
  float u = px_atan2(rd.z, rd.x) / kTwoPI + 0.5f;
  float v = 0.5f - px_asin(clampf(rd.y, -1.0f, 1.0f)) / kPI;
  float lc = clampf(lod, 0.0f, (float)(a.env_levels - 1));
  int l0 = to_i32(floorf(lc));
  float f = lc - (float)l0;
  int l1 = l0 + 1 < a.env_levels ? l0 + 1 : a.env_levels - 1;
  float4 s0 = bilinear(a.env + a.env_off[l0], a.env_lw[l0], a.env_lh[l0], u, v, true);
  float4 s1 = bilinear(a.env + a.env_off[l1], a.env_lw[l1], a.env_lh[l1], u, v, true);
  float g = 1.0f - f;
  float ei = a.p.env_intensity;
  return make_float4((s0.x * g + s1.x * f) * ei, (s0.y * g + s1.y * f) * ei, (s0.z * g + s1.z * f) * ei, 0.0f);
}

__device__ __forceinline__ float curve(const PostArgs& a, int lut, float x) {
  int i = clampi(to_i32(x * 255.0f), 0, 255);
  return f16_to_f32(a.curves[lut * 256 + i]);
}

__device__ __forceinline__ F3 srgb_to_linear(F3 c) {
  return f3(weight_pow(mx(c.x, 0.0f), 2.2f), weight_pow(mx(c.y, 0.0f), 2.2f), weight_pow(mx(c.z, 0.0f), 2.2f));
}
__device__ __forceinline__ F3 linear_to_srgb(F3 c) {
  const float e = 0.454545468091964721680f;   // f32(1 / 2.2)
  return f3(weight_pow(mx(c.x, 0.0f), e), weight_pow(mx(c.y, 0.0f), e), weight_pow(mx(c.z, 0.0f), e));
}
__device__ __forceinline__ F3 tonemap(F3 c, float exposure) {
  F3 e = muls(c, exposure);
  return f3(e.x / (e.x + 1.0f), e.y / (e.y + 1.0f), e.z / (e.z + 1.0f));
}
__device__ __forceinline__ float geom_direct(float ndv, float r) {
  float r1 = r + 1.0f;
  float k = r1 * r1 / 8.0f;
  return ndv / (ndv * (1.0f - k) + k);
}

__global__ void __launch_bounds__(256) k_lighting(PostArgs a) {
  // the environment's rotation (sin, cos) and its top mip level are the same
  // for every pixel: computed once per block (same functions, same bits)
  __shared__ float s_env[3];
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    px_sincos(a.p.env_rotation, &s_env[0], &s_env[1]);
    s_env[2] = px_log2((float)a.env_w);
  }
  __syncthreads();
  int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= a.W || y >= a.H) return;
  uint64_t idx = (uint64_t)y * a.W + x;
  uint2* out = reinterpret_cast<uint2*>(a.lit + (uint64_t)y * a.lit_pitch) + x;
  float4 col = ld_color(a, x, y);
  F3 albedoSrgb = f3(col.x, col.y, col.z);
  float depth = ld_depth(a, x, y);
  const bool hasEnv = a.env_w > 1;
  if (depth >= 0.9999f || depth <= 0.0001f) {
    if (hasEnv) {
      float nx = ((float)x + 0.5f) / a.vw * 2.0f - 1.0f;
      float ny = 1.0f - ((float)y + 0.5f) / a.vh * 2.0f;
      float wn[4], wf[4];
      mat4_mul(a.p.view_proj_inverse, nx, ny, 0.0f, 1.0f, wn);
      mat4_mul(a.p.view_proj_inverse, nx, ny, 1.0f, 1.0f, wf);
      F3 vd = normalize(sub(f3(wf[0] / wf[3], wf[1] / wf[3], wf[2] / wf[3]),
                            f3(wn[0] / wn[3], wn[1] / wn[3], wn[2] / wn[3])));
      const float rs = s_env[0], rc = s_env[1];
      float4 e = sample_env(a, rs, rc, vd, 0.0f);
      F3 m = linear_to_srgb(tonemap(f3(e.x, e.y, e.z), a.p.exposure));
      *out = pack_h4(m.x, m.y, m.z, 0.0f);
    } else {
      *out = pack_h4(albedoSrgb.x, albedoSrgb.y, albedoSrgb.z, 0.0f);
    }
    return;
  }
  const F3 lumw = f3(0.2126f, 0.7152f, 0.0722f);
  float albedoLum = dot(albedoSrgb, lumw);
  float remapped = curve(a, 2, albedoLum);
  float albedoScale = albedoLum < 0.001f ? 1.0f : remapped / mx(albedoLum, 0.001f);
  F3 albedo = srgb_to_linear(muls(albedoSrgb, albedoScale));

  F3 Nraw = oct_dec_word(a.nrm[idx]);
  F3 worldPos = recon(a, (float)x + 0.5f, (float)y + 0.5f, depth);
  F3 V = normalize(sub(f3(a.p.camera_pos[0], a.p.camera_pos[1], a.p.camera_pos[2]), worldPos));
  F3 N = face_forward(Nraw, V);
  F3 L = normalize(neg(f3(a.p.light_dir[0], a.p.light_dir[1], a.p.light_dir[2])));
  F3 Hh = normalize(add(V, L));
  float NdotL = mx(dot(N, L), 0.0f);
  float NdotV = mx(dot(N, V), 0.001f);
  float NdotH = mx(dot(N, Hh), 0.0f);
  float HdotV = mx(dot(Hh, V), 0.0f);

  uint4 mat = ld_material(a, x, y);
  float roughness = mx(curve(a, 0, lo16(mat.x)), 0.04f);
  float metallic = curve(a, 1, hi16(mat.x));
  F3 F0 = mix3(f3(0.04f, 0.04f, 0.04f), albedo, metallic);

  float ra = roughness * roughness;
  float ra2 = ra * ra;
  float dd = NdotH * NdotH * (ra2 - 1.0f) + 1.0f;
  float D = ra2 / (kPI * dd * dd);
  float G = geom_direct(NdotV, roughness) * geom_direct(NdotL, roughness);
  float fp = weight_pow(sat(1.0f - HdotV), 5.0f);
  F3 F = f3(F0.x + (1.0f - F0.x) * fp, F0.y + (1.0f - F0.y) * fp, F0.z + (1.0f - F0.z) * fp);
  float den = 4.0f * NdotV * NdotL + 0.0001f;
  F3 spec = f3(D * G * F.x / den, D * G * F.y / den, D * G * F.z / den);
  float km = 1.0f - metallic;
  F3 kD = f3((1.0f - F.x) * km, (1.0f - F.y) * km, (1.0f - F.z) * km);

  float4 aoS = h4(a.ao[idx]);
  float emr = lo16(mat.y), emg = hi16(mat.y), emb = lo16(mat.z);
  float emag = mx(emr, mx(emg, emb));
  float bu = ((float)x + 0.5f) / a.vw, bv = ((float)y + 0.5f) / a.vh;
  float4 bs = bilinear(a.bloom_a, a.hw, a.hh, bu, bv, true);
  float bloomMag = dot(f3(bs.x, bs.y, bs.z), lumw);
  float eLift = sat(emag * a.p.emissive_intensity * 0.5f);
  float bLift = sat(bloomMag * 2.0f);
  float ao = mx(aoS.x, mx(eLift, bLift));

  const F3 lc = f3(1.0f, 0.949999988079071044922f, 0.899999976158142089844f);
  const float li = a.p.light_intensity;
  F3 color;
  if (a.p.specular_only != 0u) {
    color = f3(spec.x * lc.x * li * NdotL, spec.y * lc.y * li * NdotL, spec.z * lc.z * li * NdotL);
  } else {
    F3 Lo = f3((kD.x * albedo.x / kPI + spec.x) * lc.x * li * NdotL, (kD.y * albedo.y / kPI + spec.y) * lc.y * li * NdotL,
               (kD.z * albedo.z / kPI + spec.z) * lc.z * li * NdotL);
    F3 ambient;
    if (hasEnv) {
      F3 bentN = oct_dec(aoS.y, aoS.z);
      F3 diffDir = normalize(mix3(N, bentN, 0.5f));
      const float maxLod = s_env[2];
      float diffLod = mx(maxLod - 2.0f, 3.0f);
      const float rs = s_env[0], rc = s_env[1];
      float4 irr = sample_env(a, rs, rc, diffDir, diffLod);
      F3 diffIBL = f3(kD.x * albedo.x * irr.x, kD.y * albedo.y * irr.y, kD.z * albedo.z * irr.z);
      F3 I = neg(V);
      float dNI = 2.0f * dot(N, I);
      F3 Rr = f3(I.x - dNI * N.x, I.y - dNI * N.y, I.z - dNI * N.z);
      float4 pref = sample_env(a, rs, rc, Rr, roughness * maxLod);
      int bxi = to_i32(clampf(NdotV * 255.0f, 0.0f, 255.0f));
      int byi = to_i32(clampf(roughness * 255.0f, 0.0f, 255.0f));
      uint32_t bw = a.brdf[byi * kBrdfSize + bxi];
      float bA = lo16(bw), bB = hi16(bw);
      float om = 1.0f - roughness;
      float fr = weight_pow(sat(1.0f - NdotV), 5.0f);
      F3 Fi = f3(F0.x + (mx(om, F0.x) - F0.x) * fr, F0.y + (mx(om, F0.y) - F0.y) * fr,
                 F0.z + (mx(om, F0.z) - F0.z) * fr);
      float graze = smoothstepf(0.0f, 0.02f, NdotV);
      F3 specIBL = f3(pref.x * (Fi.x * bA + bB) * graze, pref.y * (Fi.y * bA + bB) * graze,
                      pref.z * (Fi.z * bA + bB) * graze);
      ambient = muls(add(diffIBL, specIBL), ao);
    } else {
      F3 amb = f3(a.p.ambient_intensity, a.p.ambient_intensity, a.ambient_b);
      ambient = f3(amb.x * albedo.x * ao, amb.y * albedo.y * ao, amb.z * albedo.z * ao);
    }
    color = add(ambient, Lo);
  }
  F3 mapped = linear_to_srgb(tonemap(color, a.p.exposure));
  if (emag > a.p.emissive_threshold) {
    const float ei = a.p.emissive_intensity;
    mapped = f3(mapped.x + emr * ei, mapped.y + emg * ei, mapped.z + emb * ei);
  }
  *out = pack_h4(mapped.x, mapped.y, mapped.z, col.w);
}

// ---------------------------------------------------------------------------
// IBL resources
// ---------------------------------------------------------------------------
__device__ __forceinline__ float radical_inverse(uint32_t b) {
  b = (b << 16) | (b >> 16);
  b = ((b & 0x55555555u) << 1) | ((b & 0xAAAAAAAAu) >> 1);
  b = ((b & 0x33333333u) << 2) | ((b & 0xCCCCCCCCu) >> 2);
  b = ((b & 0x0F0F0F0Fu) << 4) | ((b & 0xF0F0F0F0u) >> 4);
  b = ((b & 0x00FF00FFu) << 8) | ((b & 0xFF00FF00u) >> 8);
  return (float)b * 2.3283064365386963e-10f;
}
__device__ __forceinline__ float geom_ibl(float ndv, float r) {
  float k = r * r / 2.0f;
  return ndv / (ndv * (1.0f - k) + k);
}

__global__ void __launch_bounds__(256) k_brdf_lut(uint32_t* lut) {
  int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= kBrdfSize || y >= kBrdfSize) return;
  float NdotV = mx((float)x / (float)(kBrdfSize - 1), 0.001f);
  float rough = mx((float)y / (float)(kBrdfSize - 1), 0.001f);
  F3 V = f3(sqrtf(1.0f - NdotV * NdotV), 0.0f, NdotV);
  F3 N = f3(0.0f, 0.0f, 1.0f);
  float A = 0.0f, B = 0.0f;
  const float ra = rough * rough;
  // importanceSampleGGX's frame for N = (0, 0, 1): up = (1, 0, 0)
  F3 up = fabsf(N.z) < 0.999f ? f3(0.0f, 0.0f, 1.0f) : f3(1.0f, 0.0f, 0.0f);
  F3 tangent = normalize(cross(up, N));
  F3 bitangent = cross(N, tangent);
  for (uint32_t i = 0; i < 1024u; ++i) {
    float xi0 = (float)i / 1024.0f, xi1 = radical_inverse(i);
    float phi = kTwoPI * xi0;
    float cosT = sqrtf((1.0f - xi1) / (1.0f + (ra * ra - 1.0f) * xi1));
    float sinT = sqrtf(1.0f - cosT * cosT);
    float sp, cp;
    px_sincos(phi, &sp, &cp);
    F3 Hs = f3(cp * sinT, sp * sinT, cosT);
    F3 H = normalize(f3(tangent.x * Hs.x + bitangent.x * Hs.y + N.x * Hs.z,
                        tangent.y * Hs.x + bitangent.y * Hs.y + N.y * Hs.z,
                        tangent.z * Hs.x + bitangent.z * Hs.y + N.z * Hs.z));
    float vh2 = 2.0f * dot(V, H);
    F3 L = normalize(f3(vh2 * H.x - V.x, vh2 * H.y - V.y, vh2 * H.z - V.z));
    float NdotL = mx(L.z, 0.0f);
    float NdotH = mx(H.z, 0.0f);
    float VdotH = mx(dot(V, H), 0.0f);
    if (NdotL > 0.0f) {
      float G = geom_ibl(mx(dot(N, V), 0.0f), rough) * geom_ibl(mx(dot(N, L), 0.0f), rough);
      float gv = G * VdotH / (NdotH * NdotV);
      float Fc = px_pow(1.0f - VdotH, 5.0f);
      A = A + (1.0f - Fc) * gv;
      B = B + Fc * gv;
    }
  }
  A = A / 1024.0f;
  B = B / 1024.0f;
  lut[y * kBrdfSize + x] = pack2x16(A, B);
}

__global__ void __launch_bounds__(256) k_env_mip(const uint2* src, int sw, int sh, uint2* dst, int dw, int dh) {
  int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= dw || y >= dh) return;
  int x0 = clampi(2 * x, 0, sw - 1), x1 = clampi(2 * x + 1, 0, sw - 1);
  int y0 = clampi(2 * y, 0, sh - 1), y1 = clampi(2 * y + 1, 0, sh - 1);
  float4 a = h4(src[y0 * sw + x0]), b = h4(src[y0 * sw + x1]);
  float4 c = h4(src[y1 * sw + x0]), d = h4(src[y1 * sw + x1]);
  dst[y * dw + x] = pack_h4((a.x + b.x + c.x + d.x) * 0.25f, (a.y + b.y + c.y + d.y) * 0.25f,
                            (a.z + b.z + c.z + d.z) * 0.25f, (a.w + b.w + c.w + d.w) * 0.25f);
}

dim3 grid16(int w, int h) { return dim3((unsigned)((w + 15) / 16), (unsigned)((h + 15) / 16)); }

// the reference's radius (3) unrolled; any other radius loops
void launch_bilateral(dim3 g, dim3 blk, size_t smem, cudaStream_t s, const PostArgs& a) {
  if (a.p.bilateral_radius == 3u) k_bilateral<3><<<g, blk, smem, s>>>(a);
  else k_bilateral<0><<<g, blk, smem, s>>>(a);
}

// the reference's 4 steps per side unrolled; any other count loops
void launch_gtao_main(dim3 g, dim3 blk, cudaStream_t s, const PostArgs& a, float4 projInfo) {
  if (a.p.ao_steps == 4u) k_gtao_main<4><<<g, blk, 0, s>>>(a, projInfo);
  else k_gtao_main<0><<<g, blk, 0, s>>>(a, projInfo);
}

}  // namespace

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------
struct hdsr_post {
  int W = 0, H = 0, hw = 0, hh = 0, m1w = 0, m1h = 0, m2w = 0, m2h = 0;
  uint32_t* ssn = nullptr; uint32_t* nrm = nullptr;
  float* mip0 = nullptr; float* mip1 = nullptr; float* mip2 = nullptr;
  uint2* ao_raw = nullptr; uint2* ao = nullptr; uint2* bloom_a = nullptr; uint2* bloom_b = nullptr;
  uint32_t* brdf = nullptr;
  uint2* env = nullptr; uint64_t env_texels = 0;
  int env_w = 1, env_h = 1, env_levels = 1;
  int env_lw[kMaxEnvLevels] = {}, env_lh[kMaxEnvLevels] = {};
  uint32_t env_off[kMaxEnvLevels] = {};
  uint16_t* curves = nullptr;
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  bool profiling = false;
  cudaEvent_t ev[kPasses + 1] = {};
  float pass_ms[kPasses] = {};
  std::string err;
};

namespace {

hdsr_status fail(hdsr_post* p, hdsr_status st, const std::string& msg) {
  if (p) p->err = msg;
  return st;
}
hdsr_status cuda_fail(hdsr_post* p, cudaError_t e, const char* what) {
  return fail(p, e == cudaErrorMemoryAllocation ? HDSR_ERR_OOM : HDSR_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

// materialCurves.ts generateLUT (:26-41) in double, stored as f32, then
// f32ToF16 (:44-55, truncating, no subnormals) into the rgba16float LUT.
uint16_t f16_trunc(float f) {
  uint32_t bits;
  std::memcpy(&bits, &f, 4);
  uint32_t sign = (bits >> 16) & 0x8000u;
  int e = (int)((bits >> 23) & 0xFFu) - 127 + 15;
  uint32_t frac = bits & 0x7FFFFFu;
  if (e <= 0) return (uint16_t)sign;
  if (e >= 31) return (uint16_t)(sign | 0x7C00u);
  return (uint16_t)(sign | ((uint32_t)e << 10) | (frac >> 13));
}
void curve_lut(float contrast, float brightness, float gamma, uint16_t out[256]) {
  for (int i = 0; i < 256; ++i) {
    double v = (double)i / 255.0;
    v = (v - 0.5) * (double)contrast + 0.5;
    v += (double)brightness;
    v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
    v = std::pow(v, (double)gamma);
    v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
    out[i] = f16_trunc((float)v);
  }
}

PostArgs make_args(hdsr_post* p) {
  PostArgs a;
  std::memset(&a, 0, sizeof(a));
  a.W = p->W; a.H = p->H; a.hw = p->hw; a.hh = p->hh;
  a.m1w = p->m1w; a.m1h = p->m1h; a.m2w = p->m2w; a.m2h = p->m2h;
  a.ssn = p->ssn; a.nrm = p->nrm; a.mip0 = p->mip0; a.mip1 = p->mip1; a.mip2 = p->mip2;
  a.ao_raw = p->ao_raw; a.ao = p->ao; a.bloom_a = p->bloom_a; a.bloom_b = p->bloom_b;
  a.brdf = p->brdf; a.env = p->env; a.env_w = p->env_w; a.env_h = p->env_h; a.env_levels = p->env_levels;
  for (int i = 0; i < kMaxEnvLevels; ++i) {
    a.env_lw[i] = p->env_lw[i]; a.env_lh[i] = p->env_lh[i]; a.env_off[i] = p->env_off[i];
  }
  a.curves = p->curves;
  a.vw = (float)p->W; a.vh = (float)p->H;
  a.texel_x = (float)(1.0 / (double)p->hw);
  a.texel_y = (float)(1.0 / (double)p->hh);
  a.blur_dir_h = a.texel_x; a.blur_dir_v = a.texel_y;
  return a;
}

hdsr_status set_placeholder_env(hdsr_post* p) {
  if (p->env) cudaFree(p->env);
  p->env = nullptr;
  cudaError_t e = cudaMalloc(&p->env, sizeof(uint2));
  if (e != cudaSuccess) return cuda_fail(p, e, "cudaMalloc(env)");
  uint2 white = make_uint2(0x3C003C00u, 0x3C003C00u);
  e = cudaMemcpy(p->env, &white, sizeof(uint2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(p, e, "cudaMemcpy(env)");
  p->env_w = p->env_h = 1; p->env_levels = 1; p->env_texels = 1;
  for (int i = 0; i < kMaxEnvLevels; ++i) { p->env_lw[i] = 1; p->env_lh[i] = 1; p->env_off[i] = 0; }
  return HDSR_OK;
}

}  // namespace

extern "C" {

void hdsr_post_default_params(hdsr_post_params* q) {
  if (!q) return;
  std::memset(q, 0, sizeof(*q));
  for (int i = 0; i < 16; i += 5) { q->view_proj_inverse[i] = 1.0f; q->proj[i] = 1.0f; q->view[i] = 1.0f; }
  q->normal_recovery_mode = 0;
  q->grazing_start = 0.45f; q->grazing_end = 0.80f;
  q->bilateral_spatial_sigma = 3.0f; q->bilateral_depth_sigma = 0.05f; q->bilateral_normal_sigma = 1.5f;
  q->bilateral_radius = 3;
  q->near_plane = 0.01f; q->far_plane = 100.0f;
  q->ao_radius_world = 0.15f; q->ao_falloff_end = 1.0f; q->ao_intensity = 1.5f; q->ao_thickness = 1.81f;
  q->ao_slices = 3; q->ao_steps = 4; q->frame_counter = 0; q->ao_denoise_strength = 60.0f;
  q->bloom_threshold = 0.8f; q->bloom_soft_knee = 0.5f;
  q->light_dir[0] = 0.0f; q->light_dir[1] = -1.0f; q->light_dir[2] = 0.0f;
  q->light_intensity = 3.0f; q->ambient_intensity = 0.12f;
  q->specular_only = 0;
  q->emissive_intensity = 3.0f; q->emissive_threshold = 0.05f;
  q->env_intensity = 1.0f; q->env_rotation = 0.0f; q->exposure = 1.0f;
  q->fallback_roughness = 0.65f; q->fallback_metallic = 0.0f;
}

hdsr_status hdsr_post_create(uint32_t width, uint32_t height, hdsr_post** out) {
  if (!out || width == 0 || height == 0 || width > 16384 || height > 16384)
    return HDSR_ERR_INVALID_ARG;
  *out = nullptr;
  hdsr_post* p = new (std::nothrow) hdsr_post();
  if (!p) return HDSR_ERR_OOM;
  p->W = (int)width; p->H = (int)height;
  p->hw = (p->W + 1) / 2; p->hh = (p->H + 1) / 2;
  p->m1w = (p->W + 1) / 2; p->m1h = (p->H + 1) / 2;
  p->m2w = (p->W + 3) / 4; p->m2h = (p->H + 3) / 4;
  const uint64_t px = (uint64_t)p->W * p->H, half = (uint64_t)p->hw * p->hh;
  struct { void** ptr; uint64_t bytes; } allocs[] = {
      {(void**)&p->ssn, px * 4}, {(void**)&p->nrm, px * 4}, {(void**)&p->mip0, px * 4},
      {(void**)&p->mip1, (uint64_t)p->m1w * p->m1h * 4}, {(void**)&p->mip2, (uint64_t)p->m2w * p->m2h * 4},
      {(void**)&p->ao_raw, px * 8}, {(void**)&p->ao, px * 8}, {(void**)&p->bloom_a, half * 8},
      {(void**)&p->bloom_b, half * 8}, {(void**)&p->brdf, (uint64_t)kBrdfSize * kBrdfSize * 4},
      {(void**)&p->curves, 3 * 256 * 2}};
  for (auto& al : allocs) {
    cudaError_t e = cudaMalloc(al.ptr, al.bytes);
    if (e != cudaSuccess) { hdsr_post_destroy(p); return e == cudaErrorMemoryAllocation ? HDSR_ERR_OOM : HDSR_ERR_CUDA; }
  }
  if (set_placeholder_env(p) != HDSR_OK) { hdsr_post_destroy(p); return HDSR_ERR_CUDA; }
  uint16_t lut[3 * 256];
  for (int i = 0; i < 3; ++i) curve_lut(1.0f, 0.0f, 1.0f, lut + 256 * i);
  if (cudaMemcpy(p->curves, lut, sizeof(lut), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming) != cudaSuccess) {
    hdsr_post_destroy(p);
    return HDSR_ERR_CUDA;
  }
  for (auto& e : p->ev)
    if (cudaEventCreate(&e) != cudaSuccess) { hdsr_post_destroy(p); return HDSR_ERR_CUDA; }
  k_brdf_lut<<<grid16(kBrdfSize, kBrdfSize), dim3(16, 16)>>>(p->brdf);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { hdsr_post_destroy(p); return HDSR_ERR_CUDA; }
  *out = p;
  return HDSR_OK;
}

void hdsr_post_destroy(hdsr_post* p) {
  if (!p) return;
  if (p->side) cudaStreamSynchronize(p->side);
  void* bufs[] = {p->ssn, p->nrm, p->mip0, p->mip1, p->mip2, p->ao_raw, p->ao,
                  p->bloom_a, p->bloom_b, p->brdf, p->env, p->curves};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (p->side) cudaStreamDestroy(p->side);
  if (p->fork) cudaEventDestroy(p->fork);
  if (p->join) cudaEventDestroy(p->join);
  for (auto e : p->ev)
    if (e) cudaEventDestroy(e);
  delete p;
}

hdsr_status hdsr_post_set_environment(hdsr_post* p, const uint16_t* rgba16f, uint32_t width, uint32_t height,
                                      void* stream) {
  if (!p) return HDSR_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  // earlier encodes may still read the old chain on any stream
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(p, e, "set_environment sync");
  if (width == 0 || height == 0 || !rgba16f) return set_placeholder_env(p);
  if (width > 65536 || height > 65536) return fail(p, HDSR_ERR_INVALID_ARG, "environment larger than 65536");
  // mipCount = floor(log2(max(w, h))) + 1 (ibl.ts:109)
  int levels = 1;
  while ((std::max(width, height) >> levels) > 0) ++levels;
  if (levels > kMaxEnvLevels) return fail(p, HDSR_ERR_INVALID_ARG, "too many environment levels");
  int lw[kMaxEnvLevels], lh[kMaxEnvLevels];
  uint32_t off[kMaxEnvLevels];
  uint64_t total = 0;
  for (int l = 0; l < levels; ++l) {
    lw[l] = std::max(1, (int)(width >> l));
    lh[l] = std::max(1, (int)(height >> l));
    off[l] = (uint32_t)total;
    total += (uint64_t)lw[l] * lh[l];
  }
  if (total > 0xFFFFFFFFull) return fail(p, HDSR_ERR_INVALID_ARG, "environment too large");
  uint2* env = nullptr;
  e = cudaMalloc(&env, total * sizeof(uint2));
  if (e != cudaSuccess) return cuda_fail(p, e, "cudaMalloc(env)");
  e = cudaMemcpyAsync(env, rgba16f, (uint64_t)width * height * 8, cudaMemcpyHostToDevice, s);
  for (int l = 1; l < levels && e == cudaSuccess; ++l) {
    k_env_mip<<<grid16(lw[l], lh[l]), dim3(16, 16), 0, s>>>(env + off[l - 1], lw[l - 1], lh[l - 1], env + off[l],
                                                              lw[l], lh[l]);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { cudaFree(env); return cuda_fail(p, e, "environment mip chain"); }
  if (p->env) cudaFree(p->env);
  p->env = env; p->env_texels = total;
  p->env_w = (int)width; p->env_h = (int)height; p->env_levels = levels;
  for (int l = 0; l < kMaxEnvLevels; ++l) {
    p->env_lw[l] = l < levels ? lw[l] : 1;
    p->env_lh[l] = l < levels ? lh[l] : 1;
    p->env_off[l] = l < levels ? off[l] : 0;
  }
  return HDSR_OK;
}

hdsr_status hdsr_post_set_material_curves(hdsr_post* p, const float curves[9]) {
  if (!p || !curves) return HDSR_ERR_INVALID_ARG;
  uint16_t lut[3 * 256];
  for (int i = 0; i < 3; ++i) curve_lut(curves[3 * i], curves[3 * i + 1], curves[3 * i + 2], lut + 256 * i);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(p->curves, lut, sizeof(lut), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? HDSR_OK : cuda_fail(p, e, "set_material_curves");
}

hdsr_status hdsr_post_encode(hdsr_post* p, const hdsr_post_inputs* in, const hdsr_post_params* q, void* lit,
                             uint64_t lit_pitch, void* stream) {
  if (!p || !in || !q || !lit) return fail(p, HDSR_ERR_INVALID_ARG, "null argument");
  if (!in->color || !in->depth || !in->normal || !in->material)
    return fail(p, HDSR_ERR_INVALID_ARG, "every input image is required");
  const uint64_t cb = in->color_format == HDSR_COLOR_RGBA32F ? 16u : 8u;
  if (in->color_format > HDSR_COLOR_RGBA32F) return fail(p, HDSR_ERR_INVALID_ARG, "color_format");
  if (in->color_pitch < cb * p->W || in->depth_pitch < 4u * p->W || in->normal_pitch < 4u * p->W ||
      in->material_pitch < 16u * p->W || lit_pitch < 8u * p->W)
    return fail(p, HDSR_ERR_INVALID_ARG, "row pitch smaller than the viewport");
  if (((uintptr_t)in->material | in->material_pitch) & 15u || ((uintptr_t)lit | lit_pitch) & 7u ||
      ((uintptr_t)in->color | in->color_pitch) & (cb - 1) || ((uintptr_t)in->depth | in->depth_pitch) & 3u ||
      ((uintptr_t)in->normal | in->normal_pitch) & 3u)
    return fail(p, HDSR_ERR_INVALID_ARG, "misaligned image or pitch");
  if (q->bilateral_radius > 8u) return fail(p, HDSR_ERR_INVALID_ARG, "bilateral_radius above 8");
  if (q->ao_slices == 0u || q->ao_steps == 0u) return fail(p, HDSR_ERR_INVALID_ARG, "ao slices/steps must be > 0");
  if (q->normal_recovery_mode > 2u) return fail(p, HDSR_ERR_INVALID_ARG, "normal_recovery_mode");

  PostArgs a = make_args(p);
  a.color = (const unsigned char*)in->color; a.color_pitch = in->color_pitch;
  a.color_f32 = in->color_format == HDSR_COLOR_RGBA32F;
  a.depth = (const unsigned char*)in->depth; a.depth_pitch = in->depth_pitch;
  a.src_normal = (const unsigned char*)in->normal; a.normal_pitch = in->normal_pitch;
  a.material = (const unsigned char*)in->material; a.material_pitch = in->material_pitch;
  a.lit = (unsigned char*)lit; a.lit_pitch = lit_pitch;
  a.p = *q;
  a.ambient_b = (float)((double)q->ambient_intensity * 1.1);
  // gtao.ts:145-151: projInfo from projMatrix, computed in double, stored f32
  float4 projInfo = make_float4((float)(2.0 / (double)q->proj[0]), (float)(-2.0 / (double)q->proj[5]),
                                (float)(-1.0 / (double)q->proj[0]), (float)(1.0 / (double)q->proj[5]));

  cudaStream_t s = (cudaStream_t)stream;
  const dim3 blk(16, 16);
  const dim3 g = grid16(p->W, p->H), gh = grid16(p->hw, p->hh);
  const int R = (int)q->bilateral_radius;
  const size_t bil_smem = (size_t)(16 + 2 * R) * (16 + 2 * R) * sizeof(float4);
  cudaError_t e = cudaSuccess;
  if (p->profiling) {
    cudaEventRecord(p->ev[0], s);
    k_ss_normals<<<g, blk, 0, s>>>(a);
    cudaEventRecord(p->ev[1], s);
    launch_bilateral(g, blk, bil_smem, s, a);
    cudaEventRecord(p->ev[2], s);
    k_gtao_prefilter<<<g, blk, 0, s>>>(a);
    cudaEventRecord(p->ev[3], s);
    launch_gtao_main(g, blk, s, a, projInfo);
    cudaEventRecord(p->ev[4], s);
    k_gtao_denoise<<<g, blk, 0, s>>>(a);
    cudaEventRecord(p->ev[5], s);
    k_bloom_threshold<<<gh, blk, 0, s>>>(a);
    k_bloom_blur<<<gh, blk, 0, s>>>(a, p->bloom_a, p->bloom_b, a.blur_dir_h, 0.0f);
    k_bloom_blur<<<gh, blk, 0, s>>>(a, p->bloom_b, p->bloom_a, 0.0f, a.blur_dir_v);
    cudaEventRecord(p->ev[6], s);
    k_lighting<<<g, blk, 0, s>>>(a);
    cudaEventRecord(p->ev[7], s);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(p->ev[7]);
    if (e == cudaSuccess)
      for (int i = 0; i < kPasses; ++i) cudaEventElapsedTime(&p->pass_ms[i], p->ev[i], p->ev[i + 1]);
  } else {
    // bloom reads only the material image: it runs on the side stream while
    // the normal and AO chain runs on the caller's
    e = cudaEventRecord(p->fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p->side, p->fork, 0);
    if (e == cudaSuccess) {
      k_bloom_threshold<<<gh, blk, 0, p->side>>>(a);
      k_bloom_blur<<<gh, blk, 0, p->side>>>(a, p->bloom_a, p->bloom_b, a.blur_dir_h, 0.0f);
      k_bloom_blur<<<gh, blk, 0, p->side>>>(a, p->bloom_b, p->bloom_a, 0.0f, a.blur_dir_v);
      e = cudaEventRecord(p->join, p->side);
    }
    if (e == cudaSuccess) {
      k_ss_normals<<<g, blk, 0, s>>>(a);
      launch_bilateral(g, blk, bil_smem, s, a);
      k_gtao_prefilter<<<g, blk, 0, s>>>(a);
      launch_gtao_main(g, blk, s, a, projInfo);
      k_gtao_denoise<<<g, blk, 0, s>>>(a);
      e = cudaStreamWaitEvent(s, p->join, 0);
    }
    if (e == cudaSuccess) {
      k_lighting<<<g, blk, 0, s>>>(a);
      e = cudaGetLastError();
    }
  }
  return e == cudaSuccess ? HDSR_OK : cuda_fail(p, e, "post encode");
}

hdsr_status hdsr_post_get_buffer(hdsr_post* p, hdsr_post_buffer_id id, void** ptr, uint64_t* bytes) {
  if (!p || !ptr || !bytes) return HDSR_ERR_INVALID_ARG;
  const uint64_t px = (uint64_t)p->W * p->H, half = (uint64_t)p->hw * p->hh;
  switch (id) {
    case HDSR_POST_SCREEN_NORMALS: *ptr = p->ssn; *bytes = px * 4; break;
    case HDSR_POST_NORMALS: *ptr = p->nrm; *bytes = px * 4; break;
    case HDSR_POST_DEPTH_MIP0: *ptr = p->mip0; *bytes = px * 4; break;
    case HDSR_POST_DEPTH_MIP1: *ptr = p->mip1; *bytes = (uint64_t)p->m1w * p->m1h * 4; break;
    case HDSR_POST_DEPTH_MIP2: *ptr = p->mip2; *bytes = (uint64_t)p->m2w * p->m2h * 4; break;
    case HDSR_POST_AO_RAW: *ptr = p->ao_raw; *bytes = px * 8; break;
    case HDSR_POST_AO: *ptr = p->ao; *bytes = px * 8; break;
    case HDSR_POST_BLOOM: *ptr = p->bloom_a; *bytes = half * 8; break;
    case HDSR_POST_BLOOM_H: *ptr = p->bloom_b; *bytes = half * 8; break;
    case HDSR_POST_BRDF_LUT: *ptr = p->brdf; *bytes = (uint64_t)kBrdfSize * kBrdfSize * 4; break;
    case HDSR_POST_ENV: *ptr = p->env; *bytes = p->env_texels * 8; break;
    case HDSR_POST_CURVES: *ptr = p->curves; *bytes = 3 * 256 * 2; break;
    default: return fail(p, HDSR_ERR_INVALID_ARG, "unknown buffer id");
  }
  return HDSR_OK;
}

hdsr_status hdsr_post_set_profiling(hdsr_post* p, int enable) {
  if (!p) return HDSR_ERR_INVALID_ARG;
  p->profiling = enable != 0;
  return HDSR_OK;
}

hdsr_status hdsr_post_pass_times(hdsr_post* p, float ms[7]) {
  if (!p || !ms) return HDSR_ERR_INVALID_ARG;
  for (int i = 0; i < kPasses; ++i) ms[i] = p->pass_ms[i];
  return HDSR_OK;
}

const char* hdsr_post_last_error(const hdsr_post* p) { return p ? p->err.c_str() : "null handle"; }

}  // extern "C"
