// hdsr_raster.cu — front-to-back tile rasteriser with G-buffer voting.
//
// Follows composite in gpu_tile_splat_composite.wgsl:162-370: per pixel
// (centre at +0.5) over the tile's entries in order, power = -0.5 a dx^2 -
// 0.5 c dy^2 - b dx dy; skip the splat when all four powers of a 2x2 quad are
// <= -4; alpha = min(0.99, opacity * exp(power)); a pixel takes the splat
// only when power > -4, alpha > 1/255 and T >= 0.001; G-buffer votes are
// gated at weight > 0.01; a quad stops once all four T < 0.001.
//
// GB300 layout: a warp owns half a tile (16x8 pixels, one 2x2 quad per
// lane), taken from an atomic counter in the work order, so that each half
// stops on its own. The work order starts the most expensive tiles first:
// every raster records each half tile's cost, and the next frame's
// k_work_order sorts the tiles by it (a tile's list length does not predict
// how far its pixels go before they saturate, its last cost does). It
// reads the tile's entries straight from its superblock's depth-ordered list
// (no per-tile list is written on the frame path; see k_raster), culls them
// against the half tile, gathers the kept ones from the SoA projection cache
// (one entry per lane, 16-byte loads) into the warp's shared-memory slab and
// reads them as broadcasts. FP32 transmittance.
// Arithmetic is the canonical form: power = fma(c' dy, dy, fma(b' dx, dy,
// (a' dx) dx)), the Gaussian splat_expf(power) (hdsr_math.cuh) and every
// "acc += v * w" is fma(v, w, acc).
#include "hdsr_internal.cuh"

namespace hdsr {

namespace {

constexpr int kWarps = 4;
// A staged entry is five float4 rows (entry-major): the splat loop reads them
// as five broadcast 16-byte loads; the staging stores (80-byte lane stride)
// touch distinct banks within each 8-lane phase.
//   row 0: cx, cy, -a/2, -b     row 1: -c/2, opacity, r, g
//   row 2: b, depth, rough, met row 3: nx, ny, nz, confidence
//   row 4: er, eg, eb, flags (bits, not a value: kEmits, kVotesNonFinite)
constexpr int kRows = 5;
constexpr uint32_t kEmits = 1u;           // some emissive channel is not zero
constexpr uint32_t kVotesNonFinite = 2u;  // depth, material, normal, confidence or emission not finite

struct Quad {
  float T[4];
  float c[4][3];
  float gd[4], gw[4], gc[4];
  float m[4][2];
  float n[4][3];
  float e[4][3];
  bool done;
};

__device__ __forceinline__ void quad_init(Quad& q) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q.T[i] = 1.0f;
    q.gd[i] = q.gw[i] = q.gc[i] = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) { q.c[i][k] = 0.0f; q.n[i][k] = 0.0f; q.e[i][k] = 0.0f; }
    q.m[i][0] = q.m[i][1] = 0.0f;
  }
  q.done = false;
}

// The composites' normalisations divide by one correctly rounded reciprocal
// (1 / |v|, 1 / (|x| + |y| + |z|), 1 / weight sum) and multiply: the canonical
// form of WGSL's normalize and '/', which allow 2.5 ulp (the oracle's
// composites take the same steps).
__device__ __forceinline__ void oct_decode(float ex, float ey, float& nx, float& ny, float& nz) {
  float x = ex, y = ey, z = (1.0f - fabsf(ex)) - fabsf(ey);
  if (z < 0.0f) {
    float sx = x >= 0.0f ? 1.0f : -1.0f;
    float sy = y >= 0.0f ? 1.0f : -1.0f;
    float x2 = (1.0f - fabsf(y)) * sx;
    float y2 = (1.0f - fabsf(x)) * sy;
    x = x2;
    y = y2;
  }
  const float rl = 1.0f / sqrtf(x * x + y * y + z * z);
  nx = x * rl;
  ny = y * rl;
  nz = z * rl;
}

__device__ __forceinline__ uint32_t oct_pack_norm(float x, float y, float z) {
  const float rl = 1.0f / sqrtf(x * x + y * y + z * z);
  x = x * rl; y = y * rl; z = z * rl;
  const float rs = 1.0f / (fabsf(x) + fabsf(y) + fabsf(z));
  float px = x * rs, py = y * rs;
  if (z < 0.0f) {
    float sx = px >= 0.0f ? 1.0f : -1.0f;
    float sy = py >= 0.0f ? 1.0f : -1.0f;
    float nx = (1.0f - fabsf(py)) * sx;
    float ny = (1.0f - fabsf(px)) * sy;
    px = nx;
    py = ny;
  }
  return pack2x16(px, py);
}

// The f16 composite variant (gpu_tile_splat_composite_f16.wgsl:53-54, 254):
// its thresholds and background are f16 constants.
__device__ __forceinline__ __half h16_bits(unsigned short b) { return __ushort_as_half(b); }
constexpr unsigned short kAlphaTh16 = 0x1C04u;  // 1.0h / 255.0h
constexpr unsigned short kCutoff16 = 0x1419u;   // 0.001h
constexpr unsigned short kBgRG16 = 0x251Fu;     // 0.02h
constexpr unsigned short kBgB16 = 0x291Fu;      // 0.04h

// One entry on the lane's quad. F16 selects the f16 variant
// (gpu_tile_splat_composite_f16.wgsl:186-233): alpha rounded to f16, T' =
// T * (1 - alpha) and the weight alpha * T as f16 products, colour by one f16
// fused multiply-add per channel; the Gaussian, alpha and the G-buffer votes
// stay f32. Every f16 operation is IEEE round-to-nearest-even (__hmul,
// __hsub, __hfma); T and the colour sums are kept as the floats of their f16
// values.
template <bool F16>
__device__ __forceinline__ void quad_splat(Quad& q, float p00x, float p00y, const float4 (*s)[kRows], int i) {
  const float4 r0 = s[i][0], r1 = s[i][1];
  const float cx = r0.x, cy = r0.y;
  const float ka = r0.z, kb = r0.w, kc = r1.x;
  const float dx0 = p00x - cx, dy0 = p00y - cy;
  const float dx1 = dx0 + 1.0f, dy1 = dy0 + 1.0f;
  const float dxv[4] = {dx0, dx1, dx0, dx1};
  const float dyv[4] = {dy0, dy0, dy1, dy1};
  float pw[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) pw[k] = fmaf(kc * dyv[k], dyv[k], fmaf(kb * dxv[k], dyv[k], (ka * dxv[k]) * dxv[k]));
  if (pw[0] <= -4.0f && pw[1] <= -4.0f && pw[2] <= -4.0f && pw[3] <= -4.0f) return;
  const float4 r2 = s[i][2], r3 = s[i][3], r4 = s[i][4];
  const float op = r1.y;
  const float sr = r1.z, sg = r1.w, sb = r2.x;
  const float sd = r2.y, mr = r2.z, mm = r2.w;
  const float nx = r3.x, ny = r3.y, nz = r3.z;
  const float sc = r3.w, er = r4.x, eg = r4.y, eb = r4.z;
  // a splat without emission adds exactly +0 to the emissive sums: skip it
  // (uniform across the warp, all lanes read the same splat)
  const uint32_t flags = f2u(r4.w);
  const bool emits = (flags & kEmits) != 0u;
  float wv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    // alpha = min(0.99, op * splat_expf(power)), with 2^k added into op's
    // exponent bits (op is 0 or a normal f16 value <= 0.99, op * 2^k stays
    // normal for k >= -6; for op = 0 and k < 0 the sum is negative or -inf,
    // an alpha the validity test rejects as it rejects 0; at a power <= -4 the
    // alpha is unused)
    const SplatExp ex = splat_exp_parts(pw[k]);
    const float al = mn(0.99f, u2f(f2u(op) + ex.kb) * ex.p);
    float w;
    if (F16) {
      const __half a16 = __float2half_rn(al), T16 = __float2half_rn(q.T[k]);
      const bool valid = (pw[k] > -4.0f) && (al > __half2float(h16_bits(kAlphaTh16))) &&
                         (q.T[k] >= __half2float(h16_bits(kCutoff16)));
      const __half w16 = valid ? __hmul(a16, T16) : __float2half_rn(0.0f);
      w = __half2float(w16);
      q.c[k][0] = __half2float(__hfma(__float2half_rn(sr), w16, __float2half_rn(q.c[k][0])));
      q.c[k][1] = __half2float(__hfma(__float2half_rn(sg), w16, __float2half_rn(q.c[k][1])));
      q.c[k][2] = __half2float(__hfma(__float2half_rn(sb), w16, __float2half_rn(q.c[k][2])));
      if (valid) q.T[k] = __half2float(__hmul(T16, __hsub(__float2half_rn(1.0f), a16)));
    } else {
      const float nT = q.T[k] * (1.0f - al);
      const bool valid = (pw[k] > -4.0f) && (al > (1.0f / 255.0f)) && (q.T[k] >= 0.001f);
      w = valid ? al * q.T[k] : 0.0f;
      q.c[k][0] = fmaf(sr, w, q.c[k][0]);
      q.c[k][1] = fmaf(sg, w, q.c[k][1]);
      q.c[k][2] = fmaf(sb, w, q.c[k][2]);
      if (valid) q.T[k] = nT;
    }
    wv[k] = w;
    if (emits) {
      q.e[k][0] = fmaf(er, w, q.e[k][0]);
      q.e[k][1] = fmaf(eg, w, q.e[k][1]);
      q.e[k][2] = fmaf(eb, w, q.e[k][2]);
    }
  }
  // G-buffer votes, weight w > 0.01 else 0 (the reference's select). A zero
  // vote of finite attributes adds +-0 to sums that start at +0 and never
  // become -0, so it leaves them as they are: the lane skips the votes when
  // none of its pixels has a weight above 0.01 and the splat's attributes
  // are finite (a non-finite one makes even a zero vote NaN, as in the
  // reference).
  if (wv[0] > 0.01f || wv[1] > 0.01f || wv[2] > 0.01f || wv[3] > 0.01f || (flags & kVotesNonFinite) != 0u) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float gw = wv[k] > 0.01f ? wv[k] : 0.0f;
      q.gd[k] = fmaf(gw, sd, q.gd[k]);
      q.gw[k] = q.gw[k] + gw;
      q.m[k][0] = fmaf(mr, gw, q.m[k][0]);
      q.m[k][1] = fmaf(mm, gw, q.m[k][1]);
      q.n[k][0] = fmaf(nx, gw, q.n[k][0]);
      q.n[k][1] = fmaf(ny, gw, q.n[k][1]);
      q.n[k][2] = fmaf(nz, gw, q.n[k][2]);
      q.gc[k] = fmaf(sc, gw, q.gc[k]);
    }
  }
  const float cut = F16 ? __half2float(h16_bits(kCutoff16)) : 0.001f;
  q.done = q.T[0] < cut && q.T[1] < cut && q.T[2] < cut && q.T[3] < cut;
}

template <bool F16>
__device__ __forceinline__ void quad_store(const FrameArgs& a, const Quad& q, uint32_t bx, uint32_t by) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t px = bx + (uint32_t)(k & 1), py = by + (uint32_t)(k >> 1);
    if (px >= a.W || py >= a.H) continue;
    const float rsw = 1.0f / mx(q.gw[k], 0.0001f);
    float cr, cg, cb;
    if (F16) {
      const __half T16 = __float2half_rn(q.T[k]);
      cr = __half2float(__hfma(T16, h16_bits(kBgRG16), __float2half_rn(q.c[k][0])));
      cg = __half2float(__hfma(T16, h16_bits(kBgRG16), __float2half_rn(q.c[k][1])));
      cb = __half2float(__hfma(T16, h16_bits(kBgB16), __float2half_rn(q.c[k][2])));
    } else {
      cr = fmaf(q.T[k], 0.02f, q.c[k][0]);
      cg = fmaf(q.T[k], 0.02f, q.c[k][1]);
      cb = fmaf(q.T[k], 0.04f, q.c[k][2]);
    }
    const float ca = 1.0f - q.T[k];
    char* crow = static_cast<char*>(a.out_color) + (size_t)py * a.color_pitch;
    if (a.color_f32) {
      reinterpret_cast<float4*>(crow)[px] = make_float4(cr, cg, cb, ca);
    } else {
      reinterpret_cast<uint2*>(crow)[px] = make_uint2(pack2x16(cr, cg), pack2x16(cb, ca));
    }
    reinterpret_cast<float*>(reinterpret_cast<char*>(a.out_depth) + (size_t)py * a.depth_pitch)[px] = q.gd[k] * rsw;
    reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(a.out_normal) + (size_t)py * a.normal_pitch)[px] =
        oct_pack_norm(q.n[k][0], q.n[k][1] + 0.0001f, q.n[k][2]);
    reinterpret_cast<uint4*>(reinterpret_cast<char*>(a.out_material) + (size_t)py * a.material_pitch)[px] =
        make_uint4(pack2x16(q.m[k][0] * rsw, q.m[k][1] * rsw), pack2x16(q.e[k][0], q.e[k][1]),
                   pack2x16(q.e[k][2], 0.0f), pack2x16(q.gc[k] * rsw, 0.0f));
  }
}

// One entry's cache row, as loaded (prefetched a chunk ahead).
struct Row {
  float4 g;
  uint4 ap, gb;
  uint32_t conf, depth;
};

__device__ __forceinline__ Row load_row(const FrameArgs& a, uint32_t r) {
  Row w;
  w.g = __ldg(a.geo + r);
  w.ap = __ldg(a.app + r);
  w.gb = __ldg(a.gb + r);
  w.conf = __ldg(&a.aux[r].y);
  w.depth = __ldg(a.depth + r);
  return w;
}

// Is any value the entry's G-buffer votes or emission multiply by a weight
// infinite or NaN? From the stored bits: the depth (f32), the material,
// octahedral normal, emission and confidence halves (f16, exponent all ones).
// Finite octahedral halves decode to a finite normal (the vector they
// normalise is never zero), so the halves decide for the normal too.
__device__ __forceinline__ bool vote_inputs_nonfinite(const Row& w) {
  constexpr uint32_t e2 = 0x7C007C00u;
  const uint32_t halves = __vcmpeq2(w.gb.x & e2, e2) | __vcmpeq2(w.gb.y & e2, e2) | __vcmpeq2(w.gb.z & e2, e2) |
                          __vcmpeq2(((w.gb.w & 0xFFFFu) | (w.conf << 16)) & e2, e2);
  return halves != 0u || (w.depth & 0x7F800000u) == 0x7F800000u;
}

__device__ __forceinline__ void stage_row(float4 (*s)[kRows], const Row& w, bool nonfinite, uint32_t slot) {
  float nx, ny, nz;
  oct_decode(lo16(w.gb.y), hi16(w.gb.y), nx, ny, nz);
  const float er = lo16(w.gb.z), eg = hi16(w.gb.z), eb = lo16(w.gb.w);
  const uint32_t flags = (er != 0.0f || eg != 0.0f || eb != 0.0f ? kEmits : 0u) | (nonfinite ? kVotesNonFinite : 0u);
  s[slot][0] = make_float4(w.g.x, w.g.y, w.g.z * -0.5f, -w.g.w);
  s[slot][1] = make_float4(u2f(w.ap.x) * -0.5f, hi16(w.ap.y), lo16(w.ap.z), hi16(w.ap.z));
  s[slot][2] = make_float4(lo16(w.ap.w), u2f(w.depth), lo16(w.gb.x), hi16(w.gb.x));
  s[slot][3] = make_float4(nx, ny, nz, lo16(w.conf));
  s[slot][4] = make_float4(er, eg, eb, u2f(flags));
}

// Resident blocks per SM the register budget is fitted to.
#ifndef HDSR_RASTER_MIN_BLOCKS
#define HDSR_RASTER_MIN_BLOCKS 4
#endif

// Work unit: half a tile (rows 0-7 or 8-15), taken from an atomic counter.
// The tile's entries come from its superblock's list through a TileWalk
// (hdsr_internal.cuh), in batches of up to 32: each lane gathers one cache
// row, the rows of the next batch in flight while the current one is
// composited.
template <bool F16>
__global__ void __launch_bounds__(kWarps * 32, HDSR_RASTER_MIN_BLOCKS) k_raster(FrameArgs a) {
  __shared__ float4 s_pay[kWarps][32][kRows];
  __shared__ uint32_t s_queue[kWarps][kWalkQueue];
  if (a.ctl[kCtlFlags] & kSkipFlags) return;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  float4 (*s)[kRows] = s_pay[warp];
  const uint32_t items = 2u * a.tile_count;
  for (;;) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(a.ctl + kCtlRasterTile, 1u);
    item = __shfl_sync(0xFFFFFFFFu, item, 0);
    if (item >= items) break;
    const uint32_t tile = a.tile_order[item >> 1], half = item & 1u;
    const uint32_t tx = tile & 0xFFFFu, ty = tile >> 16;
    const uint32_t bx = tx * 16u + (lane & 7u) * 2u;
    const uint32_t by = ty * 16u + ((lane >> 3) + 4u * half) * 2u;
    const float p00x = (float)bx + 0.5f, p00y = (float)by + 0.5f;
    // pixel centres of this half tile
    const float rx0 = (float)(tx * 16u) + 0.5f, ry0 = (float)(ty * 16u + 8u * half) + 0.5f;
    const uint32_t lt = (1u << lane) - 1u;
    Quad q;
    quad_init(q);
    TileWalk walk;
    walk.start(a, tx, ty, s_queue[warp]);
    uint32_t kept_total = 0, batches = 0;
    uint32_t rank = 0;
    uint32_t n = walk.take(a, lane, 32u, rank);
    Row cur;
    if (lane < n) cur = load_row(a, rank);
    while (n > 0u) {
      // keep, in order, the batch's entries that can reach this half tile:
      // power > -4 and alpha > 1/255 at some pixel, or power > -4 alone for
      // an entry with non-finite vote or emission inputs (the reference
      // multiplies them by the zero weight of every pixel of a quad it
      // visits, and 0 * NaN poisons the sums; the test with opacity 0.99 is
      // power > -4 alone)
      const bool nonfinite = lane < n && vote_inputs_nonfinite(cur);
      const bool keep = lane < n && reaches_rect(cur.g.x, cur.g.y, cur.g.z, cur.g.w, u2f(cur.ap.x),
                                                 nonfinite ? 0.99f : hi16(cur.ap.y), rx0, rx0 + 15.0f, ry0,
                                                 ry0 + 7.0f);
      const uint32_t kept = __ballot_sync(0xFFFFFFFFu, keep);
      if (keep) stage_row(s, cur, nonfinite, __popc(kept & lt));
      // the next batch: its rows in flight while this one is composited
      const uint32_t n2 = walk.take(a, lane, 32u, rank);
      if (lane < n2) cur = load_row(a, rank);
      __syncwarp();
      const uint32_t nk = __popc(kept);
      kept_total += nk;
      ++batches;
      for (uint32_t i = 0; i < nk; ++i)
        if (!q.done) quad_splat<F16>(q, p00x, p00y, s, (int)i);
      __syncwarp();
      if (__all_sync(0xFFFFFFFFu, q.done)) break;
      n = n2;
    }
    quad_store<F16>(a, q, bx, by);
    // this half tile's cost for the next frame's work order, in units of
    // about 0.04 us of a warp at full load (fitted to per-item times:
    // about 0.28 us per composited entry, 2.2 us per batch, 7 us per item)
    if (lane == 0) a.tile_cost[2u * (ty * a.cols + tx) + half] = 7u * kept_total + 55u * batches + 180u;
  }
}

// Work order from the last raster's costs (a tile's cost: the larger of its
// halves'), most expensive first, by a counting sort on 4 buckets per octave
// of cost: the longest tiles start first and the cheap ones fill in at the
// end (longest-processing-time-first list scheduling). The order decides
// only which warp takes a tile when; the images do not depend on it. With no
// costs recorded (a new scene's first frame) the tile scan's order stays.
constexpr int kOrderThreads = 1024;
constexpr int kOrderBuckets = 128;  // 4 per lane of one warp in the bucket scan
constexpr int kOrderUnroll = 8;

// a tile's cost: the larger of its halves' (0 past the grid)
__device__ __forceinline__ uint32_t tile_cost_of(const FrameArgs& a, uint32_t t) {
  if (t >= a.tile_count) return 0u;
  const uint2 c = reinterpret_cast<const uint2*>(a.tile_cost)[t];
  return max(c.x, c.y);
}

__device__ __forceinline__ uint32_t cost_bucket(uint32_t c) {
  const uint32_t v = c + 1u;
  const uint32_t lg = 31u - (uint32_t)__clz(v);
  const uint32_t frac = lg >= 2u ? (v >> (lg - 2u)) & 3u : (v << (2u - lg)) & 3u;
  return lg * 4u + frac;
}

__global__ void __launch_bounds__(kOrderThreads) k_work_order(FrameArgs a) {
  __shared__ uint32_t hist[kOrderBuckets];
  __shared__ uint32_t any;
  if (a.ctl[kCtlFlags] & kSkipFlags) return;
  const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
  for (uint32_t b = threadIdx.x; b < (uint32_t)kOrderBuckets; b += blockDim.x) hist[b] = 0u;
  if (threadIdx.x == 0) any = 0u;
  __syncthreads();
  // bucket sizes: one shared-memory atomic per distinct bucket of a warp;
  // each thread's costs are loaded kOrderUnroll at a time (one latency)
  const uint32_t step = blockDim.x * kOrderUnroll;
  for (uint32_t t0 = 0; t0 < a.tile_count; t0 += step) {
    uint32_t c[kOrderUnroll];
#pragma unroll
    for (int u = 0; u < kOrderUnroll; ++u) c[u] = tile_cost_of(a, t0 + u * blockDim.x + threadIdx.x);
#pragma unroll
    for (int u = 0; u < kOrderUnroll; ++u) {
      const uint32_t t = t0 + u * blockDim.x + threadIdx.x;
      if (c[u]) any = 1u;
      const uint32_t b = t < a.tile_count ? cost_bucket(c[u]) : 0xFFFFFFFFu;
      const uint32_t same = __match_any_sync(0xFFFFFFFFu, b);
      if (b != 0xFFFFFFFFu && (same & lt) == 0u) atomicAdd(&hist[b], (uint32_t)__popc(same));
    }
  }
  __syncthreads();
  if (!any) return;
  if (threadIdx.x < 32u) {
    // most expensive bucket first: each bucket's first position (a warp
    // scan over the buckets in descending order, 4 per lane)
    constexpr int kPer = kOrderBuckets / 32;
    uint32_t v[kPer], sum = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      v[k] = hist[kOrderBuckets - 1 - (int)(lane * kPer) - k];
      sum += v[k];
    }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += t;
    }
    uint32_t run = inc - sum;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      hist[kOrderBuckets - 1 - (int)(lane * kPer) - k] = run;
      run += v[k];
    }
  }
  __syncthreads();
  for (uint32_t t0 = 0; t0 < a.tile_count; t0 += step) {
    uint32_t c[kOrderUnroll];
#pragma unroll
    for (int u = 0; u < kOrderUnroll; ++u) c[u] = tile_cost_of(a, t0 + u * blockDim.x + threadIdx.x);
#pragma unroll
    for (int u = 0; u < kOrderUnroll; ++u) {
      const uint32_t t = t0 + u * blockDim.x + threadIdx.x;
      const uint32_t b = t < a.tile_count ? cost_bucket(c[u]) : 0xFFFFFFFFu;
      const uint32_t same = __match_any_sync(0xFFFFFFFFu, b);
      const uint32_t leader = (uint32_t)__ffs(same) - 1u;
      uint32_t base = 0;
      if (b != 0xFFFFFFFFu && lane == leader) base = atomicAdd(&hist[b], (uint32_t)__popc(same));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (b != 0xFFFFFFFFu) a.tile_order[base + __popc(same & lt)] = (t / a.cols) << 16 | (t % a.cols);
    }
  }
}

}  // namespace

cudaError_t launch_work_order(const FrameArgs& a, cudaStream_t s) {
  if (a.tile_count) k_work_order<<<1, kOrderThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_raster(const FrameArgs& a, cudaStream_t s) {
  // persistent warps: enough blocks to fill every SM, tiles from a counter
  const uint32_t want = (2u * a.tile_count + kWarps - 1) / kWarps;
  const uint32_t cap = (uint32_t)a.num_sms * 8u;
  const uint32_t blocks = want < cap ? want : cap;
  if (blocks) {
    if (a.composite_f16) k_raster<true><<<blocks, kWarps * 32, 0, s>>>(a);
    else k_raster<false><<<blocks, kWarps * 32, 0, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace hdsr
