// hdsr_project.cu — frame init, projection and tile counting.
//
// k_project follows gpu_project_splats.wgsl:112-358 step by step (one thread
// per sortRank) and writes the reference's 14-word projection cache as four
// SoA streams plus the f32 depth word, the splat's depth sort key and the
// number of superblocks (square groups of tiles) its tile box touches.
// Tile counts (count_tile_refs, gpu_tile_splat_composite.wgsl:65-84) come
// from a 2D difference grid: each splat adds its tile box with four
// additions, a 2D prefix sum gives every tile's count; a second grid at
// superblock (8x8 tiles) granularity gives the length of every superblock's
// list and so the lists' starts and their 256-entry segments. The
// superblock scan (hdsr_scan.cu) lists each splat, in ascending (depth,
// sortRank) order, once per superblock it touches, with its tile box clipped
// to the superblock; the lists replace scatter_tile_refs and the cooperative
// large-splat scatter (gpu_large_splat_scatter.wgsl). When the 20-bit log-depth keys are
// requested, k_depth_range keeps the per-tile depth min/max of the hot-tile
// bucket mapping (gpu_tile_bucket_sort.wgsl:67-72).
#include "hdsr_internal.cuh"

namespace hdsr {

namespace {

struct V3 { float x, y, z; };
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3 add3(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mul3s(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
// Quotients that share a denominator take one correctly rounded reciprocal
// and products (the canonical form of WGSL's '/' and normalize, which allow
// 2.5 ulp; the oracle's projection takes the same steps).
__device__ __forceinline__ V3 div3s(V3 a, float s) {
  const float r = 1.0f / s;
  return v3(a.x * r, a.y * r, a.z * r);
}
__device__ __forceinline__ float len3(V3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ V3 norm3(V3 a) { return div3s(a, len3(a)); }

// gpu_project_splats.wgsl:75-79
__device__ __forceinline__ V3 rotate_axis(float4 q4, V3 axis) {
  float ql = sqrtf(q4.x * q4.x + q4.y * q4.y + q4.z * q4.z + q4.w * q4.w);
  float d = mx(ql, 0.000001f);
  const float rd = 1.0f / d;
  float qx = q4.x * rd, qy = q4.y * rd, qz = q4.z * rd, qw = q4.w * rd;
  V3 u = v3(qy, qz, qw);
  V3 inner = add3(cross3(u, axis), mul3s(axis, qx));
  V3 c = cross3(u, inner);
  return add3(axis, mul3s(c, 2.0f));
}

// gpu_project_splats.wgsl:82-89
__device__ __forceinline__ uint32_t oct_pack(V3 n) {
  const float rs = 1.0f / (fabsf(n.x) + fabsf(n.y) + fabsf(n.z));
  float px = n.x * rs, py = n.y * rs;
  if (n.z < 0.0f) {
    float sx = px >= 0.0f ? 1.0f : -1.0f;
    float sy = py >= 0.0f ? 1.0f : -1.0f;
    float nx = (1.0f - fabsf(py)) * sx;
    float ny = (1.0f - fabsf(px)) * sy;
    px = nx;
    py = ny;
  }
  return pack2x16(px, py);
}

__device__ __forceinline__ float ldf(const float* p) { return __ldg(p); }

__global__ void k_frame_init(FrameArgs a) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    a.ctl[kCtlEpoch] += 1u;
    for (int k = 1; k < kCtlWords; ++k) a.ctl[k] = 0u;
    a.ctl[kCtlSplats] = a.N;
    a.ctl[kCtlDepthMin] = 0xFFFFFFFFu;
  }
  if (i < a.M) {
    a.tile_cnt[i] = 0u;
    a.tile_dmin[i] = 0xFFFFFFFFu;
    a.tile_dmax[i] = 0u;
  }
  if (i < (a.cols + 1u) * (a.rows + 1u)) a.tile_diff[i] = 0;
  if (i < (a.sb_cols + 1u) * (a.sb_rows + 1u)) a.sb_diff[i] = 0;
}

__device__ __forceinline__ void write_invisible(const FrameArgs& a, uint32_t r) {
  a.aux[r] = make_uint2(kSentinel, 0u);
  a.depth[r] = kSentinel;
  a.ntiles[r] = 0u;
  a.nsb[r] = 0u;
  a.dkeys_a[r] = ((unsigned long long)kSentinel << 32) | r;
}

// MINB: resident 256-thread blocks per SM the register budget is fitted to.
// The gathers are latency-bound, so more threads in flight help while the
// registers suffice: 6 blocks (40 registers) for scenes of SH degree 0-1
// (hot760k: 0.058 -> 0.054 ms); degrees 2-3 keep the unconstrained budget
// (at 6 blocks the degree-3 terms spill: sh3_3m 0.474 -> 0.527 ms). Both
// instantiations compute the same frame; the bound scene's degree picks one.
template <int MINB>
__global__ void __launch_bounds__(256, MINB) k_project(FrameArgs a) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.N) return;
  const float* U = a.U;
  const uint32_t N = f2u(ldf(U + 22));
  const uint32_t splatId = __ldg(a.sorted + r);
  if (splatId >= N) {
    // The reference returns without writing (stale cache); here: invisible.
    write_invisible(a, r);
    atomicOr(a.ctl + kCtlFlags, 0x4u);
    return;
  }
  const float* p = a.pos + (uint64_t)splatId * 3;
  V3 center = v3(ldf(p), ldf(p + 1), ldf(p + 2));
  float clip[4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
    clip[k] = ((ldf(U + k) * center.x + ldf(U + 4 + k) * center.y) + ldf(U + 8 + k) * center.z) +
              ldf(U + 12 + k) * 1.0f;
  if (clip[3] <= 0.0f) { write_invisible(a, r); return; }
  const float rW = 1.0f / mx(clip[3], 0.0001f);
  float ndcx = clip[0] * rW, ndcy = clip[1] * rW;
  float vpW = ldf(U + 16), vpH = ldf(U + 17);
  float cpx = (ndcx * 0.5f + 0.5f) * vpW;
  float cpy = (1.0f - (ndcy * 0.5f + 0.5f)) * vpH;
  float depthNdc = clip[2] * rW;

  const float* sl = a.scl + (uint64_t)splatId * 3;
  float4 q = __ldg(reinterpret_cast<const float4*>(a.rot) + splatId);
  float splatScale = ldf(U + 24);
  float scx = hx_expf(ldf(sl)) * splatScale;
  float scy = hx_expf(ldf(sl + 1)) * splatScale;
  float scz = hx_expf(ldf(sl + 2)) * splatScale;
  V3 axis0 = mul3s(rotate_axis(q, v3(1.0f, 0.0f, 0.0f)), scx);
  V3 axis1 = mul3s(rotate_axis(q, v3(0.0f, 1.0f, 0.0f)), scy);
  V3 axis2 = mul3s(rotate_axis(q, v3(0.0f, 0.0f, 1.0f)), scz);
  float len0 = dot3(axis0, axis0), len1 = dot3(axis1, axis1), len2 = dot3(axis2, axis2);
  float minLen = mn(len0, mn(len1, len2));
  V3 normalAxis = (len0 == minLen) ? axis0 : ((len1 == minLen) ? axis1 : axis2);
  V3 localNormal = norm3(normalAxis);

  V3 w0 = v3(ldf(U + 32), ldf(U + 36), ldf(U + 40));
  V3 w1 = v3(ldf(U + 33), ldf(U + 37), ldf(U + 41));
  V3 w2 = v3(ldf(U + 34), ldf(U + 38), ldf(U + 42));
  float vc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    vc[k] = ((ldf(U + 32 + k) * center.x + ldf(U + 36 + k) * center.y) + ldf(U + 40 + k) * center.z) +
            ldf(U + 44 + k) * 1.0f;
  float vz = mn(vc[2], -0.001f);
  const float rvz = 1.0f / vz;
  float J1x = ldf(U + 48) * rvz, J1y = ldf(U + 49) * rvz;
  float J2x = (-J1x * rvz) * vc[0];
  float J2y = (-J1y * rvz) * vc[1];
  V3 tt0 = v3(J1x * w0.x + J2x * w2.x, J1x * w0.y + J2x * w2.y, J1x * w0.z + J2x * w2.z);
  V3 tt1 = v3(J1y * w1.x + J2y * w2.x, J1y * w1.y + J2y * w2.y, J1y * w1.z + J2y * w2.z);
  V3 b0 = v3(dot3(axis0, tt0), dot3(axis1, tt0), dot3(axis2, tt0));
  V3 b1 = v3(dot3(axis0, tt1), dot3(axis1, tt1), dot3(axis2, tt1));
  float covXXraw = dot3(b0, b0), covXY = dot3(b0, b1), covYYraw = dot3(b1, b1);
  float detOrig = covXXraw * covYYraw - covXY * covXY;
  float covXX = covXXraw + 0.3f;
  float covYY = covYYraw + 0.3f;
  float detBlur = covXX * covYY - covXY * covXY;
  const float detInv = 1.0f / mx(detBlur, 0.000001f);
  float aaFactor = sqrtf(mx(detOrig * detInv, 0.0f));
  float mid = 0.5f * (covXX + covYY);
  float det = mx(detBlur, 0.1f);
  float lambda = mid + sqrtf(mx(mid * mid - det, 0.1f));
  float radius = ceilf(3.0f * sqrtf(lambda));
  if (radius <= 0.0f) { write_invisible(a, r); return; }
  float icx = covYY * detInv, icy = -covXY * detInv, icz = covXX * detInv;
  float sourceOpacity = clampf(ldf(a.opa + splatId) * aaFactor, 0.0f, 0.99f);

  float tileSize = mx(ldf(U + 18), 1.0f);
  uint32_t gx = f2u(ldf(U + 20)), gy = f2u(ldf(U + 21));
  uint32_t maxTx = (gx > 1u ? gx : 1u) - 1u, maxTy = (gy > 1u ? gy : 1u) - 1u;
  float clampedRadius = mn(radius, tileSize * 8.0f);
  float minPx = mx(cpx - clampedRadius, 0.0f), minPy = mx(cpy - clampedRadius, 0.0f);
  float maxPx = mn(cpx + clampedRadius, vpW), maxPy = mn(cpy + clampedRadius, vpH);
  const float rTile = 1.0f / tileSize;
  uint32_t t0x = min(sat_u32(floorf(minPx * rTile)), maxTx);
  uint32_t t0y = min(sat_u32(floorf(minPy * rTile)), maxTy);
  uint32_t t1x = min(sat_u32(floorf(mx((maxPx - 0.000000001f) * rTile, 0.0f))), maxTx);
  uint32_t t1y = min(sat_u32(floorf(mx((maxPy - 0.000000001f) * rTile, 0.0f))), maxTy);
  uint32_t box = (t0x & 0xFFu) | ((t0y & 0xFFu) << 8) | ((t1x & 0xFFu) << 16) | ((t1y & 0xFFu) << 24);

  // normals (gpu_project_splats.wgsl:234-291)
  V3 splatNormal = localNormal;
  const uint64_t nlen = a.nrm ? a.nrm_len : 0;
  const uint64_t nb = (uint64_t)splatId * 3;
  if (nb + 2 < nlen) {
    V3 baked = v3(ldf(a.nrm + nb), ldf(a.nrm + nb + 1), ldf(a.nrm + nb + 2));
    float bl = len3(baked);
    if (bl > 0.001f) splatNormal = div3s(baked, bl);
  }
  const uint64_t db = (uint64_t)N * 3 + (uint64_t)splatId * 3;
  if (db + 2 < nlen) {
    V3 detail = v3(ldf(a.nrm + db), ldf(a.nrm + db + 1), ldf(a.nrm + db + 2));
    float dl = len3(detail);
    if (dl > 0.001f) {
      V3 tc = (len0 >= len1 && len0 >= len2) ? axis0 : ((len1 >= len2) ? axis1 : axis2);
      V3 tp = sub3(tc, mul3s(splatNormal, dot3(tc, splatNormal)));
      float tl = len3(tp);
      if (tl > 0.001f) {
        V3 T = div3s(tp, tl);
        V3 B = cross3(splatNormal, T);
        V3 dn = div3s(detail, dl);
        V3 m = v3((T.x * dn.x + B.x * dn.y) + splatNormal.x * dn.z,
                  (T.y * dn.x + B.y * dn.y) + splatNormal.y * dn.z,
                  (T.z * dn.x + B.z * dn.y) + splatNormal.z * dn.z);
        splatNormal = norm3(m);
      }
    }
  }
  V3 cam = v3(ldf(U + 28), ldf(U + 29), ldf(U + 30));
  V3 nvd = norm3(sub3(cam, center));
  V3 fnrm = norm3(splatNormal);
  V3 fv = norm3(nvd);
  V3 faced = dot3(fnrm, fv) < 0.0f ? v3(-fnrm.x, -fnrm.y, -fnrm.z) : fnrm;
  float conf = clampf(dot3(faced, nvd), 0.0f, 1.0f);
  V3 wn = v3((ldf(U + 52) * faced.x + ldf(U + 56) * faced.y) + ldf(U + 60) * faced.z,
             (ldf(U + 53) * faced.x + ldf(U + 57) * faced.y) + ldf(U + 61) * faced.z,
             (ldf(U + 54) * faced.x + ldf(U + 58) * faced.y) + ldf(U + 62) * faced.z);
  wn = norm3(wn);
  uint32_t octw = oct_pack(wn);

  // SH colour, WGSL basis and signs (gpu_project_splats.wgsl:293-351)
  const uint32_t deg = f2u(ldf(U + 25));
  const uint32_t shStride = ((deg + 1) * (deg + 1) - 1) * 3;
  const float* sh = a.sh + (uint64_t)splatId * (3 + shStride + 3);
  float cr = ldf(sh), cg = ldf(sh + 1), cb = ldf(sh + 2);
  if (deg >= 1) {
    V3 vd = norm3(sub3(cam, center));
    float vx = vd.x, vy = vd.y, vzz = vd.z;
    const float* b1c = sh + 3;
    const float C1 = 0.4886025119029199f;
    cr = cr + C1 * ((ldf(b1c + 0) * vy + ldf(b1c + 3) * vzz) + ldf(b1c + 6) * vx);
    cg = cg + C1 * ((ldf(b1c + 1) * vy + ldf(b1c + 4) * vzz) + ldf(b1c + 7) * vx);
    cb = cb + C1 * ((ldf(b1c + 2) * vy + ldf(b1c + 5) * vzz) + ldf(b1c + 8) * vx);
    if (deg >= 2) {
      float xx = vx * vx, yy = vy * vy, zz = vzz * vzz;
      float xy = vx * vy, yz = vy * vzz, xz = vx * vzz;
      float e0 = 1.0925484305920792f * xy, e1 = 1.0925484305920792f * yz;
      float e2 = 0.31539156525252005f * ((2.0f * zz - xx) - yy);
      float e3 = 1.0925484305920792f * xz, e4 = 0.5462742152960396f * (xx - yy);
      const float* b2 = b1c + 9;
      cr = cr + ((((ldf(b2 + 0) * e0 + ldf(b2 + 3) * e1) + ldf(b2 + 6) * e2) + ldf(b2 + 9) * e3) + ldf(b2 + 12) * e4);
      cg = cg + ((((ldf(b2 + 1) * e0 + ldf(b2 + 4) * e1) + ldf(b2 + 7) * e2) + ldf(b2 + 10) * e3) + ldf(b2 + 13) * e4);
      cb = cb + ((((ldf(b2 + 2) * e0 + ldf(b2 + 5) * e1) + ldf(b2 + 8) * e2) + ldf(b2 + 11) * e3) + ldf(b2 + 14) * e4);
      if (deg >= 3) {
        float f0 = 0.5900435899266435f * vy * (3.0f * xx - yy);
        float f1 = 2.890611442640554f * vx * vy * vzz;
        float f2 = 0.4570457994644658f * vy * ((4.0f * zz - xx) - yy);
        float f3 = 0.3731763325901154f * vzz * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
        float f4 = 0.4570457994644658f * vx * ((4.0f * zz - xx) - yy);
        float f5 = 1.445305721320277f * vzz * (xx - yy);
        float f6 = 0.5900435899266435f * vx * (xx - 3.0f * yy);
        const float* b3 = b2 + 15;
        cr = cr + ((((((ldf(b3 + 0) * f0 + ldf(b3 + 3) * f1) + ldf(b3 + 6) * f2) + ldf(b3 + 9) * f3) + ldf(b3 + 12) * f4) + ldf(b3 + 15) * f5) + ldf(b3 + 18) * f6);
        cg = cg + ((((((ldf(b3 + 1) * f0 + ldf(b3 + 4) * f1) + ldf(b3 + 7) * f2) + ldf(b3 + 10) * f3) + ldf(b3 + 13) * f4) + ldf(b3 + 16) * f5) + ldf(b3 + 19) * f6);
        cb = cb + ((((((ldf(b3 + 2) * f0 + ldf(b3 + 5) * f1) + ldf(b3 + 8) * f2) + ldf(b3 + 11) * f3) + ldf(b3 + 14) * f4) + ldf(b3 + 17) * f5) + ldf(b3 + 20) * f6);
      }
    }
  }
  cr = clampf(cr, 0.0f, 1.0f);
  cg = clampf(cg, 0.0f, 1.0f);
  cb = clampf(cb, 0.0f, 1.0f);
  const float* em = sh + 3 + shStride;

  a.geo[r] = make_float4(cpx, cpy, icx, icy);
  a.app[r] = make_uint4(f2u(icz), pack2x16(radius, sourceOpacity), pack2x16(cr, cg), pack2x16(cb, 0.0f));
  a.gb[r] = make_uint4(__ldg(a.mat + splatId), octw, pack2x16(ldf(em), ldf(em + 1)), pack2x16(ldf(em + 2), 0.0f));
  a.aux[r] = make_uint2(box, pack2x16(conf, 0.0f));
  a.depth[r] = f2u(depthNdc);
  a.ntiles[r] = (t1x - t0x + 1u) * (t1y - t0y + 1u);
  const uint32_t nsb = ((t1x >> a.sb_shift) - (t0x >> a.sb_shift) + 1u) * ((t1y >> a.sb_shift) - (t0y >> a.sb_shift) + 1u);
  a.nsb[r] = nsb;
  // the superblock count (<= 9) rides in bits 24-31 of the key's sortRank word,
  // so the depth order carries it to the superblock scan without a gather
  a.dkeys_a[r] = ((unsigned long long)f2u(depthNdc) << 32) | ((unsigned long long)nsb << 24) | r;
}

// Tile counts: each visible splat adds +1 over its tile box to a 2D
// difference grid (four corner updates); a privatised copy per block lives
// in shared memory when the grid fits there.
__device__ __forceinline__ void diff_add(int* g, uint32_t stride, uint32_t box) {
  const uint32_t x0 = box & 0xFFu, y0 = (box >> 8) & 0xFFu, x1 = ((box >> 16) & 0xFFu) + 1u, y1 = (box >> 24) + 1u;
  atomicAdd(g + y0 * stride + x0, 1);
  atomicAdd(g + y0 * stride + x1, -1);
  atomicAdd(g + y1 * stride + x0, -1);
  atomicAdd(g + y1 * stride + x1, 1);
}

// The superblock box of a tile box.
__device__ __forceinline__ uint32_t sb_box(uint32_t box) {
  const uint32_t x0 = (box & 0xFFu) >> kSbShift, y0 = ((box >> 8) & 0xFFu) >> kSbShift;
  const uint32_t x1 = ((box >> 16) & 0xFFu) >> kSbShift, y1 = (box >> 24) >> kSbShift;
  return x0 | (y0 << 8) | (x1 << 16) | (y1 << 24);
}

constexpr uint32_t kDiffSmemMaxWords = (200u * 1024u) / 4u;
constexpr uint32_t kSbDiffWords = 33u * 33u;

__global__ void __launch_bounds__(1024, 1) k_tile_diff_smem(FrameArgs a) {
  extern __shared__ int s_diff[];
  const uint32_t stride = a.cols + 1u, n = stride * (a.rows + 1u);
  const uint32_t sstride = a.sb_cols + 1u, sn = sstride * (a.sb_rows + 1u);
  int* s_sb = s_diff + n;
  for (uint32_t i = threadIdx.x; i < n + sn; i += blockDim.x) s_diff[i] = 0;
  __syncthreads();
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < a.N; r += gridDim.x * blockDim.x) {
    const uint32_t box = a.aux[r].x;
    if (box != kSentinel) {
      diff_add(s_diff, stride, box);
      diff_add(s_sb, sstride, sb_box(box));
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
    if (s_diff[i]) atomicAdd(a.tile_diff + i, s_diff[i]);
  for (uint32_t i = threadIdx.x; i < sn; i += blockDim.x)
    if (s_sb[i]) atomicAdd(a.sb_diff + i, s_sb[i]);
}

__global__ void __launch_bounds__(256) k_tile_diff(FrameArgs a) {
  __shared__ int s_sb[kSbDiffWords];
  const uint32_t sstride = a.sb_cols + 1u, sn = sstride * (a.sb_rows + 1u);
  for (uint32_t i = threadIdx.x; i < sn; i += blockDim.x) s_sb[i] = 0;
  __syncthreads();
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < a.N) {
    const uint32_t box = a.aux[r].x;
    if (box != kSentinel) {
      diff_add(a.tile_diff, a.cols + 1u, box);
      diff_add(s_sb, sstride, sb_box(box));
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < sn; i += blockDim.x)
    if (s_sb[i]) atomicAdd(a.sb_diff + i, s_sb[i]);
}

// 2D inclusive prefix of the difference grid: rows, then columns; writes the
// count of tile (x, y) to tile_cnt[morton(x, y)]. The same on the superblock
// grid gives every superblock's list length; one exclusive block scan of
// (length, segments) turns those into list starts and the segment plan.
// One block of 1024 threads (>= kMaxSuperblocks).
// The cols x rows part of the grid is staged in shared memory when it fits
// (launch with that much dynamic shared memory), else scanned in place.
constexpr uint32_t kPrefixSmemMaxWords = (200u * 1024u) / 4u;

__global__ void __launch_bounds__(1024) k_tile_prefix(FrameArgs a) {
  __shared__ unsigned long long s_warp[32];
  extern __shared__ int s_grid[];
  const uint32_t stride = a.cols + 1u, cols = a.cols, rows = a.rows;
  int* g = a.tile_diff;
  uint32_t gs = stride;
  if (cols * rows <= kPrefixSmemMaxWords) {
    for (uint32_t i = threadIdx.x; i < cols * rows; i += blockDim.x)
      s_grid[i] = a.tile_diff[(i / cols) * stride + i % cols];
    g = s_grid;
    gs = cols;
    __syncthreads();
  }
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t nwarps = blockDim.x >> 5;
  // rows, then columns: one warp per line, 32 cells per step with a carry
  for (uint32_t y = warp; y < rows; y += nwarps) {
    int carry = 0;
    int* row = g + y * gs;
    for (uint32_t x0 = 0; x0 < cols; x0 += 32u) {
      const uint32_t x = x0 + lane;
      int v = x < cols ? row[x] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= (uint32_t)o) v += t;
      }
      v += carry;
      if (x < cols) row[x] = v;
      carry = __shfl_sync(0xFFFFFFFFu, v, 31);
    }
  }
  __syncthreads();
  for (uint32_t x = warp; x < cols; x += nwarps) {
    int carry = 0;
    for (uint32_t y0 = 0; y0 < rows; y0 += 32u) {
      const uint32_t y = y0 + lane;
      int v = y < rows ? g[y * gs + x] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= (uint32_t)o) v += t;
      }
      v += carry;
      if (y < rows) a.tile_cnt[morton(x, y)] = (uint32_t)v;
      carry = __shfl_sync(0xFFFFFFFFu, v, 31);
    }
  }
  // superblock list lengths
  const uint32_t ss = a.sb_cols + 1u;
  if (tid < a.sb_rows) {
    int run = 0;
    for (uint32_t x = 0; x < a.sb_cols; ++x) {
      run += a.sb_diff[tid * ss + x];
      a.sb_diff[tid * ss + x] = run;
    }
  }
  __syncthreads();
  if (tid < a.sb_cols) {
    int run = 0;
    for (uint32_t y = 0; y < a.sb_rows; ++y) {
      run += a.sb_diff[y * ss + tid];
      a.sb_diff[y * ss + tid] = run;
    }
  }
  __syncthreads();
  // exclusive scan of (segments << 32 | length) over the superblocks
  unsigned long long v = 0ull;
  if (tid < a.num_sb) {
    const uint32_t len = (uint32_t)a.sb_diff[(tid / a.sb_cols) * ss + tid % a.sb_cols];
    v = ((unsigned long long)((len + kSegEntries - 1u) / kSegEntries) << 32) | len;
  }
  unsigned long long inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= (uint32_t)o) inc += t;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  unsigned long long off = 0ull;
  for (uint32_t w = 0; w < warp; ++w) off += s_warp[w];
  const unsigned long long ex = off + inc - v;
  if (tid < a.num_sb) {
    a.sb_start[tid] = (uint32_t)ex;
    a.seg_first[tid] = (uint32_t)(ex >> 32);
  }
  if (tid + 1u == a.num_sb) {  // totals
    const unsigned long long all = ex + v;
    a.sb_start[a.num_sb] = (uint32_t)all;
    a.seg_first[a.num_sb] = (uint32_t)(all >> 32);
    a.ctl[kCtlSegments] = (uint32_t)(all >> 32);
    if ((uint32_t)all > a.sb_cap || (uint32_t)(all >> 32) > a.seg_cap) atomicOr(a.ctl + kCtlFlags, 0x1u);
  }
}

// Per-tile depth min/max (verification mode only): one thread per splat,
// splats above 16 tiles spread over the warp.
__global__ void __launch_bounds__(256) k_depth_range(FrameArgs a) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t box = kSentinel, d = 0u, n = 0u;
  if (r < a.N) {
    box = a.aux[r].x;
    if (box != kSentinel) { d = a.depth[r]; n = a.ntiles[r]; }
  }
  if (box != kSentinel && n <= kLargeSplatTiles) {
    const uint32_t x0 = box & 0xFFu, y0 = (box >> 8) & 0xFFu, x1 = (box >> 16) & 0xFFu, y1 = box >> 24;
    for (uint32_t ty = y0; ty <= y1; ++ty)
      for (uint32_t tx = x0; tx <= x1; ++tx) {
        const uint32_t t = morton(tx, ty);
        atomicMin(a.tile_dmin + t, d);
        atomicMax(a.tile_dmax + t, d);
      }
  }
  uint32_t large = __ballot_sync(0xFFFFFFFFu, box != kSentinel && n > kLargeSplatTiles);
  while (large) {
    const int src = __ffs(large) - 1;
    large &= large - 1u;
    const uint32_t lb = __shfl_sync(0xFFFFFFFFu, box, src);
    const uint32_t ld = __shfl_sync(0xFFFFFFFFu, d, src);
    const uint32_t ln = __shfl_sync(0xFFFFFFFFu, n, src);
    const uint32_t x0 = lb & 0xFFu, y0 = (lb >> 8) & 0xFFu, x1 = (lb >> 16) & 0xFFu;
    const uint32_t spanX = x1 - x0 + 1u;
    for (uint32_t i = lane; i < ln; i += 32u) {
      const uint32_t t = morton(x0 + i % spanX, y0 + i / spanX);
      atomicMin(a.tile_dmin + t, ld);
      atomicMax(a.tile_dmax + t, ld);
    }
  }
}

}  // namespace

cudaError_t launch_frame_init(const FrameArgs& a, cudaStream_t s) {
  const uint32_t grid_words = (a.cols + 1u) * (a.rows + 1u);
  uint32_t n = a.M > grid_words ? a.M : grid_words;
  if (n < (a.sb_cols + 1u) * (a.sb_rows + 1u)) n = (a.sb_cols + 1u) * (a.sb_rows + 1u);
  k_frame_init<<<(n + 255) / 256, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_project(const FrameArgs& a, cudaStream_t s) {
  if (a.N) {
    if (a.sh_degree <= 1u) k_project<6><<<(a.N + 255) / 256, 256, 0, s>>>(a);
    else k_project<1><<<(a.N + 255) / 256, 256, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_tile_counts(const FrameArgs& a, cudaStream_t s) {
  const uint32_t words = (a.cols + 1u) * (a.rows + 1u) + (a.sb_cols + 1u) * (a.sb_rows + 1u);
  if (a.N) {
    if (words <= kDiffSmemMaxWords) {
      static bool attr_set = false;
      if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_tile_diff_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(kDiffSmemMaxWords * 4u));
        if (e != cudaSuccess) return e;
        attr_set = true;
      }
      k_tile_diff_smem<<<a.num_sms, 1024, words * 4u, s>>>(a);
    } else {
      k_tile_diff<<<(a.N + 255) / 256, 256, 0, s>>>(a);
    }
  }
  const uint32_t pw = a.cols * a.rows;
  const size_t psmem = pw <= kPrefixSmemMaxWords ? pw * 4u : 0u;
  static bool prefix_attr_set = false;
  if (!prefix_attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_tile_prefix, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(kPrefixSmemMaxWords * 4u));
    if (e != cudaSuccess) return e;
    prefix_attr_set = true;
  }
  k_tile_prefix<<<1, 1024, psmem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_depth_range(const FrameArgs& a, cudaStream_t s) {
  if (a.N) k_depth_range<<<(a.N + 255) / 256, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hdsr
