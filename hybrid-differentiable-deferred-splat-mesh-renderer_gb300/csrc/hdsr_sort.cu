// hdsr_sort.cu — one-sweep LSD radix sort of the (tile, log-depth) pair keys
// and the per-segment depth sort.
//
// Keys are u64: tile << (20+R) | k20 << R | sortRank, where R = rank bits.
// The radix sorts only the 20 + Morton bits above R, 8 bits per pass; the
// sortRank bits need no pass because the sort is stable and keys are emitted
// in ascending sortRank. This is the (Morton tile, log-depth) radix order the
// reference documents (README.md:77-80, gpuRadixSort.ts:1-354, never
// dispatched there) with its 16-bucket / 4-bit digits replaced by 256-way
// digits, warp match ranking, shared-memory staging and decoupled lookback
// on the digit offsets (one launch per digit, no separate scan passes).
//
// The segment check + sort replace tile_depth_sort (gpu_tile_depth_sort.wgsl:
// 114-165) and chunk_sort (gpu_tile_chunk_sort.wgsl:345-395): every segment
// (a tile of 2..4096 entries, or a 4096-entry chunk of a hot tile) ends up in
// ascending 64-bit (depth bits, sortRank) order, a total order, so the result
// is the canonical per-tile order whatever the input order.
#include "hdsr_internal.cuh"

namespace hdsr {

namespace {

__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}
__device__ __forceinline__ void st_volatile(unsigned long long* p, unsigned long long v) {
  *reinterpret_cast<volatile unsigned long long*>(p) = v;
}
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
__device__ __forceinline__ uint32_t frame_pairs(const FrameArgs& a) {
  return a.ctl[kCtlPairsLo];
}

__global__ void __launch_bounds__(256) k_radix_hist(FrameArgs a) {
  __shared__ uint32_t s_hist[kMaxPasses * 256];
  if (a.ctl[kCtlFlags] & 0x1u) return;
  const uint32_t P = frame_pairs(a);
  for (uint32_t i = threadIdx.x; i < a.passes * 256u; i += blockDim.x) s_hist[i] = 0u;
  __syncthreads();
  const uint32_t R = a.rank_bits;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    const unsigned long long k = a.pairs_a[i];
    for (uint32_t p = 0; p < a.passes; ++p) atomicAdd(&s_hist[p * 256u + (uint32_t)((k >> (R + 8u * p)) & 0xFFull)], 1u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < a.passes * 256u; i += blockDim.x)
    if (s_hist[i]) atomicAdd(a.digit_hist + i, s_hist[i]);
}

// Exclusive scan of each pass's 256 digit counts (one block per pass).
__global__ void __launch_bounds__(256) k_radix_hist_scan(FrameArgs a) {
  __shared__ uint32_t s_w[8];
  if (a.ctl[kCtlFlags] & 0x1u) return;
  const uint32_t p = blockIdx.x, d = threadIdx.x, lane = d & 31u, w = d >> 5;
  uint32_t v = a.digit_hist[p * 256u + d];
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= (uint32_t)o) inc += t;
  }
  if (lane == 31) s_w[w] = inc;
  __syncthreads();
  uint32_t off = 0;
  for (uint32_t k = 0; k < w; ++k) off += s_w[k];
  a.digit_hist[p * 256u + d] = off + inc - v;
}

template <bool LAST>
__global__ void __launch_bounds__(kRadixThreads) k_onesweep(FrameArgs a, uint32_t pass,
                                                            const unsigned long long* __restrict__ in,
                                                            unsigned long long* __restrict__ out) {
  constexpr uint32_t W = kRadixThreads / 32;
  __shared__ unsigned long long s_keys[kRadixTile];
  __shared__ uint32_t s_whist[W][256];
  __shared__ uint32_t s_excl[256];
  __shared__ uint32_t s_gbase[256];
  __shared__ uint32_t s_wsum[W];
  __shared__ uint32_t s_tile;
  if (a.ctl[kCtlFlags] & 0x1u) return;
  const uint32_t P = frame_pairs(a);
  const uint32_t num_tiles = (P + kRadixTile - 1) / kRadixTile;
  const uint32_t shift = a.rank_bits + 8u * pass;
  const uint32_t epoch = a.ctl[kCtlEpoch];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  unsigned long long* status = a.radix_status + (size_t)pass * a.radix_tiles_cap * 256u;
  const unsigned long long rank_mask = (1ull << a.rank_bits) - 1ull;
  const uint32_t lt = lanemask_lt();
  for (;;) {
    if (tid == 0) s_tile = atomicAdd(a.ctl + kCtlRadixTile + pass, 1u);
    for (uint32_t i = tid; i < W * 256u; i += kRadixThreads) (&s_whist[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= num_tiles) break;
    const uint32_t base = tile * kRadixTile;
    unsigned long long key[kRadixItems];
    uint32_t dig[kRadixItems];
    uint32_t rank[kRadixItems];
#pragma unroll
    for (uint32_t i = 0; i < kRadixItems; ++i) {
      const uint32_t g = base + warp * (32u * kRadixItems) + i * 32u + lane;
      if (g < P) {
        key[i] = in[g];
        dig[i] = (uint32_t)((key[i] >> shift) & 0xFFull);
      } else {
        key[i] = 0ull;
        dig[i] = 256u;
      }
    }
#pragma unroll
    for (uint32_t i = 0; i < kRadixItems; ++i) {
      const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dig[i]);
      const uint32_t lower = __popc(peers & lt);
      const bool valid = dig[i] < 256u;
      const uint32_t prior = valid ? s_whist[warp][dig[i]] : 0u;
      __syncwarp();
      if (valid && lower == 0u) s_whist[warp][dig[i]] = prior + __popc(peers);
      __syncwarp();
      rank[i] = prior + lower;
    }
    __syncthreads();
    // per digit: exclusive over warps, tile total, tile-local exclusive prefix
    const uint32_t d = tid;
    uint32_t run = 0;
#pragma unroll
    for (uint32_t w = 0; w < W; ++w) {
      uint32_t c = s_whist[w][d];
      s_whist[w][d] = run;
      run += c;
    }
    if (tile == 0) st_volatile(status + d, make_status(epoch, kFlagInc, run));
    else st_volatile(status + (size_t)tile * 256u + d, make_status(epoch, kFlagAgg, run));
    uint32_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += t;
    }
    if (lane == 31) s_wsum[warp] = inc;
    // lookback over previous tiles for digit d
    uint32_t prefix = 0;
    if (tile > 0) {
      int t = (int)tile - 1;
      while (t >= 0) {
        unsigned long long st;
        uint32_t spins = 0;
        for (;;) {
          st = ld_volatile(status + (size_t)t * 256u + d);
          if ((uint32_t)(st >> 34) == (epoch & 0x3FFFFFFFu) && ((st >> 32) & 3ull) != 0ull) break;
          if (++spins > kSpinLimit) {
            atomicOr(a.ctl + kCtlFlags, 0x2u);
            st = make_status(epoch, kFlagInc, 0u);
            break;
          }
          __nanosleep(32);
        }
        prefix += (uint32_t)st;
        if (((st >> 32) & 3ull) == kFlagInc) break;
        --t;
      }
      st_volatile(status + (size_t)tile * 256u + d, make_status(epoch, kFlagInc, prefix + run));
    }
    s_gbase[d] = a.digit_hist[pass * 256u + d] + prefix;
    __syncthreads();
    uint32_t woff = 0;
    for (uint32_t w = 0; w < warp; ++w) woff += s_wsum[w];
    s_excl[d] = woff + inc - run;
    __syncthreads();
#pragma unroll
    for (uint32_t i = 0; i < kRadixItems; ++i) {
      if (dig[i] < 256u) s_keys[s_excl[dig[i]] + s_whist[warp][dig[i]] + rank[i]] = key[i];
    }
    __syncthreads();
    const uint32_t count = P - base < kRadixTile ? P - base : kRadixTile;
    for (uint32_t j = tid; j < count; j += kRadixThreads) {
      const unsigned long long k = s_keys[j];
      const uint32_t dj = (uint32_t)((k >> shift) & 0xFFull);
      const uint32_t o = s_gbase[dj] + (j - s_excl[dj]);
      if (LAST) {
        a.entries[o] = (uint32_t)(k & rank_mask);
        if (a.sorted_keys) a.sorted_keys[o] = k;
      } else {
        out[o] = k;
      }
    }
    __syncthreads();
  }
}


// Check pass: one warp per segment compares every adjacent pair of entries
// under the (depth bits, sortRank) order. The radix output is ordered by the
// 20-bit log-depth key with sortRank ties, and the key is monotone in the
// depth, so a segment can only be out of order inside a run of equal keys;
// on the scenes measured here no segment is. Segments with an inversion are
// appended to the dirty list for the full sort below.
__global__ void __launch_bounds__(256) k_segcheck(FrameArgs a) {
  if (a.ctl[kCtlFlags] & 0x1u) return;
  const uint32_t nseg = min(a.ctl[kCtlSegments], a.seg_cap);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  constexpr uint32_t U = 4;  // 128 entries per warp step
  for (uint32_t sidx = wid; sidx < nseg; sidx += nw) {
    const uint2 sg = a.segments[sidx];
    const uint32_t start = sg.x;
    const uint32_t count = (sg.y <= kMaxTileEntries && (uint64_t)start + sg.y <= a.cap) ? sg.y : 0u;
    bool bad = false;
    unsigned long long carry = 0ull;  // last key of the previous step (lane-uniform)
    for (uint32_t base = 0; base < count; base += 32u * U) {
      uint32_t r[U];
      unsigned long long k[U];
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
        const uint32_t i = base + u * 32u + lane;
        r[u] = i < count ? __ldg(a.entries + start + i) : 0u;
      }
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
        const uint32_t i = base + u * 32u + lane;
        k[u] = i < count ? (((unsigned long long)__ldg(a.depth + r[u]) << 32) | r[u]) : ~0ull;
      }
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
        const uint32_t i = base + u * 32u + lane;
        const unsigned long long next = __shfl_down_sync(0xFFFFFFFFu, k[u], 1);
        const unsigned long long first = __shfl_sync(0xFFFFFFFFu, k[u], 0);
        if (lane < 31u && i + 1u < count && k[u] > next) bad = true;
        if ((base > 0u || u > 0u) && lane == 0u && carry > first) bad = true;
        carry = __shfl_sync(0xFFFFFFFFu, k[u], 31);
      }
    }
    if (__any_sync(0xFFFFFFFFu, bad) && lane == 0u) {
      const uint32_t slot = atomicAdd(a.ctl + kCtlDirty, 1u);
      a.dirty[slot] = sidx;
    }
  }
}

__device__ __forceinline__ uint32_t insert_zero_bit(uint32_t v, uint32_t bit) {
  uint32_t mask = (1u << bit) - 1u;
  return ((v >> bit) << (bit + 1u)) | (v & mask);
}

// Full sort of the dirty segments: bitonic network over the 64-bit
// (depth bits, sortRank) keys in shared memory, sized to the next power of
// two of the segment. The keys are unique, so the result is the canonical
// order whatever the input order.
__global__ void __launch_bounds__(256) k_segsort(FrameArgs a) {
  __shared__ unsigned long long s[kMaxTileEntries];
  __shared__ uint32_t s_seg;
  if (a.ctl[kCtlFlags] & 0x1u) return;
  const uint32_t ndirty = min(a.ctl[kCtlDirty], a.seg_cap);
  const uint32_t tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_seg = atomicAdd(a.ctl + kCtlSegTile, 1u);
    __syncthreads();
    const uint32_t didx = s_seg;
    if (didx >= ndirty) break;
    const uint2 sg = a.segments[a.dirty[didx]];
    const uint32_t start = sg.x;
    const uint32_t count = (sg.y <= kMaxTileEntries && (uint64_t)start + sg.y <= a.cap) ? sg.y : 0u;
    uint32_t npad = 1;
    while (npad < count) npad <<= 1;
    for (uint32_t i = tid; i < npad; i += blockDim.x) {
      if (i < count) {
        uint32_t r = a.entries[start + i];
        s[i] = ((unsigned long long)a.depth[r] << 32) | r;
      } else {
        s[i] = ~0ull;
      }
    }
    __syncthreads();
    for (uint32_t k = 2; k <= npad; k <<= 1) {
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        const uint32_t bit = __ffs(j) - 1;
        for (uint32_t c = tid; c < npad / 2; c += blockDim.x) {
          uint32_t l = insert_zero_bit(c, bit);
          uint32_t r = l | j;
          bool asc = (l & k) == 0u;
          unsigned long long x = s[l], y = s[r];
          if ((x > y) == asc) { s[l] = y; s[r] = x; }
        }
        __syncthreads();
      }
    }
    for (uint32_t i = tid; i < count; i += blockDim.x) a.entries[start + i] = (uint32_t)s[i];
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_radix_hist(const FrameArgs& a, cudaStream_t s) {
  k_radix_hist<<<a.num_sms * 4, 256, 0, s>>>(a);
  k_radix_hist_scan<<<a.passes, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// Pass p reads pairs_a (even p) or pairs_b (odd p); the last pass writes the
// sortRank entries instead of keys.
cudaError_t launch_radix_pass(const FrameArgs& a, cudaStream_t s, uint32_t p) {
  const unsigned long long* in = (p & 1u) ? a.pairs_b : a.pairs_a;
  unsigned long long* out = (p & 1u) ? a.pairs_a : a.pairs_b;
  if (p + 1 == a.passes) {
    k_onesweep<true><<<a.num_sms * 4, kRadixThreads, 0, s>>>(a, p, in, out);
  } else {
    k_onesweep<false><<<a.num_sms * 4, kRadixThreads, 0, s>>>(a, p, in, out);
  }
  return cudaGetLastError();
}

cudaError_t launch_segment_sort(const FrameArgs& a, cudaStream_t s) {
  k_segcheck<<<a.num_sms * 8, 256, 0, s>>>(a);
  k_segsort<<<a.num_sms * 4, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hdsr
