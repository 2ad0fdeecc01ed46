// hdsr_dsort.cu — the frame's depth sort: the N per-splat keys
// depth bits << 32 | superblock count << 24 | sortRank into ascending
// (depth bits, sortRank) order (the order every tile's entries end in; see
// hdsr_sort.cu), as a stable LSD radix sort with 9-bit digits over a
// per-frame compressed key, with only as many passes as the frame's depth
// range needs.
//
// Compressed key. The projection writes the sentinel 0xFFFFFFFF for every
// invisible splat. Over the other keys the first kernel finds the minimum
// and maximum depth bits; with base = min rounded down to a multiple of 512
// and R = max - base, a visible key sorts on t = bits - base (order kept,
// since every visible key is >= base) and a sentinel on t = 0xFFFFFFFF. The
// pass count L is the least L <= 3 with R >> 9 (L - 1) <= 510: visible keys
// then fit in L digits whose top digit is <= 510, while a sentinel's digits
// are all 511, so after L stable passes the visible keys come first in
// (bits, sortRank) order and the sentinels follow in sortRank order — the
// order of a full 32-bit sort with ties broken by sortRank. When no L <= 3
// fits (depths spanning more than 2^26 bit patterns, e.g. negative depths
// beside positive ones), base = 0 and L = 4: the full 36-bit LSD sort of
// the raw bits, identical by construction. Rounding base to 512 keeps digit
// 0 of t equal to bits & 511, so the first histogram is taken before the
// range is known. On hot760k (depths of one sign within a factor of ~1.01)
// two passes replace four.
//
// Kernels (a fixed launch skeleton, so the frame graph can hold it; a pass
// beyond L returns at once):
//   k_dsort_upsweep0   per 2,560-key block: digit-0 counts; the visible
//                      depth range (atomic min / max, one per block);
//   k_dsort_colscan(p) pass 0 also picks (base, L); per digit, exclusive
//                      prefix of its per-block counts and the digit total;
//                      zeroes the table the next pass accumulates into;
//   k_dsort_downsweep(p) ranks each block's keys by digit p (warp match,
//                      stable), scatters them to their global positions and,
//                      unless it is the last pass, counts digit p+1 of every
//                      key by its destination block into the next table
//                      (warp-aggregated atomics); the last pass writes the
//                      sortRank words (the low 32 bits) to the depth order.
#include "hdsr_internal.cuh"

namespace hdsr {

namespace {

constexpr uint32_t kDBits = 9;
constexpr uint32_t kDBins = 1u << kDBits;
constexpr uint32_t kDMask = kDBins - 1u;
constexpr uint32_t kDPerThread = kDBins / kRadixThreads;  // digits per thread in the bookkeeping
static_assert(kDPerThread * kRadixThreads == kDBins, "digits split evenly over the threads");
constexpr uint32_t kDTopLimit = kDBins - 2u;  // the top digit of a visible key stays below the sentinel's

__device__ __forceinline__ uint32_t lane_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t dsort_t(unsigned long long key, uint32_t base) {
  const uint32_t bits = (uint32_t)(key >> 32);
  return bits == kSentinel ? bits : bits - base;
}

__global__ void __launch_bounds__(kRadixThreads) k_dsort_upsweep0(FrameArgs a) {
  __shared__ uint32_t s_hist[kDBins];
  __shared__ uint32_t s_min[kRadixThreads / 32], s_max[kRadixThreads / 32];
  __shared__ uint32_t s_flag;
  pdl_wait();
  pdl_trigger();
  if (block_skipped(a.ctl + kCtlFlags, &s_flag)) return;
  const uint32_t N = a.N, tiles = (N + kRadixTile - 1u) / kRadixTile;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  uint32_t lo = kSentinel, hi = 0u;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    for (uint32_t i = tid; i < kDBins; i += kRadixThreads) s_hist[i] = 0u;
    __syncthreads();
    const uint32_t base = tile * kRadixTile;
#pragma unroll
    for (uint32_t i = 0; i < kRadixItems; ++i) {
      const uint32_t g = base + i * kRadixThreads + tid;
      if (g < N) {
        const uint32_t bits = (uint32_t)(a.dkeys_a[g] >> 32);
        atomicAdd(&s_hist[bits & kDMask], 1u);
        if (bits != kSentinel) {
          lo = bits < lo ? bits : lo;
          hi = bits > hi ? bits : hi;
        }
      }
    }
    __syncthreads();
    for (uint32_t b = tid; b < kDBins; b += kRadixThreads) a.dsort_hist0[(size_t)b * a.dsort_tiles_cap + tile] = s_hist[b];
    __syncthreads();
  }
  lo = __reduce_min_sync(0xFFFFFFFFu, lo);
  hi = __reduce_max_sync(0xFFFFFFFFu, hi);
  if (lane == 0) {
    s_min[warp] = lo;
    s_max[warp] = hi;
  }
  __syncthreads();
  if (tid == 0) {
    for (uint32_t w = 1; w < kRadixThreads / 32; ++w) {
      lo = s_min[w] < lo ? s_min[w] : lo;
      hi = s_max[w] > hi ? s_max[w] : hi;
    }
    if (lo != kSentinel) atomicMin(a.ctl + kCtlDepthMin, lo);
    if (hi != 0u) atomicMax(a.ctl + kCtlDepthMax, hi);
  }
}

__global__ void __launch_bounds__(256) k_dsort_colscan(FrameArgs a, uint32_t p) {
  constexpr uint32_t IT = 16;
  __shared__ uint32_t s_w[8];
  __shared__ uint32_t s_carry;
  __shared__ uint32_t s_flag;
  pdl_wait();
  pdl_trigger();
  if (block_skipped(a.ctl + kCtlFlags, &s_flag)) return;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
  if (p == 0u) {
    if (blockIdx.x == 0 && tid == 0) {
      const uint32_t dmin = a.ctl[kCtlDepthMin], dmax = a.ctl[kCtlDepthMax];
      uint32_t base = 0u, L = 1u;
      if (dmin <= dmax) {  // some visible key
        base = dmin & ~kDMask;
        const uint32_t R = dmax - base;
        while (L <= 3u && (R >> (kDBits * (L - 1u))) > kDTopLimit) ++L;
        if (L > 3u) {
          base = 0u;  // the full sort of the raw bits
          L = 4u;
        }
      }
      a.ctl[kCtlDepthBase] = base;
      a.ctl[kCtlDepthPasses] = L;
    }
  } else if (p >= a.ctl[kCtlDepthPasses]) {
    return;
  }
  const uint32_t N = a.N, tiles = (N + kRadixTile - 1u) / kRadixTile;
  uint32_t* cur = (p & 1u) ? a.dsort_hist1 : a.dsort_hist0;
  uint32_t* nxt = (p & 1u) ? a.dsort_hist0 : a.dsort_hist1;
  // the next pass counts into the other table: clear it (its last reader,
  // the downsweep of pass p - 1, has finished)
  if (p + 1u < 4u) {
    const size_t words = (size_t)kDBins * a.dsort_tiles_cap;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + tid; i < words; i += (size_t)gridDim.x * blockDim.x) nxt[i] = 0u;
  }
  const uint32_t bin = blockIdx.x;
  uint32_t* col = cur + (size_t)bin * a.dsort_tiles_cap;
  if (tid == 0) s_carry = 0u;
  __syncthreads();
  for (uint32_t t0 = 0; t0 < tiles; t0 += 256u * IT) {
    const uint32_t tb = t0 + tid * IT;
    uint32_t v[IT];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < IT; ++k) {
      v[k] = tb + k < tiles ? col[tb + k] : 0u;
      sum += v[k];
    }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += x;
    }
    if (lane == 31) s_w[w] = inc;
    __syncthreads();
    uint32_t run = s_carry;
    for (uint32_t k = 0; k < w; ++k) run += s_w[k];
    run += inc - sum;
#pragma unroll
    for (uint32_t k = 0; k < IT; ++k) {
      if (tb + k < tiles) col[tb + k] = run;
      run += v[k];
    }
    __syncthreads();
    if (tid == 255) s_carry = run;
    __syncthreads();
  }
  if (tid == 0) a.dsort_total[bin] = s_carry;
}

struct DSweepSmem {
  unsigned long long keys[kRadixTile];
  uint32_t whist[kRadixThreads / 32][kDBins];
  uint32_t excl[kDBins];
  uint32_t wsum[kRadixThreads / 32];
};

// Block-wide exclusive scan of one value per thread (256 threads).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* wsum, uint32_t lane, uint32_t warp) {
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= (uint32_t)o) inc += t;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint32_t off = 0;
  for (uint32_t w = 0; w < warp; ++w) off += wsum[w];
  __syncthreads();
  return off + inc - v;
}

__global__ void __launch_bounds__(kRadixThreads, 3) k_dsort_downsweep(FrameArgs a, uint32_t p) {
  constexpr uint32_t W = kRadixThreads / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DSweepSmem& S = *reinterpret_cast<DSweepSmem*>(smem_raw);
  __shared__ uint32_t s_flag;
  pdl_wait();
  pdl_trigger();
  if (block_skipped(a.ctl + kCtlFlags, &s_flag)) return;
  const uint32_t L = a.ctl[kCtlDepthPasses];
  if (p >= L) return;
  const bool last = p + 1u == L;
  const uint32_t base_t = a.ctl[kCtlDepthBase];
  const uint32_t shift = kDBits * p;
  const uint32_t N = a.N, tiles = (N + kRadixTile - 1u) / kRadixTile;
  const unsigned long long* in = (p & 1u) ? a.dkeys_b : a.dkeys_a;
  unsigned long long* out = (p & 1u) ? a.dkeys_a : a.dkeys_b;
  const uint32_t* offs = (p & 1u) ? a.dsort_hist1 : a.dsort_hist0;
  uint32_t* nxt = (p & 1u) ? a.dsort_hist0 : a.dsort_hist1;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t lt = lane_lt();
  // global base of this thread's digits: exclusive scan of the digit totals
  uint32_t dbase[kDPerThread];
  {
    uint32_t tot[kDPerThread], sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kDPerThread; ++k) {
      tot[k] = a.dsort_total[tid * kDPerThread + k];
      sum += tot[k];
    }
    uint32_t run = block_excl_scan(sum, S.wsum, lane, warp);
#pragma unroll
    for (uint32_t k = 0; k < kDPerThread; ++k) {
      dbase[k] = run;
      run += tot[k];
    }
  }
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    for (uint32_t i = tid; i < W * kDBins; i += kRadixThreads) (&S.whist[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t base = tile * kRadixTile;
    {
      unsigned long long key[kRadixItems];
      uint32_t rank[kRadixItems];
#pragma unroll
      for (uint32_t i = 0; i < kRadixItems; ++i) {
        const uint32_t g = base + warp * (32u * kRadixItems) + i * 32u + lane;
        key[i] = g < N ? in[g] : ~0ull;
      }
#pragma unroll
      for (uint32_t i = 0; i < kRadixItems; ++i) {
        const uint32_t g = base + warp * (32u * kRadixItems) + i * 32u + lane;
        const uint32_t dig = g < N ? (dsort_t(key[i], base_t) >> shift) & kDMask : kDBins;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dig);
        const uint32_t lower = __popc(peers & lt);
        const uint32_t leader = __ffs(peers) - 1u;
        uint32_t prior = 0u;
        if (lower == 0u && dig < kDBins) prior = atomicAdd(&S.whist[warp][dig], (uint32_t)__popc(peers));
        prior = __shfl_sync(0xFFFFFFFFu, prior, leader);
        rank[i] = prior + lower;
      }
      __syncthreads();
      // this thread's digits: count over warps, tile-local start, per-warp starts
      uint32_t cnt[kDPerThread], sum = 0;
#pragma unroll
      for (uint32_t k = 0; k < kDPerThread; ++k) {
        const uint32_t d = tid * kDPerThread + k;
        uint32_t c = 0;
#pragma unroll
        for (uint32_t w = 0; w < W; ++w) c += S.whist[w][d];
        cnt[k] = c;
        sum += c;
      }
      uint32_t e = block_excl_scan(sum, S.wsum, lane, warp);
#pragma unroll
      for (uint32_t k = 0; k < kDPerThread; ++k) {
        const uint32_t d = tid * kDPerThread + k;
        S.excl[d] = dbase[k] + offs[(size_t)d * a.dsort_tiles_cap + tile] - e;
        uint32_t r = e;
#pragma unroll
        for (uint32_t w = 0; w < W; ++w) {
          const uint32_t c = S.whist[w][d];
          S.whist[w][d] = r;
          r += c;
        }
        e += cnt[k];
      }
      __syncthreads();
#pragma unroll
      for (uint32_t i = 0; i < kRadixItems; ++i) {
        const uint32_t g = base + warp * (32u * kRadixItems) + i * 32u + lane;
        if (g < N) {
          const uint32_t dig = (dsort_t(key[i], base_t) >> shift) & kDMask;
          S.keys[S.whist[warp][dig] + rank[i]] = key[i];
        }
      }
    }
    __syncthreads();
    const uint32_t count = N - base < kRadixTile ? N - base : kRadixTile;
    const uint32_t nshift = shift + kDBits;  // < 32 whenever a next pass exists (p <= 2)
    for (uint32_t j0 = 0; j0 < count; j0 += kRadixThreads) {
      const uint32_t jj = j0 + tid;
      bool act = jj < count;
      const unsigned long long k = act ? S.keys[jj] : 0ull;
      const uint32_t t = dsort_t(k, base_t);
      const uint32_t o = act ? S.excl[(t >> shift) & kDMask] + jj : 0u;
      if (act && o >= N) {  // inconsistent counts (a bug): report, do not write
        atomicOr(a.ctl + kCtlFlags, 0x10u);
        act = false;
      }
      if (last) {
        if (act) a.order[o] = (uint32_t)k;
      } else {
        if (act) out[o] = k;
        // the next pass's counts, by destination block (warp-aggregated)
        const uint32_t nd = nshift < 32u ? (t >> nshift) & kDMask : 0u;
        const uint32_t tag = act ? ((o / kRadixTile) << kDBits) | nd : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, tag);
        if (act && (peers & lt) == 0u)
          atomicAdd(nxt + (size_t)(tag & kDMask) * a.dsort_tiles_cap + (tag >> kDBits), (uint32_t)__popc(peers));
      }
    }
    __syncthreads();
  }
}

template <class K>
int resident_grid(K kernel, int threads, int sms, size_t smem) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  return per_sm * sms;
}

}  // namespace

uint32_t depth_sort_tiles(uint32_t N) { return (N + kRadixTile - 1u) / kRadixTile + 1u; }
uint32_t depth_sort_bins() { return kDBins; }

cudaError_t launch_depth_sort(const FrameArgs& a, cudaStream_t s) {
  if (!a.N) return cudaSuccess;
  static int grid = 0;
  const size_t smem = sizeof(DSweepSmem);
  if (!grid) {
    cudaError_t e = cudaFuncSetAttribute(k_dsort_downsweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    grid = resident_grid(k_dsort_downsweep, kRadixThreads, a.num_sms, smem);
  }
  const uint32_t tiles = (a.N + kRadixTile - 1u) / kRadixTile;
  const uint32_t up_grid = tiles < (uint32_t)a.num_sms * 8u ? tiles : (uint32_t)a.num_sms * 8u;
  const uint32_t down_grid = tiles < (uint32_t)grid ? tiles : (uint32_t)grid;
  // programmatic dependent launches: each kernel of the chain is scheduled
  // while its predecessor runs and waits for it in pdl_wait()
  cudaError_t e = launch_pdl(k_dsort_upsweep0, dim3(up_grid), dim3(kRadixThreads), 0, s, a);
  for (uint32_t p = 0; p < 4u && e == cudaSuccess; ++p) {
    e = launch_pdl(k_dsort_colscan, dim3(kDBins), dim3(256), 0, s, a, p);
    if (e == cudaSuccess) e = launch_pdl(k_dsort_downsweep, dim3(down_grid), dim3(kRadixThreads), smem, s, a, p);
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace hdsr
