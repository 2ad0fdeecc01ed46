// hdsr_sort.cu — the stable LSD radix sort of the frame and the optional
// 20-bit log-depth key readback.
//
// Per-tile order. Every tile's entries end in ascending (depth bits,
// sortRank) order: the order of tile_depth_sort (gpu_tile_depth_sort.wgsl:
// 28-79) and chunk_sort (gpu_tile_chunk_sort.wgsl:36-89) with sortRank
// breaking their ties, and — because the 128 log-depth buckets of the
// hot-tile cascade (gpu_tile_bucket_sort.wgsl:75-107) are monotone in the
// depth — also the cascade's order when a bucket keeps (depth, sortRank)
// order. So the frame's sort is one stable LSD radix over the composite key
// (Morton tile, depth bits, sortRank), done in two stages:
//   1. the depth digits on the N splats (depth is per splat): as many 9-bit
//      passes over u64 keys depth << 32 | sortRank as the frame's depth
//      range needs (hdsr_dsort.cu); the pairs are then emitted in that depth
//      order (hdsr_scan.cu);
//   2. the tile: the pairs are listed per superblock of 8x8 tiles by one
//      (two above 512 superblocks) stable 9-bit pass over the superblock
//      index. A tile's entries are then its superblock list filtered by the
//      entries' local rects: the rasterisers walk the lists (k_chunk_masks
//      marks which 32-entry chunks hold which tiles), and only on demand is
//      each list split by tile with a stable count/scan/scatter over
//      256-entry segments (k_seg_*), which writes the 1-u32 per-tile entries
//      (sortRank).
// Each pass is reduce-then-scan: an upsweep counts the digits of every block
// tile of keys, a column scan turns the counts into per-tile digit offsets
// and digit totals, and a downsweep (which scans the totals into the digits'
// global bases) ranks the keys
// per warp with __match_any_sync (stable: warp-striped items keep input
// order), stages them in shared memory in digit order and writes consecutive
// addresses of each digit bucket from consecutive threads.
#include "hdsr_internal.cuh"

namespace hdsr {

namespace {

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Upsweep: per block-tile digit counts, bin-major (tile_digits[bin*cap+tile]).
// BINS: the widest digit the instantiation handles (256 or 512 bins).
template <uint32_t BINS>
__global__ void __launch_bounds__(kRadixThreads) k_radix_upsweep(RadixJob j) {
  __shared__ uint32_t s_hist[BINS];
  __shared__ uint32_t s_skip;
  pdl_wait();
  pdl_trigger();
  if (block_skipped(j.flags, &s_skip)) return;
  const uint32_t P = *j.count;
  const uint32_t num_tiles = (P + kRadixTile - 1) / kRadixTile;
  const uint32_t dmask = (1u << j.bits) - 1u;
  for (uint32_t tile = blockIdx.x; tile < num_tiles; tile += gridDim.x) {
    for (uint32_t i = threadIdx.x; i < BINS; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();
    const uint32_t base = tile * kRadixTile;
    uint32_t dig[kRadixItems];
#pragma unroll
    for (uint32_t i = 0; i < kRadixItems; ++i) {
      const uint32_t g = base + i * kRadixThreads + threadIdx.x;
      dig[i] = g < P ? (uint32_t)(j.in[g] >> j.shift) & dmask : BINS;
    }
#pragma unroll
    for (uint32_t i = 0; i < kRadixItems; ++i)
      if (dig[i] < BINS) atomicAdd(&s_hist[dig[i]], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b <= dmask; b += blockDim.x)
      j.tile_digits[(size_t)b * j.tiles_cap + tile] = s_hist[b];
    __syncthreads();
  }
}

// Column scan: for every bin, exclusive prefix of its per-tile counts; the
// bin's total goes to bin_base (the downsweep scans the totals into bases).
// One block per bin, 16 tiles per thread.
__global__ void __launch_bounds__(256) k_radix_colscan(RadixJob j) {
  constexpr uint32_t IT = 16;
  __shared__ uint32_t s_w[8];
  __shared__ uint32_t s_carry;
  __shared__ uint32_t s_skip;
  pdl_wait();
  pdl_trigger();
  if (block_skipped(j.flags, &s_skip)) return;
  const uint32_t P = *j.count;
  const uint32_t num_tiles = (P + kRadixTile - 1) / kRadixTile;
  const uint32_t bin = blockIdx.x, tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
  uint32_t* col = j.tile_digits + (size_t)bin * j.tiles_cap;
  if (tid == 0) s_carry = 0u;
  __syncthreads();
  for (uint32_t t0 = 0; t0 < num_tiles; t0 += 256u * IT) {
    const uint32_t tb = t0 + tid * IT;
    uint32_t v[IT];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < IT; ++k) {
      v[k] = tb + k < num_tiles ? col[tb + k] : 0u;
      sum += v[k];
    }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t x = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += x;
    }
    if (lane == 31) s_w[w] = inc;
    __syncthreads();
    uint32_t run = s_carry;
    for (uint32_t k = 0; k < w; ++k) run += s_w[k];
    run += inc - sum;
#pragma unroll
    for (uint32_t k = 0; k < IT; ++k) {
      if (tb + k < num_tiles) col[tb + k] = run;
      run += v[k];
    }
    __syncthreads();
    if (tid == 255) s_carry = run;
    __syncthreads();
  }
  if (tid == 0) j.bin_base[bin] = s_carry;
}

// Shared memory of one downsweep block (dynamic).
template <uint32_t BINS>
struct SweepSmem {
  unsigned long long keys[kRadixTile];
  uint32_t whist[kRadixThreads / 32][BINS];
  uint32_t excl[BINS];  // per digit: global offset minus tile-local bucket start
  uint32_t wsum[kRadixThreads / 32];
};

// Block-wide exclusive scan of one value per thread (kRadixThreads threads).
__device__ __forceinline__ uint32_t radix_excl_scan(uint32_t v, uint32_t* wsum, uint32_t lane, uint32_t warp) {
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

// Downsweep: rank (warp match, leader atomic + shuffle), fold per-warp
// offsets into one table, scatter to shared memory in digit order, write out.
// BINS / kRadixThreads digits per thread in the bookkeeping.
template <uint32_t BINS, bool LAST>
__global__ void __launch_bounds__(kRadixThreads, 3) k_radix_downsweep(RadixJob j) {
  constexpr uint32_t W = kRadixThreads / 32;
  constexpr uint32_t DPT = BINS / kRadixThreads;
  static_assert(DPT * kRadixThreads == BINS, "digits split evenly over the threads");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SweepSmem<BINS>& S = *reinterpret_cast<SweepSmem<BINS>*>(smem_raw);
  __shared__ uint32_t s_skip;
  pdl_wait();
  pdl_trigger();
  if (block_skipped(j.flags, &s_skip)) return;
  const uint32_t P = *j.count;
  const uint32_t num_tiles = (P + kRadixTile - 1) / kRadixTile;
  const uint32_t shift = j.shift;
  const uint32_t dmask = (1u << j.bits) - 1u;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t lt = lanemask_lt();
  // global bases of this thread's digits: exclusive scan of the bin totals
  // (each block computes it)
  uint32_t digit_base[DPT];
  {
    uint32_t tot[DPT], sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < DPT; ++k) {
      const uint32_t d = tid * DPT + k;
      tot[k] = d <= dmask ? j.bin_base[d] : 0u;
      sum += tot[k];
    }
    uint32_t run = radix_excl_scan(sum, S.wsum, lane, warp);
#pragma unroll
    for (uint32_t k = 0; k < DPT; ++k) {
      digit_base[k] = run;
      run += tot[k];
    }
  }
  for (uint32_t tile = blockIdx.x; tile < num_tiles; tile += gridDim.x) {
    for (uint32_t i = tid; i < W * BINS; i += kRadixThreads) (&S.whist[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t base = tile * kRadixTile;
    {
      unsigned long long key[kRadixItems];
      uint32_t rank[kRadixItems];
#pragma unroll
      for (uint32_t i = 0; i < kRadixItems; ++i) {
        const uint32_t g = base + warp * (32u * kRadixItems) + i * 32u + lane;
        key[i] = g < P ? j.in[g] : ~0ull;
      }
#pragma unroll
      for (uint32_t i = 0; i < kRadixItems; ++i) {
        const uint32_t g = base + warp * (32u * kRadixItems) + i * 32u + lane;
        const uint32_t dig = g < P ? (uint32_t)(key[i] >> shift) & dmask : BINS;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dig);
        const uint32_t lower = __popc(peers & lt);
        const uint32_t leader = __ffs(peers) - 1u;
        uint32_t prior = 0u;
        if (lower == 0u && dig < BINS) prior = atomicAdd(&S.whist[warp][dig], (uint32_t)__popc(peers));
        prior = __shfl_sync(0xFFFFFFFFu, prior, leader);  // every lane reads its group's leader
        rank[i] = prior + lower;
      }
      __syncthreads();
      // this thread's digits: count over warps, tile-local bucket start,
      // per-warp offsets
      uint32_t cnt[DPT], sum = 0;
#pragma unroll
      for (uint32_t k = 0; k < DPT; ++k) {
        const uint32_t d = tid * DPT + k;
        uint32_t c = 0;
#pragma unroll
        for (uint32_t w = 0; w < W; ++w) c += S.whist[w][d];
        cnt[k] = c;
        sum += c;
      }
      uint32_t e = radix_excl_scan(sum, S.wsum, lane, warp);
#pragma unroll
      for (uint32_t k = 0; k < DPT; ++k) {
        const uint32_t d = tid * DPT + k;
        if (d <= dmask) S.excl[d] = digit_base[k] + j.tile_digits[(size_t)d * j.tiles_cap + tile] - e;
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
        if (g < P) {
          const uint32_t dig = (uint32_t)(key[i] >> shift) & dmask;
          S.keys[S.whist[warp][dig] + rank[i]] = key[i];
        }
      }
    }
    __syncthreads();
    const uint32_t count = P - base < kRadixTile ? P - base : kRadixTile;
    for (uint32_t jj = tid; jj < count; jj += kRadixThreads) {
      const unsigned long long k = S.keys[jj];
      const uint32_t o = S.excl[(uint32_t)(k >> shift) & dmask] + jj;
      if (LAST) {
        if (j.out_low) j.out_low[o] = (uint32_t)(k & j.low_mask);
        if (j.out_keys) j.out_keys[o] = k;
      } else {
        j.out[o] = k;
      }
    }
    __syncthreads();
  }
}

// Tile entries from the superblock lists. Each superblock's list (its
// splats in ascending (depth, sortRank) order, each with its tile box
// clipped to the superblock) is cut into 256-entry segments; then
//   k_seg_count:   per segment, how many of its entries cover each of the
//                  superblock's 64 tiles (a 9x9 difference grid per warp);
//   k_seg_scan:    per superblock and tile, an exclusive scan over the
//                  segments plus the tile's offset: every segment's first
//                  entry position in every tile;
//   k_seg_scatter: per segment (two warps, four tile rows each), in list
//                  order, every entry appended to every tile it covers: one
//                  ballot per covered tile gives the entries' ranks, the
//                  tile's running position lives in lane (tile & 31).
// Tile j of a superblock is (j & 7, j >> 3) in its local coordinates.

// The per-superblock segment tables, staged in shared memory once per block
// (every warp item binary-searches them).
struct SegTables {
  uint32_t first[kMaxSuperblocks + 1];
  uint32_t start[kMaxSuperblocks + 1];
};

__device__ __forceinline__ void seg_tables_load(const FrameArgs& a, SegTables& t) {
  for (uint32_t i = threadIdx.x; i <= a.num_sb; i += blockDim.x) {
    t.first[i] = a.seg_first[i];
    t.start[i] = a.sb_start[i];
  }
  __syncthreads();
}

// Segment s: its superblock and its [beg, end) in the sorted list entries.
__device__ __forceinline__ void seg_locate(const FrameArgs& a, const SegTables& t, uint32_t s, uint32_t& sb,
                                           uint32_t& beg, uint32_t& end) {
  uint32_t lo = 0u, hi = a.num_sb;  // first[lo] <= s < first[hi]
  while (hi - lo > 1u) {
    const uint32_t mid = (lo + hi) >> 1;
    if (t.first[mid] <= s) lo = mid;
    else hi = mid;
  }
  sb = lo;
  beg = t.start[sb] + (s - t.first[sb]) * kSegEntries;
  const uint32_t lim = t.start[sb + 1u];
  end = lim - beg < kSegEntries ? lim : beg + kSegEntries;
}

__global__ void __launch_bounds__(256) k_seg_count(FrameArgs a) {
  constexpr uint32_t kGrid = 9u * 9u;
  __shared__ int s_diff[8][kGrid + 3u];
  __shared__ SegTables tables;
  if (a.ctl[kCtlFlags] & kSkipFlags) return;
  seg_tables_load(a, tables);
  const uint32_t lane = threadIdx.x & 31u;
  int* d = s_diff[threadIdx.x >> 5];
  const uint32_t total = a.ctl[kCtlSegments];
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < total; s += nw) {
    uint32_t sb, beg, end;
    seg_locate(a, tables, s, sb, beg, end);
    for (uint32_t i = lane; i < kGrid; i += 32u) d[i] = 0;
    __syncwarp();
    for (uint32_t i = beg + lane; i < end; i += 32u) {
      const uint32_t rc = local_rect(a.sbk_sorted[i]);
      const uint32_t x0 = rc & 7u, x1 = ((rc >> 3) & 7u) + 1u, y0 = (rc >> 6) & 7u, y1 = (rc >> 9) + 1u;
      atomicAdd(d + y0 * 9u + x0, 1);
      atomicAdd(d + y0 * 9u + x1, -1);
      atomicAdd(d + y1 * 9u + x0, -1);
      atomicAdd(d + y1 * 9u + x1, 1);
    }
    __syncwarp();
    if (lane < 8u) {
      int run = 0;
      for (uint32_t x = 0; x < 8u; ++x) {
        run += d[lane * 9u + x];
        d[lane * 9u + x] = run;
      }
    }
    __syncwarp();
    if (lane < 8u) {
      int run = 0;
      for (uint32_t y = 0; y < 8u; ++y) {
        run += d[y * 9u + lane];
        a.seg_cnt[(size_t)s * kSbTiles + y * 8u + lane] = (uint32_t)run;
      }
    }
    __syncwarp();
  }
}

// One block per superblock: 16 groups of 64 threads (one per tile), each
// group a contiguous run of the superblock's segments.
__global__ void __launch_bounds__(1024) k_seg_scan(FrameArgs a) {
  constexpr uint32_t G = 16;
  __shared__ uint32_t s_part[G][kSbTiles];
  if (a.ctl[kCtlFlags] & kSkipFlags) return;
  const uint32_t sb = blockIdx.x, j = threadIdx.x & (kSbTiles - 1u), g = threadIdx.x / kSbTiles;
  const uint32_t f0 = a.seg_first[sb], f1 = a.seg_first[sb + 1u];
  const uint32_t per = (f1 - f0 + G - 1u) / G;
  const uint32_t s0 = f0 + g * per < f1 ? f0 + g * per : f1;
  const uint32_t s1 = s0 + per < f1 ? s0 + per : f1;
  uint32_t* cnt = a.seg_cnt + j;
  uint32_t sum = 0u;
  for (uint32_t s = s0; s < s1; ++s) sum += cnt[(size_t)s * kSbTiles];
  s_part[g][j] = sum;
  __syncthreads();
  uint32_t excl = 0u;
  for (uint32_t k = 0; k < g; ++k) excl += s_part[k][j];
  const uint32_t tx = (sb % a.sb_cols) * 8u + (j & 7u), ty = (sb / a.sb_cols) * 8u + (j >> 3);
  const bool in_frame = tx < a.cols && ty < a.rows;
  const uint32_t t = in_frame ? morton(tx, ty) : 0u;
  uint32_t run = (in_frame ? a.tile_off[t] : 0u) + excl;
  for (uint32_t s = s0; s < s1; ++s) {
    const uint32_t c = cnt[(size_t)s * kSbTiles];
    cnt[(size_t)s * kSbTiles] = run;
    run += c;
  }
  if (g == G - 1u && excl + sum != (in_frame ? a.tile_cnt[t] : 0u))
    atomicOr(a.ctl + kCtlFlags, 0x8u);  // tile counts and superblock lists disagree
  if (sb == 0u && threadIdx.x == 0u && a.sb_start[a.num_sb] != a.ctl[kCtlSbPairs])
    atomicOr(a.ctl + kCtlFlags, 0x8u);
}

#ifndef HDSR_SCATTER_STEP
#define HDSR_SCATTER_STEP 8
#endif
constexpr int kScatterStep = HDSR_SCATTER_STEP;

// Two warps per segment: half h takes tile rows 4h..4h+3 (tiles 32h + lane).
__global__ void __launch_bounds__(256) k_seg_scatter(FrameArgs a) {
  constexpr uint32_t C = kSegEntries / 32u;
  __shared__ SegTables tables;
  if (a.ctl[kCtlFlags] & kSkipFlags) return;
  seg_tables_load(a, tables);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt = lanemask_lt();
  const uint32_t total = a.ctl[kCtlSegments] * 2u;
  const uint32_t P = a.ctl[kCtlPairsLo];
  // items (segment, half) from a counter: segments differ widely in work, a
  // warp that finishes early takes the next one
  for (;;) {
    uint32_t w = 0u;
    if (lane == 0u) w = atomicAdd(a.ctl + kCtlScatterItem, 1u);
    w = __shfl_sync(0xFFFFFFFFu, w, 0);
    if (w >= total) break;
    const uint32_t s = w >> 1, half = w & 1u;
    uint32_t sb, beg, end;
    seg_locate(a, tables, s, sb, beg, end);
    // lane t: first position of tile 32 * half + t in this segment; the
    // chunk's appends collect in inc and land after the chunk (every tile is
    // visited at most once per chunk)
    uint32_t pos = a.seg_cnt[(size_t)s * kSbTiles + 32u * half + lane];
    unsigned long long k[C];
#pragma unroll
    for (uint32_t c = 0; c < C; ++c) {
      const uint32_t i = beg + c * 32u + lane;
      k[c] = i < end ? a.sbk_sorted[i] : 0ull;
    }
#pragma unroll
    for (uint32_t c = 0; c < C; ++c) {
      if (beg + c * 32u >= end) break;
      uint32_t m = 0u;
      if (beg + c * 32u + lane < end) {
        const uint32_t rc = local_rect(k[c]);
        const uint32_t x0 = rc & 7u, x1 = (rc >> 3) & 7u, y0 = (rc >> 6) & 7u, y1 = rc >> 9;
        const uint32_t cols = ((2u << x1) - 1u) & ~((1u << x0) - 1u);
        const uint32_t rows = (((2u << y1) - 1u) & ~((1u << y0) - 1u)) >> (4u * half);
        // spread row bits 0..3 to the low bit of bytes 0..3, then fill the bytes
        m = (cols * 0x01010101u) & ((((rows & 0xFu) * 0x00204081u) & 0x01010101u) * 0xFFu);
      }
      const uint32_t r = (uint32_t)k[c] & 0xFFFFFFu;
      uint32_t u = __reduce_or_sync(0xFFFFFFFFu, m);
      uint32_t inc = 0u;
      // kScatterStep covered tiles per step: independent ballot / shuffle chains
      while (u) {
        uint32_t t[kScatterStep], bq[kScatterStep];
        bool has[kScatterStep], tk[kScatterStep];
#pragma unroll
        for (int q = 0; q < kScatterStep; ++q) {
          has[q] = u != 0u;
          t[q] = has[q] ? __ffs(u) - 1u : 0u;
          u &= u - 1u;  // no-op when u == 0
        }
#pragma unroll
        for (int q = 0; q < kScatterStep; ++q) {
          tk[q] = has[q] && ((m >> t[q]) & 1u);
          bq[q] = __ballot_sync(0xFFFFFFFFu, tk[q]);
        }
#pragma unroll
        for (int q = 0; q < kScatterStep; ++q) {
          const uint32_t o = __shfl_sync(0xFFFFFFFFu, pos, t[q]) + __popc(bq[q] & lt);
          if (tk[q] && o < P) a.entries[o] = r;
        }
#pragma unroll
        for (int q = 0; q < kScatterStep; ++q)
          if (has[q] && lane == t[q]) inc += __popc(bq[q]);
      }
      pos += inc;
    }
  }
}

// Verification readback of the 20-bit log-depth keys: for every final entry
// i of tile t, sorted_keys[i] = t << (20+R) | k20 << R | sortRank (k20: the
// tile's log-depth mapping, gpu_tile_bucket_sort.wgsl:75-85, scaled to
// 2^20). One warp per tile.
__global__ void __launch_bounds__(256) k_log_depth_keys(FrameArgs a) {
  if (a.ctl[kCtlFlags] & kSkipFlags) return;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  const uint32_t R = a.rank_bits;
  for (uint32_t t = w; t < a.M; t += nw) {
    const uint32_t c = a.tile_cnt[t];
    if (!c) continue;
    const uint32_t off = a.tile_off[t];
    const float2 tl = a.tile_log[t];
    for (uint32_t i = lane; i < c; i += 32u) {
      const uint32_t r = checked_rank(a.entries[off + i], a.N, a.ctl);
      const uint32_t k = key20(log_depth(a.depth[r]), tl);
      a.sorted_keys[off + i] = ((unsigned long long)t << (20u + R)) | ((unsigned long long)k << R) | r;
    }
  }
}

// Persistent grid: as many blocks as can be resident at once.
template <class K>
int resident_blocks(K kernel, int threads, int sms, size_t smem) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  return per_sm * sms;
}

}  // namespace

template <uint32_t BINS>
static cudaError_t radix_pass(const RadixJob& j, bool last, int num_sms, cudaStream_t s) {
  static int grid_mid = 0, grid_last = 0;
  const size_t smem = sizeof(SweepSmem<BINS>);
  if (!grid_mid) {
    cudaError_t e = cudaFuncSetAttribute(k_radix_downsweep<BINS, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_radix_downsweep<BINS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    grid_mid = resident_blocks(k_radix_downsweep<BINS, false>, kRadixThreads, num_sms, smem);
    grid_last = resident_blocks(k_radix_downsweep<BINS, true>, kRadixThreads, num_sms, smem);
  }
  // programmatic dependent launches (pdl_wait at the top of each kernel)
  cudaError_t e = launch_pdl(k_radix_upsweep<BINS>, dim3(num_sms * 8), dim3(kRadixThreads), 0, s, j);
  if (e == cudaSuccess) e = launch_pdl(k_radix_colscan, dim3(1u << j.bits), dim3(256), 0, s, j);
  if (e == cudaSuccess) {
    if (last) e = launch_pdl(k_radix_downsweep<BINS, true>, dim3(grid_last), dim3(kRadixThreads), smem, s, j);
    else e = launch_pdl(k_radix_downsweep<BINS, false>, dim3(grid_mid), dim3(kRadixThreads), smem, s, j);
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_radix_pass(const RadixJob& j, bool last, int num_sms, cudaStream_t s) {
  return j.bits > kRadixBits ? radix_pass<kRadixWideBins>(j, last, num_sms, s)
                             : radix_pass<kRadixBins>(j, last, num_sms, s);
}

// Chunk masks: for every 32-entry chunk of the sorted superblock lists, the
// union of its entries' local rects (bit y * 8 + x of the superblock). The
// rasteriser walks a tile's superblock list and reads only the chunks whose
// mask holds the tile. A chunk that straddles two superblocks' lists carries
// the union over both: a reader then visits a chunk that may hold none of its
// tile's entries, which costs time only.
__global__ void __launch_bounds__(256) k_chunk_masks(FrameArgs a) {
  __shared__ uint32_t s_skip;
  pdl_wait();  // a programmatic dependent launch after the superblock pass
  if (block_skipped(a.ctl + kCtlFlags, &s_skip)) return;
  const uint32_t Q = a.ctl[kCtlSbPairs];
  const uint32_t chunks = (Q + kChunkEntries - 1u) / kChunkEntries;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < chunks; c += nw) {
    const uint32_t i = c * kChunkEntries + lane;
    const unsigned long long m = i < Q ? rect_tiles(local_rect(__ldg(a.sbk_sorted + i))) : 0ull;
    const uint32_t lo = __reduce_or_sync(0xFFFFFFFFu, (uint32_t)m);
    const uint32_t hi = __reduce_or_sync(0xFFFFFFFFu, (uint32_t)(m >> 32));
    if (lane == 0u) a.chunk_mask[c] = (unsigned long long)hi << 32 | lo;
  }
}

cudaError_t launch_chunk_masks(const FrameArgs& a, cudaStream_t s) {
  if (!a.tile_count) return cudaSuccess;
  const cudaError_t e = launch_pdl(k_chunk_masks, dim3(a.num_sms * 8), dim3(256), 0, s, a);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_tile_entries(const FrameArgs& a, cudaStream_t s) {
  if (!a.tile_count) return cudaSuccess;
  k_seg_count<<<a.num_sms * 8, 256, 0, s>>>(a);
  k_seg_scan<<<a.num_sb, 1024, 0, s>>>(a);
  k_seg_scatter<<<a.num_sms * 8, 256, 0, s>>>(a);
  return cudaGetLastError();
}

namespace {

// Keys of the back-to-front sort (gpuSortPrototype.ts:120-163, the view
// depth of viewSpaceDepthUnchecked :308-320 in double, left to right, stored
// as f32 of its negation): ascending u64 order = descending key, ties by
// ascending splat id. -0 sorts as +0 (the reference compares keys with ==);
// NaN keys sort after every other key.
__global__ void __launch_bounds__(256) k_view_keys(const float* pos, uint32_t N, double v2, double v6, double v10,
                                                   double v14, unsigned long long* keys, uint32_t* ctl) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  pdl_wait();
  pdl_trigger();
  if (i == 0) {
    ctl[kCtlSortCount] = N;
    ctl[kCtlSortFlags] = 0u;
  }
  if (i >= N) return;
  const double x = pos[(uint64_t)i * 3], y = pos[(uint64_t)i * 3 + 1], z = pos[(uint64_t)i * 3 + 2];
  const double d = ((v2 * x + v6 * y) + v10 * z) + v14;
  float k = (float)(-d);
  if (k == 0.0f) k = 0.0f;
  const uint32_t u = f2u(k);
  uint32_t ord = (u & 0x80000000u) ? ~u : (u | 0x80000000u);  // increasing with k
  if (k != k) ord = 0u;
  keys[i] = ((unsigned long long)(~ord) << 32) | i;
}

}  // namespace

cudaError_t launch_sort_back_to_front(const FrameArgs& a, const double vrow[4], uint32_t* out, cudaStream_t s) {
  if (!a.N) return cudaSuccess;
  cudaError_t ek = launch_pdl(k_view_keys, dim3((a.N + 255) / 256), dim3(256), 0, s, a.pos, a.N, vrow[0], vrow[1],
                              vrow[2], vrow[3], a.dkeys_a, a.ctl);
  if (ek != cudaSuccess) return ek;
  RadixJob j{};
  j.count = a.ctl + kCtlSortCount;
  j.flags = a.ctl + kCtlSortFlags;
  j.tile_digits = a.tile_digits;
  j.bin_base = a.bin_base;
  j.tiles_cap = a.radix_tiles_cap;
  j.low_mask = 0xFFFFFFFFull;
  for (uint32_t p = 0; p < 4; ++p) {
    j.in = (p & 1u) ? a.dkeys_b : a.dkeys_a;
    j.out = (p & 1u) ? a.dkeys_a : a.dkeys_b;
    j.out_low = out;
    j.shift = 32u + 8u * p;
    j.bits = 8u;
    cudaError_t e = launch_radix_pass(j, p == 3, a.num_sms, s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t launch_log_depth_keys(const FrameArgs& a, cudaStream_t s) {
  if (a.sorted_keys) k_log_depth_keys<<<a.num_sms * 4, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hdsr
