// hdsr_sblists.cu — the superblock lists of a frame, written in place.
//
// Every visible splat, taken in the depth order (ascending depth bits,
// sortRank; hdsr_dsort.cu), has one list entry in each superblock (8x8
// tiles) its tile box meets: superblock << 36 | local rect << 24 | sortRank,
// the rect being the box clipped to the superblock. The lists, superblock
// after superblock and each in depth order, replace the reference's
// scatter_tile_refs and cooperative large-splat scatter
// (gpu_tile_splat_composite.wgsl:89-119, gpu_large_splat_scatter.wgsl:52-89)
// followed by its per-tile sorts: a tile's entries are its superblock's list
// filtered by the rects (hdsr_sort.cu).
//
// An entry's position is its superblock's list start (sb_start, from the
// difference grid of the tile counts) plus the number of earlier splats of
// the depth order that meet the same superblock. Three launches compute it,
// a reduce-then-scan over tiles of 2,048 depth-order positions:
//   k_sb_count   per tile: entries per superblock (shared-memory counts);
//   k_sb_offsets per superblock: exclusive prefix over the tiles plus its
//                list start (the totals must equal the list lengths, else
//                HDSR_DEV_COUNT_MISMATCH); one extra block does the same for
//                the per-splat entry counts (the HDSR_BUF_PAIR_OFFSETS
//                words) and stores Q, the entry total;
//   k_sb_emit    per tile, 8 warps of 256 positions: per-warp counts, their
//                prefix over the warps, then rounds of 32 positions in which
//                a 32-bit lane mask per superblock (shared memory) ranks the
//                round's entries of each superblock in lane order; every
//                entry is written once, at its final position.
// The entries thus need no unsorted copy and no sort pass (before: an emit of
// all Q entries in depth order and a stable radix pass reading them twice and
// writing them again).
#include "hdsr_internal.cuh"

namespace hdsr {

namespace {

constexpr uint32_t kSbTile = 2048;                 // depth-order positions per tile
constexpr uint32_t kSbThreads = 256;
constexpr uint32_t kSbItems = kSbTile / kSbThreads;
constexpr uint32_t kSbWarps = kSbThreads / 32;
constexpr uint32_t kSbWarpSpan = kSbTile / kSbWarps;  // positions per warp (8 rounds of 32)

__device__ __forceinline__ bool sb_skipped(const FrameArgs& a, uint32_t* s_flag) {
  if (threadIdx.x == 0) *s_flag = *reinterpret_cast<volatile const uint32_t*>(a.ctl + kCtlFlags) & kSkipFlags;
  __syncthreads();
  return *s_flag != 0u;
}

// The superblock range of a tile box: sx0..sx1, sy0..sy1 (count 0 if invisible).
struct SbRange {
  uint32_t x0, y0, x1, y1, sx0, sy0, sx1, sy1;
};

__device__ __forceinline__ SbRange sb_range(uint32_t box) {
  SbRange g;
  g.x0 = box & 0xFFu;
  g.y0 = (box >> 8) & 0xFFu;
  g.x1 = (box >> 16) & 0xFFu;
  g.y1 = box >> 24;
  g.sx0 = g.x0 >> kSbShift;
  g.sy0 = g.y0 >> kSbShift;
  g.sx1 = g.x1 >> kSbShift;
  g.sy1 = g.y1 >> kSbShift;
  return g;
}

__device__ __forceinline__ uint32_t sb_count(const SbRange& g) { return (g.sx1 - g.sx0 + 1u) * (g.sy1 - g.sy0 + 1u); }

// The k-th superblock of the range (row-major) and the box clipped to it.
__device__ __forceinline__ void sb_entry(const SbRange& g, uint32_t k, uint32_t sb_cols, uint32_t& sb,
                                         uint32_t& rect) {
  const uint32_t w = g.sx1 - g.sx0 + 1u;
  const uint32_t sx = g.sx0 + k % w, sy = g.sy0 + k / w;
  const uint32_t bx = sx << kSbShift, by = sy << kSbShift;
  const uint32_t lx0 = g.x0 > bx ? g.x0 - bx : 0u, lx1 = g.x1 - bx < 7u ? g.x1 - bx : 7u;
  const uint32_t ly0 = g.y0 > by ? g.y0 - by : 0u, ly1 = g.y1 - by < 7u ? g.y1 - by : 7u;
  sb = sy * sb_cols + sx;
  rect = lx0 | (lx1 << 3) | (ly0 << 6) | (ly1 << 9);
}

// The box of depth-order position i (sentinel past N or for a bad rank).
__device__ __forceinline__ uint32_t order_box(const FrameArgs& a, uint32_t i, uint32_t& r) {
  if (i >= a.N) {
    r = 0u;
    return kSentinel;
  }
  r = checked_rank(a.order[i] & 0xFFFFFFu, a.N, a.ctl);
  return a.aux[r].x;
}

__global__ void __launch_bounds__(kSbThreads) k_sb_count(FrameArgs a) {
  extern __shared__ uint32_t s_cnt[];  // num_sb
  __shared__ uint32_t s_flag, s_tot;
  if (sb_skipped(a, &s_flag)) return;
  const uint32_t tile = blockIdx.x, base = tile * kSbTile;
  for (uint32_t i = threadIdx.x; i < a.num_sb; i += kSbThreads) s_cnt[i] = 0u;
  if (threadIdx.x == 0) s_tot = 0u;
  __syncthreads();
  uint32_t mine = 0u;
#pragma unroll
  for (uint32_t k = 0; k < kSbItems; ++k) {
    uint32_t r;
    const uint32_t box = order_box(a, base + k * kSbThreads + threadIdx.x, r);
    if (box == kSentinel) continue;
    const SbRange g = sb_range(box);
    for (uint32_t sy = g.sy0; sy <= g.sy1; ++sy)
      for (uint32_t sx = g.sx0; sx <= g.sx1; ++sx) atomicAdd(&s_cnt[sy * a.sb_cols + sx], 1u);
    mine += sb_count(g);
  }
  mine = __reduce_add_sync(0xFFFFFFFFu, mine);
  if ((threadIdx.x & 31u) == 0u) atomicAdd(&s_tot, mine);
  __syncthreads();
  for (uint32_t sb = threadIdx.x; sb < a.num_sb; sb += kSbThreads)
    a.sb_tab[(size_t)sb * a.sb_tiles_cap + tile] = s_cnt[sb];
  if (threadIdx.x == 0) a.sb_tab[(size_t)a.num_sb * a.sb_tiles_cap + tile] = s_tot;
}

// Block b < num_sb: superblock b's column; block num_sb: the per-tile totals.
__global__ void __launch_bounds__(256) k_sb_offsets(FrameArgs a, uint32_t tiles) {
  constexpr uint32_t IT = 16;
  __shared__ uint32_t s_w[8];
  __shared__ uint32_t s_carry, s_flag;
  if (sb_skipped(a, &s_flag)) return;
  const uint32_t col_id = blockIdx.x, tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
  uint32_t* col = a.sb_tab + (size_t)col_id * a.sb_tiles_cap;
  const uint32_t start = col_id < a.num_sb ? a.sb_start[col_id] : 0u;
  if (tid == 0) s_carry = start;
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
  if (tid == 0) {
    if (col_id < a.num_sb) {
      if (s_carry != a.sb_start[col_id + 1u]) atomicOr(a.ctl + kCtlFlags, 0x8u);  // counted != list length
    } else {
      a.ctl[kCtlSbPairs] = s_carry;
      if (s_carry != a.sb_start[a.num_sb]) atomicOr(a.ctl + kCtlFlags, 0x8u);
    }
  }
}

__global__ void __launch_bounds__(kSbThreads) k_sb_emit(FrameArgs a) {
  extern __shared__ uint32_t s_dyn[];
  uint32_t* s_base = s_dyn;                          // [warp][num_sb]: counts, then running positions
  uint32_t* s_mask = s_dyn + kSbWarps * a.num_sb;    // [warp][num_sb]: lanes of the round per superblock
  __shared__ uint32_t s_wtot[kSbWarps];
  __shared__ uint32_t s_flag;
  if (sb_skipped(a, &s_flag)) return;
  const uint32_t tile = blockIdx.x, lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t nsb = a.num_sb;
  for (uint32_t i = threadIdx.x; i < 2u * kSbWarps * nsb; i += kSbThreads) s_dyn[i] = 0u;
  __syncthreads();
  uint32_t* wbase = s_base + warp * nsb;
  uint32_t* wmask = s_mask + warp * nsb;
  const uint32_t first = tile * kSbTile + warp * kSbWarpSpan;
  uint32_t rk[kSbItems], bx[kSbItems];
  uint32_t wsum = 0u;
#pragma unroll
  for (uint32_t k = 0; k < kSbItems; ++k) {
    bx[k] = order_box(a, first + k * 32u + lane, rk[k]);
    if (bx[k] == kSentinel) continue;
    const SbRange g = sb_range(bx[k]);
    for (uint32_t sy = g.sy0; sy <= g.sy1; ++sy)
      for (uint32_t sx = g.sx0; sx <= g.sx1; ++sx) atomicAdd(&wbase[sy * a.sb_cols + sx], 1u);
    wsum += sb_count(g);
  }
  wsum = __reduce_add_sync(0xFFFFFFFFu, wsum);
  if (lane == 0) s_wtot[warp] = wsum;
  __syncthreads();
  // per superblock: the tile's start (k_sb_offsets) plus the earlier warps' counts
  for (uint32_t sb = threadIdx.x; sb < nsb; sb += kSbThreads) {
    uint32_t run = a.sb_tab[(size_t)sb * a.sb_tiles_cap + tile];
#pragma unroll
    for (uint32_t w = 0; w < kSbWarps; ++w) {
      const uint32_t c = s_base[w * nsb + sb];
      s_base[w * nsb + sb] = run;
      run += c;
    }
  }
  // the splats' entry offsets (HDSR_BUF_PAIR_OFFSETS): the tile's, then the warps'
  uint32_t off = a.sb_tab[(size_t)nsb * a.sb_tiles_cap + tile];
  for (uint32_t w = 0; w < warp; ++w) off += s_wtot[w];
  __syncthreads();
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (uint32_t k = 0; k < kSbItems; ++k) {
    const uint32_t i = first + k * 32u + lane;
    const bool vis = bx[k] != kSentinel;
    SbRange g;
    uint32_t cnt = 0u;
    if (vis) {
      g = sb_range(bx[k]);
      cnt = sb_count(g);
    }
    // exclusive prefix of the round's counts (lane order = depth order)
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += t;
    }
    if (i < a.N) a.sb_off[i] = off + inc - cnt;
    off += __shfl_sync(0xFFFFFFFFu, inc, 31);
    // rank the round's entries of each superblock by lane
    for (uint32_t e = 0; e < cnt; ++e) {
      uint32_t sb, rect;
      sb_entry(g, e, a.sb_cols, sb, rect);
      atomicOr(&wmask[sb], 1u << lane);
    }
    __syncwarp();
    for (uint32_t e = 0; e < cnt; ++e) {
      uint32_t sb, rect;
      sb_entry(g, e, a.sb_cols, sb, rect);
      const uint32_t m = wmask[sb];
      const uint32_t pos = wbase[sb] + __popc(m & lt);
      if (pos < a.sb_start[sb + 1u]) {
        a.sbk_b[pos] = ((unsigned long long)sb << kSbKeyShift) | ((unsigned long long)rect << 24) | rk[k];
      } else {
        atomicOr(a.ctl + kCtlFlags, 0x8u);  // inconsistent counts (a bug): report, do not write
      }
    }
    __syncwarp();
    // the lowest lane of each superblock advances its position (one writer
    // per superblock; the masks are still intact) ...
    for (uint32_t e = 0; e < cnt; ++e) {
      uint32_t sb, rect;
      sb_entry(g, e, a.sb_cols, sb, rect);
      const uint32_t m = wmask[sb];
      if ((m & lt) == 0u) wbase[sb] += __popc(m);
    }
    __syncwarp();
    // ... then every lane clears its superblocks' masks for the next round
    for (uint32_t e = 0; e < cnt; ++e) {
      uint32_t sb, rect;
      sb_entry(g, e, a.sb_cols, sb, rect);
      wmask[sb] = 0u;
    }
    __syncwarp();
  }
}

}  // namespace

uint32_t superblock_list_tiles(uint32_t N) { return (N + kSbTile - 1u) / kSbTile + 1u; }

cudaError_t launch_superblock_lists(const FrameArgs& a, cudaStream_t s) {
  if (!a.N) return cudaSuccess;
  static bool attr = false;
  const size_t count_smem = (size_t)a.num_sb * 4u;
  const size_t emit_smem = (size_t)2u * kSbWarps * a.num_sb * 4u;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_sb_emit, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(2u * kSbWarps * kMaxSuperblocks * 4u));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const uint32_t tiles = (a.N + kSbTile - 1u) / kSbTile;
  k_sb_count<<<tiles, kSbThreads, count_smem, s>>>(a);
  k_sb_offsets<<<a.num_sb + 1u, 256, 0, s>>>(a, tiles);
  k_sb_emit<<<tiles, kSbThreads, emit_smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hdsr
