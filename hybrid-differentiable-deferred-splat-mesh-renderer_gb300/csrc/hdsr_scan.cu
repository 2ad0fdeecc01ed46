// hdsr_scan.cu — single-pass exclusive scans with decoupled lookback.
//
// Replaces the reference's three-pass Hillis-Steele scan (scan,
// scan_block_sums, add_block_sums in gpu_prefix_sum.wgsl:14-85, driven by
// gpuTileSplatCompositor.ts:1063-1088) with one launch per array:
//   - per-splat superblock counts, taken in ascending (depth, sortRank)
//     order from bits 24-31 of the depth-order words (N) -> each splat's
//     superblock list entries written at its offset, and Q, their total;
//   - per-tile counts (M) -> tile offsets (bit-identical to the reference's
//     tileOffsets), the hot-tile statistics of classify_tiles
//     (gpu_tile_classify.wgsl:44-86) and, when requested, the per-tile
//     log-depth parameters of the 20-bit keys.
// Tiles of kScanTile (2048) elements are claimed through an atomic counter, so a tile
// only waits on tiles already claimed by running blocks; every wait is
// bounded and sets HDSR_DEV_TIMEOUT when it gives up.
#include "hdsr_internal.cuh"

namespace hdsr {

namespace {

__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}
__device__ __forceinline__ void st_volatile(unsigned long long* p, unsigned long long v) {
  *reinterpret_cast<volatile unsigned long long*>(p) = v;
}

// Exclusive prefix of all tiles before `tile`, walking back through their
// status words 32 at a time (warp-collective): lane l reads tile
// base - l, waiting (bounded) until it is posted; the nearest inclusive
// prefix in the window ends the walk, else the 32 aggregates are added and
// the window moves back. Positions before tile 0 count as an inclusive 0.
__device__ uint32_t lookback(unsigned long long* status, uint32_t tile, uint32_t epoch, uint32_t* ctl,
                             uint32_t lane, uint32_t spin_limit) {
  uint32_t prefix = 0;
  for (int base = (int)tile - 1;; base -= 32) {
    const int t = base - (int)lane;
    unsigned long long st = make_status(epoch, kFlagInc, 0u);
    if (t >= 0) {
      uint32_t spins = 0;
      for (;;) {
        st = ld_volatile(status + t);
        if ((uint32_t)(st >> 34) == (epoch & 0x3FFFFFFFu) && ((st >> 32) & 3ull) != 0ull) break;
        if (++spins > spin_limit) {
          atomicOr(ctl + kCtlFlags, 0x2u);
          st = make_status(epoch, kFlagInc, 0u);
          break;
        }
        __nanosleep(64);
      }
    }
    const uint32_t inc = __ballot_sync(0xFFFFFFFFu, ((st >> 32) & 3ull) == kFlagInc);
    const uint32_t first = inc ? (uint32_t)(__ffs(inc) - 1) : 32u;
    uint32_t v = lane <= first ? (uint32_t)st : 0u;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    prefix += v;
    if (inc) break;
  }
  return prefix;
}

// Superblock lists: splat i of the depth order writes one entry per
// superblock its tile box touches, superblock << 36 | local rect << 24 |
// sortRank, starting at its exclusive prefix o of the counts in depth order.
__device__ __forceinline__ void emit_superblock_entries(const FrameArgs& a, uint32_t r, uint32_t box, uint32_t o) {
  if (box == kSentinel) return;
  const uint32_t x0 = box & 0xFFu, y0 = (box >> 8) & 0xFFu, x1 = (box >> 16) & 0xFFu, y1 = box >> 24;
  for (uint32_t sy = y0 >> kSbShift; sy <= y1 >> kSbShift; ++sy) {
    const uint32_t by = sy << kSbShift;
    const uint32_t ly0 = y0 > by ? y0 - by : 0u, ly1 = y1 - by < 7u ? y1 - by : 7u;
    for (uint32_t sx = x0 >> kSbShift; sx <= x1 >> kSbShift; ++sx) {
      const uint32_t bx = sx << kSbShift;
      const uint32_t lx0 = x0 > bx ? x0 - bx : 0u, lx1 = x1 - bx < 7u ? x1 - bx : 7u;
      const uint32_t rect = lx0 | (lx1 << 3) | (ly0 << 6) | (ly1 << 9);
      if (o < a.sb_cap)
        a.sbk_a[o] = ((unsigned long long)(sy * a.sb_cols + sx) << kSbKeyShift) | ((unsigned long long)rect << 24) | r;
      ++o;
    }
  }
}

// Scan of the superblock counts in depth order (read from bits 24-31 of the
// depth-order words), emitting every splat's list entries at its offset.
struct SbScan {
  // an overflowed frame may have skipped the depth sort: order then holds no
  // permutation
  static constexpr bool kMaySkip = true;
  static __device__ uint32_t size(const FrameArgs& a) { return a.N; }
  static __device__ uint32_t counter() { return kCtlScanNTile; }
  static __device__ unsigned long long* status(const FrameArgs& a) { return a.scan_status_n; }
  static __device__ uint32_t load(const FrameArgs& a, uint32_t i) { return a.order[i] >> 24; }
  // what store needs, loaded for all of a thread's items before any store
  struct Pre {
    uint32_t r, box;
  };
  static __device__ Pre pre(const FrameArgs& a, uint32_t i) {
    const uint32_t r = checked_rank(a.order[i] & 0xFFFFFFu, a.N, a.ctl);
    return Pre{r, a.aux[r].x};
  }
  static __device__ void store(const FrameArgs& a, uint32_t i, uint32_t excl, const Pre& p) {
    a.sb_off[i] = excl;
    emit_superblock_entries(a, p.r, p.box, excl);
  }
  // the lists' own capacity check (tile counts, on the other stream, make the
  // same one): the radix pass reads no entry past the buffers
  static __device__ void finish(const FrameArgs& a, uint32_t total) {
    if (total > a.sb_cap) atomicOr(a.ctl + kCtlFlags, 0x1u);
    a.ctl[kCtlSbPairs] = total < a.sb_cap ? total : (uint32_t)a.sb_cap;
  }
};

struct TileScan {
  static constexpr bool kMaySkip = false;  // it decides the overflow
  static __device__ uint32_t size(const FrameArgs& a) { return a.M; }
  static __device__ uint32_t counter() { return kCtlScanMTile; }
  static __device__ unsigned long long* status(const FrameArgs& a) { return a.scan_status_m; }
  static __device__ uint32_t load(const FrameArgs& a, uint32_t i) { return a.tile_cnt[i]; }
  using Pre = uint32_t;
  static __device__ Pre pre(const FrameArgs& a, uint32_t i) { return a.tile_cnt[i]; }
  static __device__ void store(const FrameArgs& a, uint32_t i, uint32_t excl, const Pre& c) {
    a.tile_off[i] = excl;
    // work order of the rasterisers: tiles of >= kHeavyTile entries first
    // (the slow ones start early), the rest from the back; the order decides
    // only which warp takes a tile when, never a pixel. One atomic per warp
    // and end (the calling lanes may be a partial warp).
    const uint32_t tx = morton_even(i), ty = morton_even(i >> 1);
    const bool in_grid = tx < a.cols && ty < a.rows, heavy = in_grid && c >= kHeavyTile;
    const uint32_t act = __activemask(), lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    const uint32_t mh = __ballot_sync(act, heavy), ml = __ballot_sync(act, in_grid && !heavy);
    const uint32_t leader = (uint32_t)(__ffs(act) - 1);
    uint32_t bh = 0u, bl = 0u;
    if (lane == leader) {
      if (mh) bh = atomicAdd(a.ctl + kCtlOrderFront, (uint32_t)__popc(mh));
      if (ml) bl = atomicAdd(a.ctl + kCtlOrderBack, (uint32_t)__popc(ml));
    }
    bh = __shfl_sync(act, bh, leader);
    bl = __shfl_sync(act, bl, leader);
    if (heavy) a.tile_order[bh + __popc(mh & lt)] = ty << 16 | tx;
    else if (in_grid) a.tile_order[a.tile_count - 1u - (bl + __popc(ml & lt))] = ty << 16 | tx;
    if (c == 0u) return;
    if (a.log_keys) a.tile_log[i] = tile_log_params(a.tile_dmin[i], a.tile_dmax[i]);
    if (c > kMaxTileEntries) {
      // hot tile: the reference's bucket cascade splits it into 4096-entry
      // chunks (gpu_tile_bucket_sort.wgsl:110-143)
      atomicAdd(a.ctl + kCtlHotTiles, 1u);
      atomicAdd(a.ctl + kCtlChunks, (c + kMaxTileEntries - 1u) / kMaxTileEntries);
    }
  }
  static __device__ void finish(const FrameArgs& a, uint32_t total) {
    a.ctl[kCtlPairsLo] = total;
    a.ctl[kCtlPairsHi] = 0u;
    if ((uint64_t)total > a.cap) atomicOr(a.ctl + kCtlFlags, 0x1u);
  }
};

template <class Policy>
__global__ void __launch_bounds__(kScanThreads) k_scan(FrameArgs a) {
  constexpr uint32_t PAD = kScanTile / 32;
  __shared__ uint32_t s_data[kScanTile + PAD];
  __shared__ uint32_t s_warp[kScanThreads / 32];
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_prefix;
  __shared__ uint32_t s_skip;
  // the superblock scan is a programmatic dependent launch after the depth
  // sort (a no-op for the tile scan's plain launch)
  pdl_wait();
  pdl_trigger();
  if (Policy::kMaySkip && block_skipped(a.ctl + kCtlFlags, &s_skip)) return;
  const uint32_t n = Policy::size(a);
  const uint32_t num_tiles = (n + kScanTile - 1) / kScanTile;
  const uint32_t epoch = a.ctl[kCtlEpoch];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  unsigned long long* status = Policy::status(a);
  for (;;) {
    if (tid == 0) s_tile = atomicAdd(a.ctl + Policy::counter(), 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= num_tiles) break;
    const uint32_t base = tile * kScanTile;
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
      uint32_t i = k * kScanThreads + tid;
      uint32_t g = base + i;
      s_data[i + i / 32] = g < n ? Policy::load(a, g) : 0u;
    }
    __syncthreads();
    uint32_t vals[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
      uint32_t i = tid * kScanItems + k;
      vals[k] = s_data[i + i / 32];
      sum += vals[k];
    }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t v = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += v;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = lane < kScanThreads / 32 ? s_warp[lane] : 0u;
      uint32_t wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xFFFFFFFFu, wi, o);
        if (lane >= (uint32_t)o) wi += v;
      }
      if (lane < kScanThreads / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
      const uint32_t total = __shfl_sync(0xFFFFFFFFu, wi, kScanThreads / 32 - 1);
      uint32_t prefix = 0u;
      // a withheld tile (test hook) computes its prefix but posts nothing:
      // its successors' waits run out and flag the frame
      const bool post = tile != a.withheld_scan_tile;
      if (tile == 0) {
        if (lane == 0 && post) st_volatile(status + tile, make_status(epoch, kFlagInc, total));
      } else {
        if (lane == 0 && post) st_volatile(status + tile, make_status(epoch, kFlagAgg, total));
        prefix = lookback(status, tile, epoch, a.ctl, lane, a.spin_limit);
        if (lane == 0 && post) st_volatile(status + tile, make_status(epoch, kFlagInc, prefix + total));
      }
      if (lane == 0) {
        s_prefix = prefix;
        if (tile == num_tiles - 1) Policy::finish(a, prefix + total);
      }
    }
    __syncthreads();
    uint32_t running = s_prefix + s_warp[warp] + (inc - sum);
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
      uint32_t i = tid * kScanItems + k;
      s_data[i + i / 32] = running;
      running += vals[k];
    }
    __syncthreads();
    // the stores' inputs for all items first (independent loads in flight
    // together), then the stores
    typename Policy::Pre pre[kScanItems];
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
      const uint32_t g = base + k * kScanThreads + tid;
      if (g < n) pre[k] = Policy::pre(a, g);
    }
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
      uint32_t i = k * kScanThreads + tid;
      uint32_t g = base + i;
      if (g < n) Policy::store(a, g, s_data[i + i / 32], pre[k]);
    }
    __syncthreads();
  }
}

int scan_grid(const FrameArgs& a, uint32_t n) {
  uint32_t tiles = (n + kScanTile - 1) / kScanTile;
  uint32_t cap = (uint32_t)a.num_sms * 4u;
  return (int)(tiles < cap ? (tiles ? tiles : 1u) : cap);
}

}  // namespace

cudaError_t launch_scan_sb(const FrameArgs& a, cudaStream_t s) {
  const cudaError_t e = launch_pdl(k_scan<SbScan>, dim3(scan_grid(a, a.N)), dim3(kScanThreads), 0, s, a);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_scan_tiles(const FrameArgs& a, cudaStream_t s) {
  k_scan<TileScan><<<scan_grid(a, a.M), kScanThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hdsr
