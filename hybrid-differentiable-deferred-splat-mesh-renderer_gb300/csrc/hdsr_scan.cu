// hdsr_scan.cu — single-pass exclusive scans with decoupled lookback.
//
// Replaces the reference's three-pass Hillis-Steele scan (scan,
// scan_block_sums, add_block_sums in gpu_prefix_sum.wgsl:169-240, driven by
// gpuTileSplatCompositor.ts:1063-1088) with one launch per array:
//   - per-splat superblock counts, taken in ascending (depth, sortRank)
//     order from bits 24-31 of the depth-order words (N) -> each splat's
//     superblock list entries written at its offset, and Q, their total;
//   - per-tile counts (M) -> tile offsets (bit-identical to the reference's
//     tileOffsets), the hot-tile statistics of classify_tiles
//     (gpu_tile_classify.wgsl:44-86) and, when requested, the per-tile
//     log-depth parameters of the 20-bit keys.
// Tiles of 4096 elements are claimed through an atomic counter, so a tile
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
// status words (single thread).
__device__ uint32_t lookback(unsigned long long* status, uint32_t tile, uint32_t epoch, uint32_t* ctl) {
  uint32_t prefix = 0;
  int t = (int)tile - 1;
  while (t >= 0) {
    unsigned long long st;
    uint32_t spins = 0;
    for (;;) {
      st = ld_volatile(status + t);
      if ((uint32_t)(st >> 34) == (epoch & 0x3FFFFFFFu) && ((st >> 32) & 3ull) != 0ull) break;
      if (++spins > kSpinLimit) {
        atomicOr(ctl + kCtlFlags, 0x2u);
        st = make_status(epoch, kFlagInc, 0u);
        break;
      }
      __nanosleep(64);
    }
    prefix += (uint32_t)st;
    if (((st >> 32) & 3ull) == kFlagInc) break;
    --t;
  }
  return prefix;
}

// Superblock lists: splat i of the depth order writes one entry per
// superblock its tile box touches, superblock << 36 | local rect << 24 |
// sortRank, starting at its exclusive prefix o of the counts in depth order.
__device__ __forceinline__ void emit_superblock_entries(const FrameArgs& a, uint32_t r, uint32_t o) {
  const uint32_t box = a.aux[r].x;
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
  // an overflowed frame skipped the depth sort: order holds no permutation
  static __device__ bool skip(const FrameArgs& a) { return (a.ctl[kCtlFlags] & 0x1u) != 0u; }
  static __device__ uint32_t size(const FrameArgs& a) { return a.N; }
  static __device__ uint32_t counter() { return kCtlScanNTile; }
  static __device__ unsigned long long* status(const FrameArgs& a) { return a.scan_status_n; }
  static __device__ uint32_t load(const FrameArgs& a, uint32_t i) { return a.order[i] >> 24; }
  static __device__ void store(const FrameArgs& a, uint32_t i, uint32_t excl) {
    a.sb_off[i] = excl;
    emit_superblock_entries(a, checked_rank(a.order[i] & 0xFFFFFFu, a.N, a.ctl), excl);
  }
  static __device__ void finish(const FrameArgs& a, uint32_t total) { a.ctl[kCtlSbPairs] = total; }
};

struct TileScan {
  static __device__ bool skip(const FrameArgs&) { return false; }  // it decides the overflow
  static __device__ uint32_t size(const FrameArgs& a) { return a.M; }
  static __device__ uint32_t counter() { return kCtlScanMTile; }
  static __device__ unsigned long long* status(const FrameArgs& a) { return a.scan_status_m; }
  static __device__ uint32_t load(const FrameArgs& a, uint32_t i) { return a.tile_cnt[i]; }
  static __device__ void store(const FrameArgs& a, uint32_t i, uint32_t excl) {
    a.tile_off[i] = excl;
    const uint32_t c = a.tile_cnt[i];
    // work order of the rasterisers: tiles of >= kHeavyTile entries first
    // (the slow ones start early), the rest from the back; the order decides
    // only which warp takes a tile when, never a pixel
    const uint32_t tx = morton_even(i), ty = morton_even(i >> 1);
    if (tx < a.cols && ty < a.rows) {
      const uint32_t packed = ty << 16 | tx;
      if (c >= kHeavyTile) a.tile_order[atomicAdd(a.ctl + kCtlOrderFront, 1u)] = packed;
      else a.tile_order[a.tile_count - 1u - atomicAdd(a.ctl + kCtlOrderBack, 1u)] = packed;
    }
    if (c == 0u) return;
    if (a.log_keys) a.tile_log[i] = tile_log_params(a.tile_dmin[i], a.tile_dmax[i]);
    if (c > kMaxTileEntries) {
      // hot tile: the reference's bucket cascade splits it into 4096-entry
      // chunks (gpu_tile_bucket_sort.wgsl:276-307)
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
  if (Policy::skip(a)) return;
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
      if (lane == kScanThreads / 32 - 1) {
        const uint32_t total = wi;
        if (tile == 0) {
          st_volatile(status + tile, make_status(epoch, kFlagInc, total));
          s_prefix = 0u;
        } else {
          st_volatile(status + tile, make_status(epoch, kFlagAgg, total));
          uint32_t prefix = lookback(status, tile, epoch, a.ctl);
          st_volatile(status + tile, make_status(epoch, kFlagInc, prefix + total));
          s_prefix = prefix;
        }
        if (tile == num_tiles - 1) Policy::finish(a, s_prefix + total);
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
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
      uint32_t i = k * kScanThreads + tid;
      uint32_t g = base + i;
      if (g < n) Policy::store(a, g, s_data[i + i / 32]);
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
  k_scan<SbScan><<<scan_grid(a, a.N), kScanThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_scan_tiles(const FrameArgs& a, cudaStream_t s) {
  k_scan<TileScan><<<scan_grid(a, a.M), kScanThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hdsr
