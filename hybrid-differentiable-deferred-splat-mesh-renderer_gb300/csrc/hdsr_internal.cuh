// hdsr_internal.cuh — device buffer layout of one compositor handle and the
// launchers each translation unit provides.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "hdsr_math.cuh"

namespace hdsr {

// Control block (u32 words) in device memory, one per handle.
enum Ctl : int {
  kCtlEpoch = 0,       // frame counter: decoupled-lookback status words carry it
  kCtlFlags = 1,       // HDSR_DEV_* bits
  kCtlPairsLo = 2,     // P, total (tile, splat) pairs of the frame
  kCtlPairsHi = 3,
  kCtlSplats = 4,      // N, the depth sort's key count (constant per handle)
  kCtlSbPairs = 10,    // Q, (superblock, splat) list entries of the frame
  kCtlSegments = 11,   // 256-entry segments of the superblock lists
  kCtlDepthMin = 12,   // depth sort: least depth bits of a visible splat (starts at 0xFFFFFFFF)
  kCtlDepthMax = 13,   // depth sort: greatest
  kCtlDepthBase = 14,  // depth sort: subtracted from visible keys
  kCtlDepthPasses = 15,// depth sort: 9-bit passes this frame (1-4)
  kCtlHotTiles = 5,
  kCtlChunks = 6,
  kCtlVisible = 7,
  kCtlScanNTile = 8,   // dynamic tile counters of the scans
  kCtlScanMTile = 9,
  kCtlRasterTile = 19, // dynamic tile counter of the rasteriser
  kCtlBwdTile = 20,    // dynamic tile counter of the adjoint rasteriser
  kCtlSortCount = 21,  // key count of the back-to-front sort (hdsr_sort_back_to_front)
  kCtlSortFlags = 22,  // its skip flags (always 0: the sort never skips)
  kCtlScatterItem = 23,// dynamic work counter of the segment scatter
  kCtlOrderFront = 24, // tiles placed at the front of the rasterisers' work order
  kCtlOrderBack = 25,  // tiles placed at its back
  kCtlWords = 64
};

constexpr uint32_t kRadixBits = 8;               // widest digit
constexpr uint32_t kRadixBins = 1u << kRadixBits;
// wide digits: the superblock passes (up to 512 superblocks in one pass)
constexpr uint32_t kRadixWideBits = 9;
constexpr uint32_t kRadixWideBins = 1u << kRadixWideBits;
constexpr uint32_t kDepthPasses = 4;             // 32 depth bits

// Superblocks: squares of 8x8 tiles. A superblock list entry is
// superblock << 36 | local rect << 24 | sortRank, the local rect being the
// splat's tile box clipped to the superblock (3 bits per edge: x0, x1, y0, y1).
constexpr uint32_t kSbShift = 3;
constexpr uint32_t kSbTiles = 64;
constexpr uint32_t kSbKeyShift = 36;
constexpr uint32_t kSegEntries = 256;            // list entries per segment
constexpr uint32_t kChunkEntries = 32;           // list entries per chunk mask
constexpr uint32_t kHeavyTile = 1024;            // entries from which a tile goes first in the work order

// Local rect of a superblock list entry: x0 | x1 << 3 | y0 << 6 | y1 << 9.
HDSR_HD uint32_t local_rect(unsigned long long k) { return (uint32_t)(k >> 24) & 0xFFFu; }

// The superblock tiles a local rect covers: bit y * 8 + x.
HDSR_HD unsigned long long rect_tiles(uint32_t rc) {
  const uint32_t x0 = rc & 7u, x1 = (rc >> 3) & 7u, y0 = (rc >> 6) & 7u, y1 = rc >> 9;
  const unsigned long long row = (unsigned long long)(((2u << x1) - (1u << x0)) & 0xFFu);
  const unsigned long long rows_hi = y1 == 7u ? ~0ull : (1ull << (8u * y1 + 8u)) - 1ull;
  const unsigned long long rows_lo = ~((1ull << (8u * y0)) - 1ull);
  return row * 0x0101010101010101ull & rows_hi & rows_lo;
}
constexpr uint32_t kMaxSuperblocks = 1024;       // 255 tiles a side -> <= 32 x 32

// One LSD radix pass over u64 keys: digit = (key >> shift) & (2^bits - 1).
struct RadixJob {
  const unsigned long long* in;
  unsigned long long* out;          // non-final passes
  uint32_t* out_low;                // final pass: key & low_mask
  unsigned long long* out_keys;     // final pass, optional: the keys themselves
  unsigned long long low_mask;
  const uint32_t* count;            // number of keys (device)
  const uint32_t* flags;            // frame flags: skip the pass on overflow
  uint32_t* tile_digits;            // kRadixWideBins * tiles_cap counts -> offsets
  uint32_t* bin_base;               // kRadixWideBins totals -> bases
  uint32_t tiles_cap;
  uint32_t shift;
  uint32_t bits;
};

// Everything a kernel of the frame needs, passed by value.
struct FrameArgs {
  const float* U;                 // 64-float frame uniform block (device)
  // scene (borrowed)
  const float* pos;
  const float* scl;
  const float* rot;
  const float* opa;
  const uint32_t* mat;
  const float* nrm;
  uint64_t nrm_len;
  const float* sh;
  const uint32_t* sorted;
  uint32_t N;
  uint32_t sh_degree;
  // plan
  uint32_t W, H, cols, rows, M, tile_count;
  uint32_t rank_bits;             // bits of a sortRank (<= 24)
  uint32_t sb_shift;              // superblock side = 1 << sb_shift tiles
  uint32_t sb_cols, sb_rows, num_sb;
  uint32_t sb_bits;               // radix digits of the superblock index
  uint64_t sb_cap;                // capacity of the superblock lists
  uint32_t seg_cap;               // capacity of the segment tables
  uint64_t cap;                   // pair capacity
  uint32_t log_keys;              // compute per-tile depth range + 20-bit keys
  uint32_t composite_f16;         // the f16 composite variant (HDSR_CFG_F16_COMPOSITE)
  // projection cache (SoA) and per-splat data
  float4* geo;                    // centerPx.xy, invCov.xy
  uint4* app;                     // invCov.z bits, f16(radius,opacity), f16 rg, f16 b|0
  uint4* gb;                      // material, oct normal, f16 em rg, f16 em b|0
  uint2* aux;                     // tile box u8x4, f16 normal confidence|0
  uint32_t* depth;                // f32 NDC depth bits
  uint32_t* ntiles;               // tiles touched per sortRank (0 if invisible)
  unsigned long long* dkeys_a;    // depth << 32 | superblock count << 24 | sortRank, per sortRank
  unsigned long long* dkeys_b;
  uint32_t* order;                // sortRanks in ascending (depth, sortRank)
  uint32_t* nsb;                  // superblocks touched per sortRank
  uint32_t* sb_off;               // exclusive prefix of nsb in depth order
  unsigned long long* sbk_a;      // superblock list entries in depth order (see kSbKeyShift)
  unsigned long long* sbk_b;
  const unsigned long long* sbk_sorted;  // sbk_a or sbk_b: the entries stably sorted by superblock
  int* tile_diff;                 // (cols+1) x (rows+1) 2D difference grid of tile counts
  int* sb_diff;                   // (sb_cols+1) x (sb_rows+1) grid of superblock list lengths
  uint32_t* sb_start;             // num_sb + 1: first entry of each superblock's list
  uint32_t* seg_first;            // num_sb + 1: first segment of each superblock's list
  uint32_t* seg_cnt;              // kSbTiles per segment: tile counts, then entry bases
  unsigned long long* chunk_mask; // per 32-entry chunk of sbk_sorted: the local tiles its entries cover
  // tiles
  uint32_t* tile_cnt;
  uint32_t* tile_dmin;
  uint32_t* tile_dmax;
  uint32_t* tile_off;
  uint32_t* tile_order;           // tile_count: ty << 16 | tx, the rasterisers' work order
  uint32_t* tile_cost;            // 2 x tile_count: each half tile's cost in the last raster
  float2* tile_log;               // (logMin, keyScale)
  // entries
  unsigned long long* sorted_keys;  // optional: tile, 20-bit log-depth key, sortRank per entry
  uint32_t* entries;              // per-tile lists (sortRank), written on demand or with HDSR_CFG_TILE_ENTRIES
  // radix scratch (shared by every pass, passes run in stream order)
  uint32_t* tile_digits;
  uint32_t* bin_base;
  uint32_t radix_tiles_cap;
  uint32_t* dsort_hist0;          // depth sort: per-block digit counts -> offsets, bin-major (even passes)
  uint32_t* dsort_hist1;          // (odd passes)
  uint32_t* dsort_total;          // per digit: the pass's total
  uint32_t dsort_tiles_cap;       // blocks of kRadixTile keys (+1)
  unsigned long long* scan_status_n; // per kScanTile-element tile of the N scan
  unsigned long long* scan_status_m;
  uint32_t* ctl;
  uint32_t spin_limit;            // bound of each decoupled-lookback wait (spins of ~100 ns)
  uint32_t withheld_scan_tile;    // test hook: this tile of each scan never posts its status (~0u: none)
  // outputs (borrowed)
  void* out_color;
  uint64_t color_pitch;
  uint32_t color_f32;
  float* out_depth;
  uint64_t depth_pitch;
  uint32_t* out_normal;
  uint64_t normal_pitch;
  uint32_t* out_material;
  uint64_t material_pitch;
  int num_sms;
};

// Adjoint of one frame (hdsr_encode_backward): the frame's own buffers plus
// the incoming image gradient and the outgoing scene gradients.
constexpr uint32_t kG2d = 12;   // per-sortRank screen-space gradient words (9 used)
struct BwdArgs {
  FrameArgs f;
  const float* d_color;           // dL/d(color output), rgba f32 per pixel
  uint64_t d_color_pitch;         // bytes per row
  float4* par;                    // per sortRank, 3 x float4: cx, cy, ia, ib | ic, opacity, r, g | b
  float* g2d;                     // per sortRank: dL/d(cx, cy, ia, ib, ic, opacity, r, g, b)
  float* d_pos;                   // per splat id: N*3
  float* d_lsc;                   // N*3
  float* d_rot;                   // N*4
  float* d_opa;                   // N
  float* d_sh;                    // N*(6 + 3K)
};

// A sortRank read from a list (tile entries, depth order) that must be < N:
// out of range sets HDSR_DEV_BAD_ENTRY and yields 0, so a broken list is
// reported instead of indexing outside the per-splat arrays.
__device__ __forceinline__ uint32_t checked_rank(uint32_t r, uint32_t N, uint32_t* ctl) {
  if (r < N) return r;
  atomicOr(ctl + kCtlFlags, 0x10u);
  return 0u;
}

// The half-tile cull of the rasteriser and of its adjoint.
// Can the entry reach any pixel centre of the rectangle [x0, x1] x [y0, y1]
// with power > -4 and alpha > 1/255? The power, -0.5 ia dx^2 - ib dx dy -
// 0.5 ic dy^2 (d = p - c), is concave: its maximum over the rectangle is 0
// when the centre lies inside, else the best point of one of the four edges
// (each a 1D parabola, vertex clamped to the edge). Conservative: the
// continuous rectangle contains every pixel centre, the alpha limit uses a
// fast log with margin, and the margin grows with the size of the terms, far
// above the rounding of this test or of the rasteriser's own power. The edge
// vertices use approximate reciprocals: a vertex off by a relative d lowers
// that edge's value by at most 0.5 ic (y d)^2 (resp. ia), about 1e-13 of the
// terms, far inside the margin. An entry that fails the test changes no pixel
// of the rectangle (every pixel is invalid for it), so skipping it is exact
// for finite inputs; the rasteriser tests an entry whose G-buffer or emission
// inputs are not finite with opacity 0.99, i.e. by power alone, since the
// reference's zero-weight products of those inputs are NaN at every pixel of
// a quad with power > -4.
__device__ __forceinline__ bool reaches_rect(float cx, float cy, float ia, float ib, float ic, float op, float x0,
                                             float x1, float y0, float y1) {
  const float xa = x0 - cx, xb = x1 - cx, ya = y0 - cy, yb = y1 - cy;
  const float xm = mx(fabsf(xa), fabsf(xb)), ym = mx(fabsf(ya), fabsf(yb));
  const float mag = 0.5f * ia * xm * xm + fabsf(ib) * xm * ym + 0.5f * ic * ym * ym;
  const float margin = 1e-3f + 1e-5f * mag;
  float best;
  if (xa <= 0.0f && xb >= 0.0f && ya <= 0.0f && yb >= 0.0f) {
    best = 0.0f;
  } else {
    float e = -3.4e38f;
    const float xs[2] = {xa, xb}, ys[2] = {ya, yb};
    const float ric = __fdividef(1.0f, ic), ria = __fdividef(1.0f, ia);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const float x = xs[k];
      const float dy = clampf(-ib * x * ric, ya, yb);
      e = mx(e, -0.5f * ia * x * x - ib * x * dy - 0.5f * ic * dy * dy);
      const float y = ys[k];
      const float dx = clampf(-ib * y * ria, xa, xb);
      e = mx(e, -0.5f * ia * dx * dx - ib * dx * y - 0.5f * ic * y * y);
    }
    best = e;
  }
  // alpha = min(0.99, op exp(power)) > 1/255 needs power > -log(255 op)
  const float lim = mx(-4.0f, -__logf(255.0f * op));
  return best > lim - margin - 1e-3f;
}

// One tile's entries, in order, read from its superblock's list (ascending
// (depth bits, sortRank)): the entries whose local rect covers the tile, the
// same sequence a per-tile list holds. Warp-collective: every lane calls
// every method. Only the list's 32-entry chunks whose mask holds the tile are
// read (mask windows of 32 chunks, one ballot each), kWalkFill chunks per
// fill with their keys loaded together, and the covering entries' sortRanks
// are appended in order to a per-warp ring of kWalkQueue words.
constexpr uint32_t kWalkQueue = 256;
#ifndef HDSR_RASTER_FILL
#define HDSR_RASTER_FILL 4
#endif
constexpr uint32_t kWalkFill = HDSR_RASTER_FILL;
constexpr uint32_t kNoChunk = 0xFFFFFFFFu;
constexpr unsigned long long kNoKey = 7ull << 24;  // a rect that covers no tile (x0 = 7 > x1 = 0)

__device__ __forceinline__ bool rect_covers(unsigned long long k, uint32_t lx, uint32_t ly) {
  const uint32_t rc = local_rect(k);
  return lx >= (rc & 7u) && lx <= ((rc >> 3) & 7u) && ly >= ((rc >> 6) & 7u) && ly <= (rc >> 9);
}

struct TileWalk {
  uint32_t* queue;
  uint32_t beg, end, clast, wnext, wbase, want, head, tail, lx, ly, tbit;
  bool more;

  __device__ __forceinline__ void start(const FrameArgs& a, uint32_t tx, uint32_t ty, uint32_t* q) {
    const uint32_t sb = (ty >> kSbShift) * a.sb_cols + (tx >> kSbShift);
    queue = q;
    beg = a.sb_start[sb];
    end = a.sb_start[sb + 1u];
    lx = tx & 7u;
    ly = ty & 7u;
    tbit = ly * 8u + lx;
    clast = beg < end ? (end - 1u) / kChunkEntries : 0u;
    wnext = beg / kChunkEntries;
    wbase = want = head = tail = 0u;
    more = beg < end;
  }
  // the next chunk (ascending) whose mask holds the tile, or kNoChunk
  __device__ __forceinline__ uint32_t next_chunk(const FrameArgs& a, uint32_t lane) {
    while (want == 0u) {
      if (wnext > clast) return kNoChunk;
      const uint32_t c = wnext + lane;
      const bool has = c <= clast && ((__ldg(a.chunk_mask + c) >> tbit) & 1ull) != 0ull;
      want = __ballot_sync(0xFFFFFFFFu, has);
      wbase = wnext;
      wnext += 32u;
    }
    const uint32_t c = wbase + (uint32_t)(__ffs(want) - 1);
    want &= want - 1u;
    return c;
  }
  // append the covering entries of up to kWalkFill chunks, in order
  __device__ __forceinline__ void fill(const FrameArgs& a, uint32_t lane) {
    unsigned long long k[kWalkFill];
#pragma unroll
    for (uint32_t j = 0; j < kWalkFill; ++j) {
      const uint32_t c = more ? next_chunk(a, lane) : kNoChunk;
      more = c != kNoChunk;
      const uint32_t i = c * kChunkEntries + lane;
      k[j] = more && i >= beg && i < end ? __ldg(a.sbk_sorted + i) : kNoKey;
    }
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (uint32_t j = 0; j < kWalkFill; ++j) {
      const bool in = rect_covers(k[j], lx, ly);
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, in);
      if (in) queue[(tail + __popc(m & lt)) & (kWalkQueue - 1u)] = (uint32_t)k[j] & 0xFFFFFFu;
      tail += __popc(m);
    }
    __syncwarp();
  }
  // the next batch: up to `limit` (<= 32) entries; lane i gets entry i's
  // sortRank (checked against N) when i < the returned count
  __device__ __forceinline__ uint32_t take(const FrameArgs& a, uint32_t lane, uint32_t limit, uint32_t& rank) {
    while (more && tail - head < limit) fill(a, lane);
    const uint32_t n = tail - head < limit ? tail - head : limit;
    if (lane < n) rank = checked_rank(queue[(head + lane) & (kWalkQueue - 1u)], a.N, a.ctl);
    head += n;
    return n;
  }
};

// Default bound of a decoupled-lookback wait (iterations of ~100 ns);
// a handle can lower it (hdsr_set_scan_wait).
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr uint32_t kNoWithheldTile = 0xFFFFFFFFu;

// Frame flags after which the frame's later kernels return at once:
// overflow (0x1, the lists do not fit) and timeout (0x2, a scan wait gave up
// and its offsets are not trustworthy).
constexpr uint32_t kSkipFlags = 0x3u;

// Does the frame skip its remaining kernels (a kSkipFlags bit in *flags)?
// Read once per block and shared, so that every thread of the block takes the
// same branch even when a kernel of the other stream (tile counts and the
// tile scan run beside the depth sort and the superblock lists) sets a flag
// meanwhile. A flag one kernel has seen, every later kernel of its stream
// sees, so a kernel that runs reads only what earlier kernels wrote in full.
__device__ __forceinline__ bool block_skipped(const uint32_t* flags, uint32_t* s_flag) {
  if (threadIdx.x == 0) *s_flag = *reinterpret_cast<volatile const uint32_t*>(flags) & kSkipFlags;
  __syncthreads();
  return *s_flag != 0u;
}

// Lookback status word: epoch (30 bits) | flag (2 bits) | value (32 bits).
constexpr unsigned long long kFlagAgg = 1ull;
constexpr unsigned long long kFlagInc = 2ull;
HDSR_HD unsigned long long make_status(uint32_t epoch, unsigned long long flag, uint32_t v) {
  return ((unsigned long long)(epoch & 0x3FFFFFFFu) << 34) | (flag << 32) | v;
}

// Programmatic dependent launch (sm_90 and later). A kernel launched with
// launch_pdl may be scheduled while the previous kernel of its stream is
// still running; it calls pdl_wait() before touching any memory, which
// returns once that kernel has completed and its writes are visible, so the
// order of effects is that of a plain launch and only the launch latency
// overlaps. pdl_trigger() lets the next such kernel be scheduled early (it
// then waits in its own pdl_wait). Without the launch attribute both are
// no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// launchers (each returns cudaGetLastError() of its launches)
cudaError_t launch_frame_init(const FrameArgs& a, cudaStream_t s);
cudaError_t launch_project(const FrameArgs& a, cudaStream_t s);
cudaError_t launch_tile_counts(const FrameArgs& a, cudaStream_t s);   // 2 launches
cudaError_t launch_depth_range(const FrameArgs& a, cudaStream_t s);
cudaError_t launch_scan_sb(const FrameArgs& a, cudaStream_t s);
cudaError_t launch_scan_tiles(const FrameArgs& a, cudaStream_t s);
cudaError_t launch_tile_entries(const FrameArgs& a, cudaStream_t s);  // 3 launches
cudaError_t launch_chunk_masks(const FrameArgs& a, cudaStream_t s);   // 1 launch
// one stable pass over j.bits digit bits (8: 256 bins; 9: 512 bins), 3 launches
cudaError_t launch_radix_pass(const RadixJob& j, bool last, int num_sms, cudaStream_t s);
// the frame's depth sort (hdsr_dsort.cu): a.dkeys_a -> a.order, 9 launches
cudaError_t launch_depth_sort(const FrameArgs& a, cudaStream_t s);
uint32_t depth_sort_tiles(uint32_t N);  // blocks of its tables (dsort_tiles_cap)
uint32_t depth_sort_bins();             // digits of a pass
cudaError_t launch_log_depth_keys(const FrameArgs& a, cudaStream_t s);
// back-to-front order of the bound positions for a view matrix (row 2 of the
// view transform: view[2], view[6], view[10], view[14]) into `out`
cudaError_t launch_sort_back_to_front(const FrameArgs& a, const double vrow[4], uint32_t* out, cudaStream_t s);
// the rasteriser's work order from the last raster's per-tile costs, most
// expensive first (1 launch; leaves the tile scan's order when there are none)
cudaError_t launch_work_order(const FrameArgs& a, cudaStream_t s);
cudaError_t launch_raster(const FrameArgs& a, cudaStream_t s);
cudaError_t launch_backward(const BwdArgs& b, cudaStream_t s);  // 3 launches
cudaError_t launch_bwd_prep(const BwdArgs& b, cudaStream_t s);  // hdsr_backward_prep.cu

// internal entry points of one compositor handle for the serving loop
// (hdsr_api.cu); C++ linkage, not part of the C ABI
}  // namespace hdsr
struct hdsr_compositor;
namespace hdsr {
uint64_t handle_device_bytes(const hdsr_compositor* h);
const FrameArgs* handle_args(const hdsr_compositor* h);
int handle_frame_checks(hdsr_compositor* h);                       // hdsr_status
int handle_upload_uniforms(hdsr_compositor* h, const float* pinned_uniforms, cudaStream_t s);
int handle_encode_pre_raster(hdsr_compositor* h, cudaStream_t s);  // capturable
int handle_encode_raster(hdsr_compositor* h, cudaStream_t s);

// sizing helpers shared with the API
#ifndef HDSR_SCAN_ITEMS
#define HDSR_SCAN_ITEMS 8
#endif
constexpr uint32_t kScanItems = HDSR_SCAN_ITEMS;
constexpr uint32_t kScanThreads = 256;
constexpr uint32_t kScanTile = kScanItems * kScanThreads;
constexpr uint32_t kRadixThreads = 256;
#ifndef HDSR_RADIX_ITEMS
#define HDSR_RADIX_ITEMS 10
#endif
constexpr uint32_t kRadixItems = HDSR_RADIX_ITEMS;
constexpr uint32_t kRadixTile = kRadixThreads * kRadixItems;

}  // namespace hdsr
