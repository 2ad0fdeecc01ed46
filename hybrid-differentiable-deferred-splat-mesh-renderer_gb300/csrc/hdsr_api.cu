// hdsr_api.cu — the C ABI declared in include/hdsr.h.
//
// Host-side mirror of the reference operator API in
// src/gpuTileSplatCompositor.ts: plan (:109-139), create (:141-728), bind
// (:792-995), frame uniforms (:730-774), encode full (:1023-1179) and
// composite-only (:1001-1014), destroy. The handle owns every internal
// device buffer; scene and output buffers are borrowed.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/hdsr.h"
#include "hdsr_internal.cuh"

using namespace hdsr;

namespace {
constexpr uint32_t kMaxProfiledPasses = 24;
// names of the profiled passes, indexed by the ids recorded in encode()
const char* const kPassNames[] = {"upload_uniforms", "frame_init", "project", "tile_counts", "unused_4",
                                  "scan_tiles", "depth_sort", "superblock_lists", "tile_entries", "chunk_masks",
                                  "unused_10", "unused_11", "unused_12", "unused_13", "unused_14",
                                  "unused_15", "unused_16", "raster"};
constexpr uint32_t kNumPassNames = sizeof(kPassNames) / sizeof(kPassNames[0]);
}  // namespace

struct hdsr_compositor {
  hdsr_plan plan{};
  hdsr_config cfg{};
  int device = 0;
  FrameArgs args{};
  float4* bwd_par = nullptr;      // adjoint buffers (HDSR_CFG_BACKWARD)
  uint64_t device_bytes = 0;      // sum of this handle's device allocations
  float* bwd_g2d = nullptr;
  std::vector<void*> allocs;
  float uniforms[64] = {};
  bool have_uniforms = false;
  bool scene_bound = false;
  bool outputs_bound = false;
  bool sorted_valid = false;
  bool entries_valid = false;      // a.entries holds the last full frame's per-tile lists
  bool cost_stale = true;          // a.tile_cost holds no raster of the bound scene: cleared by the next frame
  float cost_view[3] = {0.0f, 0.0f, 0.0f};  // view direction of the frame whose costs a.tile_cost holds
  bool cost_view_valid = false;
  cudaStream_t last_stream = nullptr;
  bool has_last_stream = false;
  uint64_t launches = 0;           // kernels queued by this handle
  bool profiling = false;
  cudaEvent_t ev[kMaxProfiledPasses + 1] = {};
  // uniform upload: a ring of pinned staging slots (an async copy from
  // pageable memory may synchronise the stream), each reused only after its
  // copy has run; no upload when the block equals the device's copy
  static constexpr uint32_t kUniformSlots = 8;
  float* pinned_u = nullptr;
  cudaEvent_t ev_u[kUniformSlots] = {};
  bool ev_u_pending[kUniformSlots] = {};
  uint32_t next_u = 0;
  float device_u[64] = {};
  bool device_u_valid = false;
  // second stream of a frame: tile counts, the tile scan and the work order
  // run there, forked after projection and joined before the rasteriser,
  // beside the depth sort and the superblock lists (none when profiling:
  // per-pass times need one stream)
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  uint32_t ev_used = 0;
  uint32_t pass_id[kMaxProfiledPasses] = {};
  // a full frame's kernels as one CUDA graph: captured on the second full
  // frame after a bind (the first runs directly) and replayed until the next
  // bind or profiling change; replays launch the same kernels with the same
  // arguments, which read the uniforms from device memory
  cudaGraphExec_t frame_graph = nullptr;
  uint64_t graph_launches = 0;    // kernels of one replay
  uint32_t direct_frames = 0;     // full frames launched directly since the last bind
  bool graph_failed = false;      // capture failed: launch directly until the next bind
  char err[256] = {0};
};

namespace {

char g_null_err[] = "null handle";

hdsr_status fail(hdsr_compositor* h, hdsr_status s, const char* msg) {
  if (h) std::snprintf(h->err, sizeof(h->err), "%s", msg);
  return s;
}

hdsr_status cuda_fail(hdsr_compositor* h, cudaError_t e, const char* where) {
  if (h) std::snprintf(h->err, sizeof(h->err), "%s: %s", where, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? HDSR_ERR_OOM : HDSR_ERR_CUDA;
}

uint32_t ceil_log2(uint64_t v) {
  uint32_t b = 0;
  while ((1ull << b) < v) ++b;
  return b;
}

template <class T>
hdsr_status dev_alloc(hdsr_compositor* h, T** p, uint64_t count, const char* what) {
  uint64_t bytes = count * sizeof(T);
  if (bytes == 0) bytes = 16;
  void* ptr = nullptr;
  cudaError_t e = cudaMalloc(&ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    char msg[128];
    std::snprintf(msg, sizeof(msg), "cudaMalloc %s (%llu bytes)", what, (unsigned long long)bytes);
    return cuda_fail(h, e, msg);
  }
  h->allocs.push_back(ptr);
  h->device_bytes += bytes;
  *p = static_cast<T*>(ptr);
  return HDSR_OK;
}

// The frame graph no longer matches the handle's arguments (or is not wanted).
void drop_graph(hdsr_compositor* h) {
  if (h->frame_graph) cudaGraphExecDestroy(h->frame_graph);
  h->frame_graph = nullptr;
  h->direct_frames = 0;
  h->graph_failed = false;
}

void free_all(hdsr_compositor* h) {
  for (void* p : h->allocs) cudaFree(p);
  h->allocs.clear();
  h->device_bytes = 0;
}

}  // namespace

extern "C" {

uint32_t hdsr_abi_version(void) { return HDSR_ABI_VERSION; }

hdsr_status hdsr_plan_tile_splat_compositor(const hdsr_plan_input* in, hdsr_plan* out) {
  if (!in || !out) return HDSR_ERR_INVALID_ARG;
  if (in->viewport_width == 0 || in->viewport_height == 0 || in->tile_size_px == 0) return HDSR_ERR_INVALID_ARG;
  const uint32_t t = in->tile_size_px;
  out->viewport_width = in->viewport_width;
  out->viewport_height = in->viewport_height;
  out->tile_size_px = t;
  out->tile_columns = (in->viewport_width + t - 1) / t;
  out->tile_rows = (in->viewport_height + t - 1) / t;
  out->tile_count = out->tile_columns * out->tile_rows;
  out->morton_tile_count = morton(out->tile_columns - 1, out->tile_rows - 1) + 1;
  out->splat_count = in->splat_count;
  const double mult = in->tile_entry_multiplier > 0.0 ? in->tile_entry_multiplier : 16.0;
  const double want = std::ceil((double)in->splat_count * mult);
  const double cap = 65535.0 * 256.0;
  out->max_total_tile_refs = (uint32_t)(want < cap ? want : cap);
  return HDSR_OK;
}

hdsr_status hdsr_create_tile_splat_compositor(const hdsr_plan* plan, const hdsr_config* cfg,
                                              hdsr_compositor** out) {
  if (!plan || !out) return HDSR_ERR_INVALID_ARG;
  *out = nullptr;
  if (plan->tile_size_px != kTilePx) return HDSR_ERR_UNSUPPORTED;
  if (plan->tile_columns == 0 || plan->tile_rows == 0 || plan->tile_columns > 255 || plan->tile_rows > 255)
    return HDSR_ERR_UNSUPPORTED;  // the u8x4 tile box packs <= 255 tiles per axis
  hdsr_compositor* h = new (std::nothrow) hdsr_compositor();
  if (!h) return HDSR_ERR_OOM;
  h->plan = *plan;
  if (cfg) h->cfg = *cfg;
  if (h->cfg.color_format > HDSR_COLOR_RGBA32F) { delete h; return HDSR_ERR_INVALID_ARG; }
  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) { hdsr_status s = cuda_fail(h, e, "cudaGetDevice"); delete h; return s; }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  const uint32_t N = plan->splat_count, M = plan->morton_tile_count;
  uint64_t cap = h->cfg.pair_capacity;
  if (cap == 0) {
    uint64_t want = (uint64_t)std::ceil((double)N * 16.0);
    cap = want > plan->max_total_tile_refs ? want : plan->max_total_tile_refs;
  }
  if (cap < 16) cap = 16;
  if (cap >= (1ull << 32)) { delete h; return HDSR_ERR_UNSUPPORTED; }
  h->cfg.pair_capacity = cap;
  FrameArgs& a = h->args;
  a.N = N;
  a.W = plan->viewport_width;
  a.H = plan->viewport_height;
  a.cols = plan->tile_columns;
  a.rows = plan->tile_rows;
  a.M = M;
  a.tile_count = plan->tile_count;
  a.rank_bits = ceil_log2(N > 1 ? N : 2);
  if (a.rank_bits > 24u) { delete h; return HDSR_ERR_UNSUPPORTED; }  // sortRank packs into 24 key bits
  // superblocks of 8x8 tiles (<= 32 x 32 of them)
  a.sb_shift = kSbShift;
  a.sb_cols = (plan->tile_columns + 7u) >> kSbShift;
  a.sb_rows = (plan->tile_rows + 7u) >> kSbShift;
  a.num_sb = a.sb_cols * a.sb_rows;
  a.sb_bits = a.num_sb > 1u ? ceil_log2(a.num_sb) : 1u;
  a.cap = cap;
  a.num_sms = sms > 0 ? sms : 1;
  a.color_f32 = h->cfg.color_format == HDSR_COLOR_RGBA32F;
  a.log_keys = (h->cfg.flags & HDSR_CFG_KEEP_SORTED_KEYS) ? 1u : 0u;
  a.composite_f16 = (h->cfg.flags & HDSR_CFG_F16_COMPOSITE) ? 1u : 0u;
  a.spin_limit = kSpinLimit;
  a.withheld_scan_tile = kNoWithheldTile;
  const uint64_t sb_cap = (uint64_t)N * 9u;  // a tile box (<= 17 tiles a side) meets <= 3x3 superblocks
  a.sb_cap = sb_cap;
  a.seg_cap = (uint32_t)((sb_cap + kSegEntries - 1u) / kSegEntries + a.num_sb);
  a.radix_tiles_cap = (uint32_t)((sb_cap + kRadixTile - 1) / kRadixTile + 1);
  const uint64_t scan_tiles_n = (N + kScanTile - 1) / kScanTile + 1;
  const uint64_t scan_tiles_m = (M + kScanTile - 1) / kScanTile + 1;
  hdsr_status s = HDSR_OK;
  float* U = nullptr;
#define ALLOC(ptr, n, what) \
  if (s == HDSR_OK) s = dev_alloc(h, &(ptr), (n), (what))
  ALLOC(U, 64, "uniforms");
  ALLOC(a.geo, N, "cache_geo");
  ALLOC(a.app, N, "cache_app");
  ALLOC(a.gb, N, "cache_gb");
  ALLOC(a.aux, N, "cache_aux");
  ALLOC(a.depth, N, "depth");
  ALLOC(a.ntiles, N, "ntiles");
  ALLOC(a.dkeys_a, N, "depth_keys_a");
  ALLOC(a.dkeys_b, N, "depth_keys_b");
  ALLOC(a.order, N, "depth_order");
  ALLOC(a.nsb, N, "superblock_counts");
  ALLOC(a.sb_off, N, "superblock_offsets");
  ALLOC(a.sbk_a, sb_cap, "superblock_keys_a");
  ALLOC(a.sbk_b, sb_cap, "superblock_keys_b");
  ALLOC(a.tile_diff, (uint64_t)(plan->tile_columns + 1) * (plan->tile_rows + 1), "tile_diff");
  ALLOC(a.sb_diff, (uint64_t)(a.sb_cols + 1) * (a.sb_rows + 1), "superblock_diff");
  ALLOC(a.sb_start, (uint64_t)a.num_sb + 1u, "superblock_starts");
  ALLOC(a.seg_first, (uint64_t)a.num_sb + 1u, "segment_firsts");
  ALLOC(a.seg_cnt, (uint64_t)a.seg_cap * kSbTiles, "segment_counts");
  ALLOC(a.chunk_mask, sb_cap / kChunkEntries + 1u, "chunk_masks");
  ALLOC(a.tile_cnt, M, "tile_counts");
  ALLOC(a.tile_dmin, M, "tile_dmin");
  ALLOC(a.tile_dmax, M, "tile_dmax");
  ALLOC(a.tile_off, M, "tile_offsets");
  ALLOC(a.tile_order, (uint64_t)plan->tile_columns * plan->tile_rows, "tile_order");
  ALLOC(a.tile_cost, 2ull * plan->tile_columns * plan->tile_rows, "tile_cost");
  ALLOC(a.tile_log, M, "tile_log");
  ALLOC(a.entries, cap, "tile_entries");
  if (h->cfg.flags & HDSR_CFG_KEEP_SORTED_KEYS) { ALLOC(a.sorted_keys, cap, "sorted_keys"); }
  ALLOC(a.tile_digits, (uint64_t)a.radix_tiles_cap * kRadixWideBins, "tile_digits");
  ALLOC(a.bin_base, (uint64_t)kRadixWideBins, "bin_base");
  a.dsort_tiles_cap = depth_sort_tiles(N);
  ALLOC(a.dsort_hist0, (uint64_t)depth_sort_bins() * a.dsort_tiles_cap, "depth_sort_counts_0");
  ALLOC(a.dsort_hist1, (uint64_t)depth_sort_bins() * a.dsort_tiles_cap, "depth_sort_counts_1");
  ALLOC(a.dsort_total, (uint64_t)depth_sort_bins(), "depth_sort_totals");
  ALLOC(a.scan_status_n, scan_tiles_n, "scan_status_n");
  ALLOC(a.scan_status_m, scan_tiles_m, "scan_status_m");
  ALLOC(a.ctl, (uint64_t)kCtlWords, "ctl");
  if (h->cfg.flags & HDSR_CFG_BACKWARD) {
    ALLOC(h->bwd_par, (uint64_t)N * 3u, "backward_screen_parameters");
    ALLOC(h->bwd_g2d, (uint64_t)N * kG2d, "backward_screen_gradients");
  }
#undef ALLOC
  if (s != HDSR_OK) { free_all(h); delete h; return s; }
  a.U = U;
  a.sbk_sorted = a.sb_bits > kRadixWideBits ? a.sbk_a : a.sbk_b;  // where the last superblock pass writes
  // status words start at epoch 0, which no frame uses. The clears run on the
  // legacy stream and are complete when create returns: the caller's stream
  // may be a non-blocking one, which does not wait for the legacy stream.
  e = cudaMemsetAsync(a.scan_status_n, 0, scan_tiles_n * 8, cudaStreamLegacy);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.scan_status_m, 0, scan_tiles_m * 8, cudaStreamLegacy);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.ctl, 0, kCtlWords * 4, cudaStreamLegacy);
  if (e == cudaSuccess) e = cudaMemsetAsync(U, 0, 256, cudaStreamLegacy);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamLegacy);
  if (e == cudaSuccess) e = cudaMallocHost(&h->pinned_u, hdsr_compositor::kUniformSlots * 256);
  for (uint32_t i = 0; e == cudaSuccess && i < hdsr_compositor::kUniformSlots; ++i)
    e = cudaEventCreateWithFlags(&h->ev_u[i], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    s = cuda_fail(h, e, "clear handle state");
    for (cudaEvent_t& ev : h->ev_u)
      if (ev) cudaEventDestroy(ev);
    if (h->fork_ev) cudaEventDestroy(h->fork_ev);
    if (h->join_ev) cudaEventDestroy(h->join_ev);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->pinned_u) cudaFreeHost(h->pinned_u);
    free_all(h);
    delete h;
    return s;
  }
  *out = h;
  return HDSR_OK;
}

void hdsr_destroy_tile_splat_compositor(hdsr_compositor* h) {
  if (!h) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  cudaDeviceSynchronize();
  for (cudaEvent_t& e : h->ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t& e : h->ev_u)
    if (e) cudaEventDestroy(e);
  if (h->pinned_u) cudaFreeHost(h->pinned_u);
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  if (h->join_ev) cudaEventDestroy(h->join_ev);
  if (h->side) cudaStreamDestroy(h->side);
  drop_graph(h);
  free_all(h);
  cudaSetDevice(prev);
  delete h;
}

hdsr_status hdsr_bind_scene(hdsr_compositor* h, const hdsr_scene_views* sc) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  if (!sc) return fail(h, HDSR_ERR_INVALID_ARG, "scene views are NULL");
  if (sc->splat_count != h->plan.splat_count)
    return fail(h, HDSR_ERR_INVALID_ARG, "scene splat_count differs from the plan");
  if (sc->sh_degree > 3) return fail(h, HDSR_ERR_INVALID_ARG, "sh_degree must be 0..3");
  if (h->plan.splat_count > 0 &&
      (!sc->positions || !sc->scales || !sc->rotations || !sc->opacities || !sc->material ||
       !sc->sh_data || !sc->sorted_indices))
    return fail(h, HDSR_ERR_INVALID_ARG, "a required scene buffer is NULL");
  if (reinterpret_cast<uintptr_t>(sc->rotations) % 16 != 0)
    return fail(h, HDSR_ERR_INVALID_ARG, "rotations must be 16-byte aligned");
  if (sc->normals == nullptr && sc->normals_len != 0)
    return fail(h, HDSR_ERR_INVALID_ARG, "normals_len without normals");
  FrameArgs& a = h->args;
  a.pos = sc->positions;
  a.scl = sc->scales;
  a.rot = sc->rotations;
  a.opa = sc->opacities;
  a.mat = sc->material;
  a.nrm = sc->normals;
  a.nrm_len = sc->normals ? sc->normals_len : 0;
  a.sh = sc->sh_data;
  a.sorted = sc->sorted_indices;
  a.sh_degree = sc->sh_degree;
  h->scene_bound = true;
  h->sorted_valid = false;
  h->cost_stale = true;
  drop_graph(h);
  return HDSR_OK;
}

hdsr_status hdsr_bind_outputs(hdsr_compositor* h, const hdsr_output_views* o) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  if (!o || !o->color || !o->depth || !o->normal || !o->material)
    return fail(h, HDSR_ERR_INVALID_ARG, "an output buffer is NULL");
  const uint64_t W = h->plan.viewport_width;
  const uint64_t cbytes = h->args.color_f32 ? 16 : 8;
  if (o->color_pitch < W * cbytes || o->depth_pitch < W * 4 || o->normal_pitch < W * 4 ||
      o->material_pitch < W * 16)
    return fail(h, HDSR_ERR_INVALID_ARG, "an output pitch is smaller than one row");
  if (o->color_pitch % cbytes || o->depth_pitch % 4 || o->normal_pitch % 4 || o->material_pitch % 16 ||
      reinterpret_cast<uintptr_t>(o->color) % cbytes || reinterpret_cast<uintptr_t>(o->material) % 16 ||
      reinterpret_cast<uintptr_t>(o->depth) % 4 || reinterpret_cast<uintptr_t>(o->normal) % 4)
    return fail(h, HDSR_ERR_INVALID_ARG, "output buffers or pitches are misaligned");
  FrameArgs& a = h->args;
  a.out_color = o->color;
  a.color_pitch = o->color_pitch;
  a.out_depth = o->depth;
  a.depth_pitch = o->depth_pitch;
  a.out_normal = o->normal;
  a.normal_pitch = o->normal_pitch;
  a.out_material = o->material;
  a.material_pitch = o->material_pitch;
  h->outputs_bound = true;
  drop_graph(h);
  return HDSR_OK;
}

void hdsr_write_tile_splat_frame_uniforms(float* target, const float* view_proj, const hdsr_plan* plan,
                                          float splat_scale, uint32_t sh_degree, const float* camera_pos,
                                          const float* view_matrix, const float* proj_matrix,
                                          const float* normal_matrix) {
  if (!target || !view_proj || !plan) return;
  auto put_u32 = [&](int i, uint32_t v) { std::memcpy(target + i, &v, 4); };
  for (int i = 0; i < 16; ++i) target[i] = view_proj[i];
  target[16] = (float)plan->viewport_width;
  target[17] = (float)plan->viewport_height;
  target[18] = (float)plan->tile_size_px;
  target[19] = 0.0f;
  put_u32(20, plan->tile_columns);
  put_u32(21, plan->tile_rows);
  put_u32(22, plan->splat_count);
  put_u32(23, plan->max_total_tile_refs);
  target[24] = splat_scale;
  put_u32(25, sh_degree);
  if (camera_pos) { target[28] = camera_pos[0]; target[29] = camera_pos[1]; target[30] = camera_pos[2]; }
  if (view_matrix) for (int i = 0; i < 16; ++i) target[32 + i] = view_matrix[i];
  if (proj_matrix) {
    // JS evaluates viewport * proj * 0.5 in double, then stores to f32
    target[48] = (float)((double)plan->viewport_width * (double)proj_matrix[0] * 0.5);
    target[49] = (float)((double)plan->viewport_height * (double)proj_matrix[5] * 0.5);
  }
  static const float kIdentity[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  const float* n = normal_matrix ? normal_matrix : kIdentity;
  target[52] = n[0]; target[53] = n[1]; target[54] = n[2]; target[55] = 0.0f;
  target[56] = n[3]; target[57] = n[4]; target[58] = n[5]; target[59] = 0.0f;
  target[60] = n[6]; target[61] = n[7]; target[62] = n[8]; target[63] = 0.0f;
}

hdsr_status hdsr_set_frame_uniforms(hdsr_compositor* h, const float* u) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  if (!u) return fail(h, HDSR_ERR_INVALID_ARG, "uniforms are NULL");
  uint32_t n, gx, gy, deg;
  std::memcpy(&gx, u + 20, 4);
  std::memcpy(&gy, u + 21, 4);
  std::memcpy(&n, u + 22, 4);
  std::memcpy(&deg, u + 25, 4);
  if (n != h->plan.splat_count || gx != h->plan.tile_columns || gy != h->plan.tile_rows)
    return fail(h, HDSR_ERR_INVALID_ARG, "uniform block does not match the plan");
  if (deg > 3) return fail(h, HDSR_ERR_INVALID_ARG, "uniform shDegree must be 0..3");
  if (u[16] != (float)h->plan.viewport_width || u[17] != (float)h->plan.viewport_height || u[18] != (float)kTilePx)
    return fail(h, HDSR_ERR_INVALID_ARG, "uniform viewport / tile size does not match the plan");
  std::memcpy(h->uniforms, u, sizeof(h->uniforms));
  h->have_uniforms = true;
  return HDSR_OK;
}

// Records a profiling event after pass `id` (no-op unless profiling).
static void mark(hdsr_compositor* h, cudaStream_t s, uint32_t id) {
  if (!h->profiling || h->ev_used >= kMaxProfiledPasses) return;
  h->pass_id[h->ev_used] = id;
  cudaEventRecord(h->ev[++h->ev_used], s);
}

// Does every full frame write the per-tile lists? (The 20-bit log-depth keys
// are computed from them.)
static bool entries_each_frame(const hdsr_compositor* h) {
  return (h->cfg.flags & (HDSR_CFG_TILE_ENTRIES | HDSR_CFG_KEEP_SORTED_KEYS)) != 0u;
}

static hdsr_status encode_checks(hdsr_compositor* h, bool full) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  if (!h->scene_bound || !h->outputs_bound) return fail(h, HDSR_ERR_NOT_BOUND, "bind scene and outputs first");
  if (!h->have_uniforms) return fail(h, HDSR_ERR_NOT_BOUND, "set frame uniforms first");
  if (!full && !h->sorted_valid) return fail(h, HDSR_ERR_NOT_BOUND, "no sorted entries: encode_full first");
  uint32_t deg;
  std::memcpy(&deg, h->uniforms + 25, 4);
  if (deg != h->args.sh_degree) return fail(h, HDSR_ERR_INVALID_ARG, "uniform shDegree differs from the bound scene");
  return HDSR_OK;
}

// Every kernel of a full frame before the rasteriser (no host work, no
// allocation: a CUDA graph can capture it).
static hdsr_status encode_pre_raster(hdsr_compositor* h, cudaStream_t s) {
  FrameArgs& a = h->args;
  const uint64_t n_splat_launch = a.N ? 1 : 0;
  cudaError_t e;
  if ((e = launch_frame_init(a, s)) != cudaSuccess) return cuda_fail(h, e, "frame_init");
  mark(h, s, 1);
  if ((e = launch_project(a, s)) != cudaSuccess) return cuda_fail(h, e, "project");
  mark(h, s, 2);
  // tile counts, the tile scan and the work order: on the side stream beside
  // the depth sort and the superblock lists (they share no buffer with them;
  // the main stream's kernels read the overflow flag the tile scan may set
  // once per block), or in line when profiling
  const bool fork = !h->profiling && h->side;
  cudaStream_t ts = fork ? h->side : s;
  if (fork && ((e = cudaEventRecord(h->fork_ev, s)) != cudaSuccess ||
               (e = cudaStreamWaitEvent(ts, h->fork_ev, 0)) != cudaSuccess))
    return cuda_fail(h, e, "fork");
  if ((e = launch_tile_counts(a, ts)) != cudaSuccess) return cuda_fail(h, e, "tile_counts");
  if (a.log_keys && (e = launch_depth_range(a, ts)) != cudaSuccess) return cuda_fail(h, e, "depth_range");
  mark(h, s, 3);
  if ((e = launch_scan_tiles(a, ts)) != cudaSuccess) return cuda_fail(h, e, "scan_tiles");
  if (a.tile_count) {
    // the raster's work order from the last frame's tile costs, on the side
    // stream after the tile scan's own order (off the frame's critical
    // path); a new scene's first frame starts from none (the scan's order)
    if (h->cost_stale) {
      e = cudaMemsetAsync(a.tile_cost, 0, 2ull * a.tile_count * sizeof(uint32_t), ts);
      if (e != cudaSuccess) return cuda_fail(h, e, "reset tile costs");
      h->cost_stale = false;
    }
    if ((e = launch_work_order(a, ts)) != cudaSuccess) return cuda_fail(h, e, "work_order");
  }
  mark(h, s, 5);
  if (fork && (e = cudaEventRecord(h->join_ev, ts)) != cudaSuccess) return cuda_fail(h, e, "fork");
  // splats: as many 9-bit passes as the frame's depth range needs -> order
  // (sortRanks by depth)
  if ((e = launch_depth_sort(a, s)) != cudaSuccess) return cuda_fail(h, e, "depth_sort");
  mark(h, s, 6);
  RadixJob dj{};
  dj.flags = a.ctl + kCtlFlags;
  dj.tile_digits = a.tile_digits;
  dj.bin_base = a.bin_base;
  dj.tiles_cap = a.radix_tiles_cap;
  dj.low_mask = 0xFFFFFFFFull;
  // superblock lists in depth order, sorted by superblock (stable)
  if ((e = launch_scan_sb(a, s)) != cudaSuccess) return cuda_fail(h, e, "scan_superblocks");
  RadixJob sj = dj;
  sj.count = a.ctl + kCtlSbPairs;
  sj.out_low = nullptr;
  // 9-bit digits: one pass up to 512 superblocks (a 4K viewport has 510)
  const uint32_t sb_passes = a.sb_bits > kRadixWideBits ? 2u : 1u;
  for (uint32_t p = 0; p < sb_passes; ++p) {
    sj.in = (p & 1u) ? a.sbk_b : a.sbk_a;
    sj.out = (p & 1u) ? nullptr : a.sbk_b;
    sj.out_keys = (p & 1u) ? a.sbk_a : a.sbk_b;
    sj.shift = kSbKeyShift + kRadixWideBits * p;
    sj.bits = p == 0 ? (a.sb_bits < kRadixWideBits ? a.sb_bits : kRadixWideBits) : a.sb_bits - kRadixWideBits;
    if ((e = launch_radix_pass(sj, p + 1 == sb_passes, a.num_sms, s)) != cudaSuccess)
      return cuda_fail(h, e, "superblock_sort");
  }
  mark(h, s, 7);
  if ((e = launch_chunk_masks(a, s)) != cudaSuccess) return cuda_fail(h, e, "chunk_masks");
  mark(h, s, 9);
  // the rasteriser needs the superblock starts and the work order, the
  // per-tile lists the tile offsets, and all of them the final overflow flag
  if (fork && (e = cudaStreamWaitEvent(s, h->join_ev, 0)) != cudaSuccess) return cuda_fail(h, e, "join");
  if (entries_each_frame(h)) {
    if ((e = launch_tile_entries(a, s)) != cudaSuccess) return cuda_fail(h, e, "tile_entries");
    mark(h, s, 8);
    if (a.tile_count) h->launches += 3;
  }
  if (a.log_keys) {
    if ((e = launch_log_depth_keys(a, s)) != cudaSuccess) return cuda_fail(h, e, "log_depth_keys");
    h->launches += 2;
  }
  h->launches += 1 + n_splat_launch + (n_splat_launch + 1) + 1 + 9 * n_splat_launch + 1 +
                 3 * (a.sb_bits > kRadixWideBits ? 2 : 1) + (a.tile_count ? 2 : 0);
  return HDSR_OK;
}

static hdsr_status encode_raster(hdsr_compositor* h, cudaStream_t s, bool full) {
  FrameArgs& a = h->args;
  cudaError_t e;
  if (!full) {
    // composite-only reuses the frame's entries; the raster's tile counter
    // is the one control word it must start from zero
    e = cudaMemsetAsync(a.ctl + kCtlRasterTile, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return cuda_fail(h, e, "reset raster counter");
  }
  if ((e = launch_raster(a, s)) != cudaSuccess) return cuda_fail(h, e, "raster");
  mark(h, s, 17);
  if (a.tile_count) h->launches += 1;
  h->last_stream = s;
  h->has_last_stream = true;
  if (full) {
    h->sorted_valid = true;
    h->entries_valid = entries_each_frame(h);
  }
  return HDSR_OK;
}

// The per-tile lists of the last full frame, queued on `s` unless the frame
// wrote them (the superblock lists they come from stay until the next frame).
static hdsr_status ensure_entries(hdsr_compositor* h, cudaStream_t s) {
  if (h->entries_valid || !h->sorted_valid) return HDSR_OK;
  cudaError_t e = launch_tile_entries(h->args, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "tile_entries");
  if (h->args.tile_count) h->launches += 3;
  h->entries_valid = true;
  return HDSR_OK;
}

// Frames go through the frame graph unless HDSR_CFG_NO_GRAPH, profiling (the
// per-pass events need direct launches), a legacy / per-thread default
// stream (which cannot be captured) or a stream the caller is capturing
// itself (the kernels then go straight into the caller's graph) says
// otherwise.
static bool use_graph(const hdsr_compositor* h, cudaStream_t s) {
  if ((h->cfg.flags & HDSR_CFG_NO_GRAPH) || h->profiling || s == nullptr || s == cudaStreamLegacy ||
      s == cudaStreamPerThread)
    return false;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone;
}

// Captures every kernel of a full frame on `s` (nothing runs) into
// h->frame_graph; on any failure the handle launches directly until the next
// bind.
static void capture_frame(hdsr_compositor* h, cudaStream_t s) {
  const uint64_t before = h->launches;
  cudaGraph_t g = nullptr;
  hdsr_status st = HDSR_ERR_CUDA;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    st = encode_pre_raster(h, s);
    if (st == HDSR_OK) st = encode_raster(h, s, true);
    if (cudaStreamEndCapture(s, &g) != cudaSuccess) st = HDSR_ERR_CUDA;
  }
  h->graph_launches = h->launches - before;
  h->launches = before;  // captured, not run
  if (st != HDSR_OK || !g || cudaGraphInstantiate(&h->frame_graph, g, 0) != cudaSuccess) {
    h->frame_graph = nullptr;
    h->graph_failed = true;
  }
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();  // a failed capture leaves no sticky error: clear its record
}

// Camera turn (degrees) up to which the last frame's tile costs still order
// the raster's tiles.
constexpr double kCostKeepDegrees = 10.0;
const double kCostKeepCos = std::cos(kCostKeepDegrees * 3.14159265358979323846 / 180.0);

static hdsr_status encode(hdsr_compositor* h, void* stream, bool full) {
  hdsr_status st = encode_checks(h, full);
  if (st != HDSR_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  FrameArgs& a = h->args;
  h->ev_used = 0;
  if (h->profiling) cudaEventRecord(h->ev[0], s);
  if (!h->device_u_valid || std::memcmp(h->device_u, h->uniforms, 256) != 0) {
    const uint32_t k = h->next_u;
    h->next_u = (k + 1) % hdsr_compositor::kUniformSlots;
    cudaError_t e = h->ev_u_pending[k] ? cudaEventSynchronize(h->ev_u[k]) : cudaSuccess;
    float* slot = h->pinned_u + 64 * k;
    if (e == cudaSuccess) {
      std::memcpy(slot, h->uniforms, 256);
      e = cudaMemcpyAsync(const_cast<float*>(a.U), slot, 256, cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) e = cudaEventRecord(h->ev_u[k], s);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload uniforms");
    h->ev_u_pending[k] = true;
    std::memcpy(h->device_u, h->uniforms, 256);
    h->device_u_valid = true;
  }
  mark(h, s, 0);
  if (full && a.tile_count) {
    // The raster's work order follows the last frame's tile costs. After a
    // camera turn of more than kCostKeepDegrees they describe other tiles
    // (an orbit's 45-degree steps made the raster 4% slower than the tile
    // scan's order), so they are cleared and this frame takes the scan's
    // order. The view direction is the view matrix's third row.
    const float* u = h->uniforms;
    const double f[3] = {u[34], u[38], u[42]};
    if (h->cost_view_valid) {
      const double dot = f[0] * h->cost_view[0] + f[1] * h->cost_view[1] + f[2] * h->cost_view[2];
      const double nn = std::sqrt((f[0] * f[0] + f[1] * f[1] + f[2] * f[2]) *
                                  ((double)h->cost_view[0] * h->cost_view[0] +
                                   (double)h->cost_view[1] * h->cost_view[1] +
                                   (double)h->cost_view[2] * h->cost_view[2]));
      if (!(dot >= kCostKeepCos * nn)) {
        cudaError_t e = cudaMemsetAsync(a.tile_cost, 0, 2ull * a.tile_count * sizeof(uint32_t), s);
        if (e != cudaSuccess) return cuda_fail(h, e, "reset tile costs");
      }
    }
    for (int k = 0; k < 3; ++k) h->cost_view[k] = (float)f[k];
    h->cost_view_valid = true;
  }
  if (full && use_graph(h, s)) {
    if (!h->frame_graph && !h->graph_failed && h->direct_frames > 0) capture_frame(h, s);
    if (h->frame_graph) {
      cudaError_t e = cudaGraphLaunch(h->frame_graph, s);
      if (e != cudaSuccess) return cuda_fail(h, e, "frame graph launch");
      h->launches += h->graph_launches;
      h->last_stream = s;
      h->has_last_stream = true;
      h->sorted_valid = true;
      h->entries_valid = entries_each_frame(h);
      return HDSR_OK;
    }
  }
  if (full && (st = encode_pre_raster(h, s)) != HDSR_OK) return st;
  st = encode_raster(h, s, full);
  if (st == HDSR_OK && full) ++h->direct_frames;
  return st;
}

hdsr_status hdsr_encode_full(hdsr_compositor* h, void* stream) { return encode(h, stream, true); }

hdsr_status hdsr_sort_back_to_front(hdsr_compositor* h, const float view[16], uint32_t* sorted_out, void* stream) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  if (!view) return fail(h, HDSR_ERR_INVALID_ARG, "view matrix is NULL");
  if (!h->scene_bound) return fail(h, HDSR_ERR_NOT_BOUND, "bind the scene first");
  if (h->args.N && !sorted_out) return fail(h, HDSR_ERR_INVALID_ARG, "output is NULL");
  const double vrow[4] = {view[2], view[6], view[10], view[14]};
  cudaError_t e = launch_sort_back_to_front(h->args, vrow, sorted_out, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(h, e, "sort_back_to_front");
  if (h->args.N) h->launches += 1 + 3 * 4;
  return HDSR_OK;
}

hdsr_status hdsr_encode_backward(hdsr_compositor* h, const hdsr_grad_views* g, void* stream) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  if (!(h->cfg.flags & HDSR_CFG_BACKWARD)) return fail(h, HDSR_ERR_UNSUPPORTED, "create with HDSR_CFG_BACKWARD");
  if (h->cfg.flags & HDSR_CFG_F16_COMPOSITE)
    return fail(h, HDSR_ERR_UNSUPPORTED, "the adjoint differentiates the f32 composite, not HDSR_CFG_F16_COMPOSITE");
  if (!g || !g->d_color) return fail(h, HDSR_ERR_INVALID_ARG, "gradient views are NULL");
  if (!h->sorted_valid) return fail(h, HDSR_ERR_NOT_BOUND, "no frame: encode_full first");
  const FrameArgs& a = h->args;
  if (a.N && (!g->d_positions || !g->d_log_scales || !g->d_rotations || !g->d_opacities || !g->d_sh))
    return fail(h, HDSR_ERR_INVALID_ARG, "a gradient output is NULL");
  if (g->d_color_pitch < (uint64_t)a.W * 16u || (g->d_color_pitch & 15u))
    return fail(h, HDSR_ERR_INVALID_ARG, "d_color pitch must be >= 16*W bytes and a multiple of 16");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t N = a.N;
  const uint64_t sh_row = 6u + 3u * (((uint64_t)a.sh_degree + 1u) * (a.sh_degree + 1u) - 1u);
  cudaError_t e = cudaSuccess;
  if (N) {
    e = cudaMemsetAsync(g->d_positions, 0, N * 12, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->d_log_scales, 0, N * 12, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->d_rotations, 0, N * 16, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->d_opacities, 0, N * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->d_sh, 0, N * sh_row * 4, s);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(a.ctl + kCtlBwdTile, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return cuda_fail(h, e, "backward clears");
  BwdArgs b{};
  b.f = a;
  b.d_color = g->d_color;
  b.d_color_pitch = g->d_color_pitch;
  b.par = h->bwd_par;
  b.g2d = h->bwd_g2d;
  b.d_pos = g->d_positions;
  b.d_lsc = g->d_log_scales;
  b.d_rot = g->d_rotations;
  b.d_opa = g->d_opacities;
  b.d_sh = g->d_sh;
  if ((e = launch_backward(b, s)) != cudaSuccess) return cuda_fail(h, e, "backward");
  h->launches += (a.N ? 2 : 0) + (a.tile_count ? 1 : 0);
  return HDSR_OK;
}

hdsr_status hdsr_encode_composite_only(hdsr_compositor* h, void* stream) { return encode(h, stream, false); }

hdsr_status hdsr_query_status(hdsr_compositor* h, hdsr_frame_stats* st) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  cudaError_t e = h->has_last_stream ? cudaStreamSynchronize(h->last_stream) : cudaSuccess;
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
  uint32_t ctl[kCtlWords];
  e = cudaMemcpy(ctl, h->args.ctl, sizeof(ctl), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(h, e, "read status");
  if (st) {
    std::memset(st, 0, sizeof(*st));
    st->total_pairs = (uint64_t)ctl[kCtlPairsLo] | ((uint64_t)ctl[kCtlPairsHi] << 32);
    st->pair_capacity = h->args.cap;
    st->visible_splats = ctl[kCtlVisible];
    st->hot_tiles = ctl[kCtlHotTiles];
    st->chunks = ctl[kCtlChunks];
    st->device_flags = ctl[kCtlFlags];
    st->superblock_entries = ctl[kCtlSbPairs];
    st->segments = ctl[kCtlSegments];
    st->depth_sort_passes = ctl[kCtlDepthPasses];
    st->reserved = 0u;
  }
  if (ctl[kCtlFlags] & HDSR_DEV_OVERFLOW) {
    h->sorted_valid = false;
    return fail(h, HDSR_ERR_OVERFLOW, "frame needs more (tile, splat) pairs than pair_capacity");
  }
  if (ctl[kCtlFlags] & HDSR_DEV_TIMEOUT) return fail(h, HDSR_ERR_TIMEOUT, "a device-side wait gave up");
  if (ctl[kCtlFlags] & HDSR_DEV_COUNT_MISMATCH)
    return fail(h, HDSR_ERR_CUDA, "internal check failed: tile counts and superblock lists disagree");
  if (ctl[kCtlFlags] & HDSR_DEV_BAD_ENTRY)
    return fail(h, HDSR_ERR_CUDA, "internal check failed: a list held a sortRank >= splat count");
  return HDSR_OK;
}

const char* hdsr_last_error(const hdsr_compositor* h) { return h ? h->err : g_null_err; }

hdsr_status hdsr_get_buffer(hdsr_compositor* h, hdsr_buffer_id id, void** ptr, uint64_t* bytes) {
  if (!h || !ptr || !bytes) return HDSR_ERR_INVALID_ARG;
  const FrameArgs& a = h->args;
  const uint64_t N = a.N, M = a.M, cap = a.cap;
  switch (id) {
    case HDSR_BUF_CACHE_GEO: *ptr = a.geo; *bytes = N * 16; break;
    case HDSR_BUF_CACHE_APP: *ptr = a.app; *bytes = N * 16; break;
    case HDSR_BUF_CACHE_GB: *ptr = a.gb; *bytes = N * 16; break;
    case HDSR_BUF_CACHE_AUX: *ptr = a.aux; *bytes = N * 8; break;
    case HDSR_BUF_DEPTH: *ptr = a.depth; *bytes = N * 4; break;
    case HDSR_BUF_TILE_COUNTS: *ptr = a.tile_cnt; *bytes = M * 4; break;
    case HDSR_BUF_TILE_OFFSETS: *ptr = a.tile_off; *bytes = M * 4; break;
    case HDSR_BUF_TILE_ENTRIES:
      if (!h->entries_valid && h->sorted_valid && h->has_last_stream) {
        hdsr_status es = ensure_entries(h, h->last_stream);
        if (es != HDSR_OK) return es;
        cudaError_t e = cudaStreamSynchronize(h->last_stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
      }
      *ptr = a.entries; *bytes = cap * 4; break;
    case HDSR_BUF_SORTED_KEYS:
      if (!a.sorted_keys) return fail(h, HDSR_ERR_UNSUPPORTED, "create with HDSR_CFG_KEEP_SORTED_KEYS");
      *ptr = a.sorted_keys; *bytes = cap * 8; break;
    case HDSR_BUF_PAIR_OFFSETS: *ptr = a.sb_off; *bytes = N * 4; break;
    case HDSR_BUF_DEPTH_ORDER: *ptr = a.order; *bytes = N * 4; break;
    case HDSR_BUF_BACKWARD_PARAMS:
      if (!h->bwd_par) return fail(h, HDSR_ERR_UNSUPPORTED, "create with HDSR_CFG_BACKWARD");
      *ptr = h->bwd_par; *bytes = N * 48; break;
    case HDSR_BUF_WORK_ORDER: *ptr = a.tile_order; *bytes = (uint64_t)a.tile_count * 4; break;
    case HDSR_BUF_TILE_COSTS: *ptr = a.tile_cost; *bytes = (uint64_t)a.tile_count * 8; break;
    case HDSR_BUF_SUPERBLOCK_LISTS:
      *ptr = const_cast<unsigned long long*>(a.sbk_sorted); *bytes = a.sb_cap * 8; break;
    case HDSR_BUF_CHUNK_MASKS: *ptr = a.chunk_mask; *bytes = (a.sb_cap / kChunkEntries + 1u) * 8; break;
    default: return fail(h, HDSR_ERR_INVALID_ARG, "unknown buffer id");
  }
  return HDSR_OK;
}

uint32_t hdsr_rank_bits(const hdsr_compositor* h) { return h ? h->args.rank_bits : 0u; }

hdsr_status hdsr_set_profiling(hdsr_compositor* h, int enable) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  if (enable) {
    for (cudaEvent_t& ev : h->ev) {
      if (ev) continue;
      cudaError_t e = cudaEventCreate(&ev);
      if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventCreate");
    }
  }
  if ((enable != 0) != h->profiling) drop_graph(h);
  h->profiling = enable != 0;
  return HDSR_OK;
}

hdsr_status hdsr_pass_times(hdsr_compositor* h, float* ms, uint32_t* ids, uint32_t max, uint32_t* count) {
  if (!h || !count) return HDSR_ERR_INVALID_ARG;
  *count = 0;
  if (!h->profiling || h->ev_used == 0) return fail(h, HDSR_ERR_NOT_BOUND, "no profiled frame");
  cudaError_t e = cudaEventSynchronize(h->ev[h->ev_used]);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventSynchronize");
  uint32_t n = h->ev_used < max ? h->ev_used : max;
  for (uint32_t i = 0; i < n; ++i) {
    float t = 0.0f;
    cudaEventElapsedTime(&t, h->ev[i], h->ev[i + 1]);
    if (ms) ms[i] = t;
    if (ids) ids[i] = h->pass_id[i];
  }
  *count = n;
  return HDSR_OK;
}

const char* hdsr_pass_name(uint32_t id) { return id < kNumPassNames ? kPassNames[id] : "unknown"; }

uint64_t hdsr_launch_count(const hdsr_compositor* h) { return h ? h->launches : 0u; }

hdsr_status hdsr_set_scan_wait(hdsr_compositor* h, uint32_t spin_limit, uint32_t withheld_tile) {
  if (!h) return HDSR_ERR_INVALID_ARG;
  h->args.spin_limit = spin_limit ? spin_limit : kSpinLimit;
  h->args.withheld_scan_tile = withheld_tile;
  drop_graph(h);  // a frame graph holds the old arguments
  return HDSR_OK;
}

}  // extern "C"

// ---- internal entry points of the serving loop (C++ linkage) --------------
namespace hdsr {

uint64_t handle_device_bytes(const hdsr_compositor* h) { return h ? h->device_bytes : 0u; }

const FrameArgs* handle_args(const hdsr_compositor* h) { return h ? &h->args : nullptr; }

int handle_frame_checks(hdsr_compositor* h) { return encode_checks(h, true); }

int handle_upload_uniforms(hdsr_compositor* h, const float* pinned_uniforms, cudaStream_t s) {
  h->device_u_valid = false;  // the caller's staging, not the handle's record
  cudaError_t e = cudaMemcpyAsync(const_cast<float*>(h->args.U), pinned_uniforms, 256, cudaMemcpyHostToDevice, s);
  return e == cudaSuccess ? HDSR_OK : cuda_fail(h, e, "upload uniforms");
}

int handle_encode_pre_raster(hdsr_compositor* h, cudaStream_t s) { return encode_pre_raster(h, s); }

int handle_encode_raster(hdsr_compositor* h, cudaStream_t s) { return encode_raster(h, s, true); }

}  // namespace hdsr
