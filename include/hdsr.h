/*
 * hdsr.h — C ABI of the GB300 tile-splat compositor.
 *
 * Drop-in for the reference's compute compositor operator API
 * (lyonsno/hybrid-differentiable-deferred-splat-mesh-renderer,
 * src/gpuTileSplatCompositor.ts). Each entry point names the reference
 * function it replaces. Plain pointers and sizes only; device pointers are
 * CUDA device addresses owned by the caller unless stated otherwise; a
 * "stream" is a cudaStream_t passed as void* (NULL = legacy default stream).
 *
 * Error model: every call returns hdsr_status; no C++ exception crosses this
 * boundary, nothing traps or aborts. Work queued on a stream reports device-
 * side conditions (pair-capacity overflow, a bounded wait that gave up) in a
 * status word read by hdsr_query_status(). A handle is externally
 * synchronised (one host thread at a time); distinct handles are independent.
 */
#ifndef HDSR_H
#define HDSR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HDSR_ABI_VERSION 4

typedef enum hdsr_status {
  HDSR_OK = 0,
  HDSR_ERR_INVALID_ARG = 1,
  HDSR_ERR_OOM = 2,
  HDSR_ERR_CUDA = 3,
  HDSR_ERR_OVERFLOW = 4,     /* more (tile, splat) pairs than the handle holds */
  HDSR_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up           */
  HDSR_ERR_UNSUPPORTED = 6,
  HDSR_ERR_NOT_BOUND = 7     /* encode before bind_scene / bind_outputs      */
} hdsr_status;

/* Device status flags (hdsr_frame_stats.device_flags). */
#define HDSR_DEV_OVERFLOW   0x1u  /* pairs > pair_capacity: frame skipped       */
#define HDSR_DEV_TIMEOUT    0x2u  /* a lookback wait exceeded its spin limit    */
#define HDSR_DEV_BAD_INDEX  0x4u  /* sortedIndices held an id >= splatCount     */
#define HDSR_DEV_COUNT_MISMATCH 0x8u /* tile counts and tile lists disagree (bug)  */
#define HDSR_DEV_BAD_ENTRY  0x10u /* an entry or order index >= N was skipped (bug) */

/* planTileSplatCompositor input — gpuTileSplatCompositor.ts:109-116. */
typedef struct hdsr_plan_input {
  uint32_t viewport_width;
  uint32_t viewport_height;
  uint32_t tile_size_px;          /* the reference always uses 16; only 16 is supported */
  uint32_t splat_count;
  double tile_entry_multiplier;   /* <= 0 selects the reference default, 16 */
} hdsr_plan_input;

/* TileSplatCompositorPlan — gpuTileSplatCompositor.ts:39-49. */
typedef struct hdsr_plan {
  uint32_t viewport_width;
  uint32_t viewport_height;
  uint32_t tile_size_px;
  uint32_t tile_columns;
  uint32_t tile_rows;
  uint32_t tile_count;
  uint32_t morton_tile_count;     /* M = morton(cols-1, rows-1) + 1 */
  uint32_t splat_count;
  uint32_t max_total_tile_refs;   /* reference budget min(ceil(N*mult), 65535*256) */
} hdsr_plan;

#define HDSR_COLOR_RGBA16F 0u     /* reference output texture format */
#define HDSR_COLOR_RGBA32F 1u

#define HDSR_CFG_KEEP_SORTED_KEYS 0x1u  /* compute the 20-bit log-depth keys per entry */
#define HDSR_CFG_NO_GRAPH         0x2u  /* launch every full frame's kernels directly; otherwise,
                                           on a stream other than the legacy or per-thread
                                           default stream and not under the caller's own
                                           capture, the second full frame after a bind is
                                           captured into a CUDA graph that later frames replay */
#define HDSR_CFG_BACKWARD         0x4u  /* allocate the adjoint's buffers (hdsr_encode_backward) */
#define HDSR_CFG_TILE_ENTRIES     0x8u  /* write the per-tile entry lists in every full frame
                                           (otherwise built on demand: see HDSR_BUF_TILE_ENTRIES) */
#define HDSR_CFG_F16_COMPOSITE    0x10u /* createTileSplatCompositor {f16: true}: the f16 composite
                                           variant (gpu_tile_splat_composite_f16.wgsl), transmittance
                                           and colour accumulated in f16; no hdsr_encode_backward */

/* Options of createTileSplatCompositor — gpuTileSplatCompositor.ts:141-145
 * ({f16?} is HDSR_CFG_F16_COMPOSITE; FP32 transmittance is the default). */
typedef struct hdsr_config {
  uint64_t pair_capacity;         /* (tile, splat) pairs held; 0 = max(budget, ceil(N*16)) */
  uint32_t color_format;          /* HDSR_COLOR_* */
  uint32_t flags;                 /* HDSR_CFG_* */
} hdsr_config;

/* Splat buffers of createTileSplatBindGroups — gpuTileSplatCompositor.ts:
 * 792-803 and the upload layout of src/splats.ts:376-500. Device pointers,
 * borrowed: the handle never frees them. */
typedef struct hdsr_scene_views {
  uint32_t splat_count;
  uint32_t sh_degree;             /* 0..3 */
  const float* positions;         /* N*3 */
  const float* scales;            /* N*3 log scales */
  const float* rotations;         /* N*4 wxyz */
  const float* opacities;         /* N activated opacities in [0,1] */
  const uint32_t* material;       /* N pack2x16float(roughness, metalness) */
  const float* normals;           /* NULL (covariance normals), N*3 or N*6 floats */
  uint64_t normals_len;           /* float count of normals */
  const float* sh_data;           /* N*(6+3K): dc3 | sh 3K | emissive3, K=(d+1)^2-1 */
  const uint32_t* sorted_indices; /* N back-to-front splat ids (gpuSortPrototype) */
} hdsr_scene_views;

/* Output textures of createTileSplatBindGroups, as headless device buffers.
 * Pitches are bytes per row. */
typedef struct hdsr_output_views {
  void* color;        uint64_t color_pitch;     /* rgba16f (8 B/px) or rgba32f (16 B/px) */
  float* depth;       uint64_t depth_pitch;     /* r32f */
  uint32_t* normal;   uint64_t normal_pitch;    /* r32u: pack2x16float(oct normal) */
  uint32_t* material; uint64_t material_pitch;  /* rgba32u */
} hdsr_output_views;

typedef struct hdsr_frame_stats {
  uint64_t total_pairs;           /* P of the last encoded frame */
  uint64_t pair_capacity;
  uint32_t visible_splats;
  uint32_t superblock_entries;    /* (8x8-tile superblock, splat) list entries */
  uint32_t hot_tiles;             /* tiles with > 4096 entries */
  uint32_t chunks;                /* 4096-entry chunks of hot tiles */
  uint32_t device_flags;          /* HDSR_DEV_* */
  uint32_t segments;              /* 256-entry segments of the superblock lists */
  uint32_t depth_sort_passes;     /* 9-bit passes the depth sort ran (1-4: the frame's depth range) */
  uint32_t reserved;
} hdsr_frame_stats;

typedef struct hdsr_compositor hdsr_compositor;

/* ABI version of the loaded library. */
uint32_t hdsr_abi_version(void);

/* planTileSplatCompositor — gpuTileSplatCompositor.ts:109-139. Pure. */
hdsr_status hdsr_plan_tile_splat_compositor(const hdsr_plan_input* in, hdsr_plan* out);

/* createTileSplatCompositor — gpuTileSplatCompositor.ts:141-728. Allocates
 * every internal device buffer on the current CUDA device. */
hdsr_status hdsr_create_tile_splat_compositor(const hdsr_plan* plan, const hdsr_config* cfg,
                                              hdsr_compositor** out);

/* resources.destroy() — gpuTileSplatCompositor.ts:710-727. NULL is a no-op. */
void hdsr_destroy_tile_splat_compositor(hdsr_compositor* h);

/* createTileSplatBindGroups, splat half — gpuTileSplatCompositor.ts:792-995. */
hdsr_status hdsr_bind_scene(hdsr_compositor* h, const hdsr_scene_views* scene);

/* createTileSplatBindGroups, output half (outputTexture, gbufferTextures). */
hdsr_status hdsr_bind_outputs(hdsr_compositor* h, const hdsr_output_views* out);

/* writeTileSplatFrameUniforms — gpuTileSplatCompositor.ts:730-774. Pure
 * host; same 64-float layout. cameraPos (3), viewMatrix (16), projMatrix (16)
 * may be NULL (left untouched, as in the reference); normalMatrix (9, column
 * major) NULL = identity. */
void hdsr_write_tile_splat_frame_uniforms(float target[64], const float view_proj[16],
                                          const hdsr_plan* plan, float splat_scale,
                                          uint32_t sh_degree, const float* camera_pos,
                                          const float* view_matrix, const float* proj_matrix,
                                          const float* normal_matrix);

/* device.queue.writeBuffer(frameUniformBuffer, ...) — splatRenderer.ts:
 * 1029-1030. The block is copied into the handle; the next encode uploads it
 * on its stream. */
hdsr_status hdsr_set_frame_uniforms(hdsr_compositor* h, const float uniforms[64]);

/* encodeFullComputeCompositorPipeline — gpuTileSplatCompositor.ts:
 * 1023-1179. Queues the whole frame (project, count, scans, key emission,
 * radix sort, per-tile sort + hot-tile cascade, rasteriser) on `stream`.
 * Returns launch errors; device-side conditions go to hdsr_query_status. */
hdsr_status hdsr_encode_full(hdsr_compositor* h, void* stream);

/* encodeCompositeOnly — gpuTileSplatCompositor.ts:1001-1014. Rasterises the
 * entries sorted by the last encode_full again (same camera). */
hdsr_status hdsr_encode_composite_only(hdsr_compositor* h, void* stream);

/* Synchronises the stream of the last encode and reports its frame. Returns
 * HDSR_ERR_OVERFLOW / HDSR_ERR_TIMEOUT when the device flagged one. */
hdsr_status hdsr_query_status(hdsr_compositor* h, hdsr_frame_stats* stats);

/* Last error message of this handle (static storage, never NULL). */
const char* hdsr_last_error(const hdsr_compositor* h);

/* Internal buffers, for parity tests and zero-copy consumers. */
typedef enum hdsr_buffer_id {
  HDSR_BUF_CACHE_GEO = 0,     /* float4[N]: centerPx.xy, invCov.xy (reference words 0-3) */
  HDSR_BUF_CACHE_APP = 1,     /* uint4[N]: invCov.z, f16(radius,opacity), f16 rgb (words 4,6,9,10) */
  HDSR_BUF_CACHE_GB = 2,      /* uint4[N]: material, oct normal, f16 emissive (words 5,8,11,12) */
  HDSR_BUF_CACHE_AUX = 3,     /* uint2[N]: tile box u8x4, f16 normal confidence (words 7,13) */
  HDSR_BUF_DEPTH = 4,         /* u32[N]: f32 NDC depth bits */
  HDSR_BUF_TILE_COUNTS = 5,   /* u32[M] */
  HDSR_BUF_TILE_OFFSETS = 6,  /* u32[M] exclusive prefix of tile counts */
  HDSR_BUF_TILE_ENTRIES = 7,  /* u32[P] sortRank per entry, final per-tile order. The rasteriser
                                 reads the superblock lists, so a frame writes these lists only
                                 with HDSR_CFG_TILE_ENTRIES or HDSR_CFG_KEEP_SORTED_KEYS; else
                                 hdsr_get_buffer builds them for the last full frame on the
                                 handle's last stream and synchronizes that stream. */
  HDSR_BUF_SORTED_KEYS = 8,   /* u64[P] per final entry: tile<<(20+R) | k20<<R | sortRank */
  HDSR_BUF_PAIR_OFFSETS = 9,  /* u32[N] exclusive prefix of per-splat superblock counts, depth order */
  HDSR_BUF_DEPTH_ORDER = 10,  /* u32[N] ascending (depth bits, sortRank): sortRank in bits 0-23,
                                 the splat's superblock count in bits 24-31 */
  HDSR_BUF_BACKWARD_PARAMS = 11, /* float4[N][3] per sortRank, written by hdsr_encode_backward: the
                                 adjoint's screen-space parameters (cx, cy, ia, ib | ic, opacity,
                                 r, g | b, 0, 0, 0); HDSR_CFG_BACKWARD handles only */
  HDSR_BUF_WORK_ORDER = 12,   /* u32[tile_count] ty << 16 | tx: the order in which the last full
                                 frame's rasteriser took its tiles (a permutation of the tiles) */
  HDSR_BUF_TILE_COSTS = 13,   /* u32[2 * tile_count] per half tile (index 2 * (ty * cols + tx) +
                                 half): the last raster's cost, from which the next full frame
                                 orders its tiles (most expensive first); 0 before any raster */
  HDSR_BUF_SUPERBLOCK_LISTS = 14, /* u64[Q] (Q: hdsr_frame_status.superblock_entries) the lists the
                                 rasterisers walk: superblock << 36 | local rect << 24 | sortRank,
                                 grouped by superblock (8x8 tiles, row-major), each list in
                                 ascending (depth bits, sortRank); the local rect is x0 | x1 << 3 |
                                 y0 << 6 | y1 << 9, the splat's tile box clipped to the superblock */
  HDSR_BUF_CHUNK_MASKS = 15   /* u64[(Q + 31) / 32] per 32 list entries: the union of their local
                                 rects as tile bits (bit y * 8 + x of the superblock) */
} hdsr_buffer_id;

/* Device address and byte size of an internal buffer (valid until destroy).
 * HDSR_BUF_TILE_ENTRIES may first build the per-tile lists (see above). */
hdsr_status hdsr_get_buffer(hdsr_compositor* h, hdsr_buffer_id id, void** device_ptr,
                            uint64_t* bytes);

/* Number of low key bits that hold the sortRank in HDSR_BUF_SORTED_KEYS. */
uint32_t hdsr_rank_bits(const hdsr_compositor* h);

/* Per-pass timing of the next encodes: CUDA events recorded on the encode
 * stream between passes (the reference times only its present pass with
 * timestamp queries, src/timestamps.ts:10-76). */
hdsr_status hdsr_set_profiling(hdsr_compositor* h, int enable);

/* Durations (ms) of the passes of the last profiled encode, with their pass
 * ids (see hdsr_pass_name). Synchronises on the last event. */
hdsr_status hdsr_pass_times(hdsr_compositor* h, float* ms, uint32_t* ids, uint32_t max, uint32_t* count);

/* Name of a profiled pass id ("project", "radix_pass_0", "raster", ...). */
const char* hdsr_pass_name(uint32_t id);

/* Number of kernels this handle has queued since creation. */
uint64_t hdsr_launch_count(const hdsr_compositor* h);

/* Bounded device waits (no reference counterpart: WebGPU has no
 * inter-workgroup waits; the reference's three-pass scan,
 * gpu_prefix_sum.wgsl:14-85, needs none). Each scan tile waits for its
 * predecessors' status words at most `spin_limit` spins of about 100 ns
 * (0 selects the default, 2^22); a wait that runs out sets HDSR_DEV_TIMEOUT,
 * every later kernel of the frame returns without writing (the output images
 * keep their previous contents), and hdsr_query_status returns
 * HDSR_ERR_TIMEOUT. `withheld_tile` (test hook; 0xFFFFFFFF = none) makes that
 * tile of each scan compute its prefix but post nothing, so that its
 * successors' waits run out. Drops the handle's frame graph. */
hdsr_status hdsr_set_scan_wait(hdsr_compositor* h, uint32_t spin_limit, uint32_t withheld_tile);

/* Gradients of one frame (no reference counterpart: the reference renders
 * only). Input: dL/d(color output) as rgba f32 per pixel. Outputs, written
 * (not accumulated), in the layouts of hdsr_scene_views, indexed by splat id:
 * positions N*3, log-scales N*3, rotations N*4 (wxyz), activated opacities
 * N, SH rows N*(6+3K) (dc, higher orders; the emissive slots get 0). */
typedef struct hdsr_grad_views {
  const float* d_color;   uint64_t d_color_pitch;   /* W x H rgba f32, bytes per row */
  float* d_positions;
  float* d_log_scales;
  float* d_rotations;
  float* d_opacities;
  float* d_sh;
} hdsr_grad_views;

/* Adjoint of the last hdsr_encode_full (same scene, uniforms and tile
 * entries), on `stream`. The differentiated function is the frame with the
 * cache's f16 opacity and colour taken at fp32, every composite threshold
 * (power > -4, alpha > 1/255, T >= 0.001, alpha cap 0.99) and projection
 * clamp held fixed (clamped quantities pass no gradient). Needs a handle
 * created with HDSR_CFG_BACKWARD; gradients w.r.t. the G-buffer outputs and
 * the emissive colour are not computed. Float atomics: results are not
 * bitwise reproducible from run to run. */
hdsr_status hdsr_encode_backward(hdsr_compositor* h, const hdsr_grad_views* grads, void* stream);

/* sortedIndices on the device: the back-to-front order of the bound scene's
 * positions for a view matrix (column-major, as in the frame uniforms), as
 * gpuSortPrototype.ts:120-163 defines it (simulateGpuViewDepthSortPrototype):
 * key = f32(-(view[2] x + view[6] y + view[10] z + view[14])) with the sum in
 * double, descending, ties by ascending splat id (-0 equal to +0; NaN keys
 * last). Writes splat_count u32 to `sorted_out` (device; it may be the bound
 * sortedIndices buffer) on `stream`; uses the handle's depth-sort scratch, so
 * it is ordered with the handle's frames on one stream. */
hdsr_status hdsr_sort_back_to_front(hdsr_compositor* h, const float view[16], uint32_t* sorted_out, void* stream);

/* ---- Serving loop ---------------------------------------------------------
 * No reference counterpart: the reference renders one scene per page
 * (splatRenderer.ts loadScene :866-961, renderFrame :1024-1140). A server
 * keeps scenes resident on the device and renders (scene, camera, viewport)
 * requests: each request runs on an idle compositor handle ("slot") of its
 * (scene, viewport, colour format), with its own stream; slots are created on
 * demand inside an HBM budget (idle slots are evicted least recently used
 * first), a slot's kernels before the rasteriser run as one CUDA graph after
 * its first frame, and a frame that overflows its slot is re-run once on a
 * slot sized to it. Results do not depend on what else is in flight. */
typedef struct hdsr_server hdsr_server;

#define HDSR_SERVER_NO_GRAPH 0x1u   /* launch every kernel directly */

typedef struct hdsr_server_config {
  uint64_t hbm_budget_bytes;    /* resident scenes + slots, bytes (> 0) */
  uint32_t max_in_flight;       /* frames running at once, 1..64 */
  uint32_t flags;               /* HDSR_SERVER_* */
} hdsr_server_config;

typedef struct hdsr_request {
  uint32_t scene_id;
  uint32_t color_format;        /* HDSR_COLOR_* */
  float uniforms[64];           /* hdsr_write_tile_splat_frame_uniforms: gives the viewport */
  hdsr_output_views outputs;    /* caller-owned device images of that viewport */
} hdsr_request;

typedef struct hdsr_request_result {
  int32_t status;               /* hdsr_status of the frame */
  uint32_t reruns;              /* overflow re-runs on a larger slot */
  uint64_t total_pairs;
  double submit_ms, start_ms, done_ms;  /* host clock, ms since the server was created */
} hdsr_request_result;

typedef struct hdsr_server_stats {
  uint64_t budget_bytes, scene_bytes, slot_bytes;
  uint32_t scenes, slots, graphs, evictions;
  uint64_t completed, reruns;
} hdsr_server_stats;

hdsr_status hdsr_server_create(const hdsr_server_config* cfg, hdsr_server** out);
void hdsr_server_destroy(hdsr_server* s);
/* Registers resident device arrays (borrowed; the caller keeps them alive
 * and unchanged while the server uses them). Counted against the budget.
 * Synchronises the legacy default stream first (uploads still in flight). */
hdsr_status hdsr_server_add_scene(hdsr_server* s, uint32_t scene_id, const hdsr_scene_views* scene);
/* Queues a request; returns at once with a ticket. Its frame starts after
 * all work issued to the legacy default stream before the call (e.g. the
 * allocation and clearing of its outputs); work on other streams that writes
 * its outputs or scene must be complete. */
hdsr_status hdsr_server_submit(hdsr_server* s, const hdsr_request* req, uint64_t* ticket);
/* Blocks until the ticket's frame is complete on the device. */
hdsr_status hdsr_server_wait(hdsr_server* s, uint64_t ticket, hdsr_request_result* result);
hdsr_status hdsr_server_query(hdsr_server* s, hdsr_server_stats* stats);
const char* hdsr_server_last_error(const hdsr_server* s);

/* Per-tile splat counts of a projected frame (the counts of count_tile_refs)
 * without any device allocation and without a handle. No reference
 * counterpart: the reference only counts inside its full pipeline.
 *   tile_boxes: device u32 tile boxes (u8 x0, y0, x1, y1; 0xFFFFFFFF =
 *     invisible), one every box_stride_words words, tile_boxes pointing at
 *     the first box (1: packed; 2: the handle's HDSR_BUF_CACHE_AUX stream;
 *     14: the reference's projection cache rows, whose box is word 7, so
 *     tile_boxes = cache + 7);
 *   tile_counts: device, tile_counts_len >= the plan's morton_tile_count
 *     words; written in Morton order, every other word set to 0.
 * Scratch is a static 256 KiB device array (a grid of <= 256 x 256 words):
 * tile grids beyond 255 x 255 tiles return HDSR_ERR_UNSUPPORTED. The first
 * call on a device (made with that device current) looks the scratch up and
 * keeps its address for the life of the process; make it before capturing a
 * stream. After cudaDeviceReset (or anything else that destroys the device's
 * primary context) the kept address is stale: do not call this function
 * again in that process. Nothing needs to start at zero. Calls
 * on one device share the scratch: calls that may run concurrently race.
 * Asynchronous on `stream`; returns launch errors only. */
hdsr_status hdsr_count_tile_refs_static(const uint32_t* tile_boxes, uint32_t box_stride_words,
                                        uint64_t splat_count, uint32_t tile_columns, uint32_t tile_rows,
                                        uint32_t* tile_counts, uint64_t tile_counts_len, void* stream);

/* ------------------------------------------------------------------------
 * Deferred passes over the G-buffer: the frame tail that
 * splatRenderer.ts:1042-1139 encodes after the compositor — screen-space
 * normal reconstruction (createScreenSpaceNormalsPass :317-385), the
 * bilateral normal filter (createBilateralNormalFilter :387-440), GTAO
 * (gtao.ts createGTAO: depth prefilter, main, denoise), bloom (bloom.ts
 * createBloom: threshold, horizontal and vertical blur), material curve LUTs
 * (materialCurves.ts), IBL (ibl.ts: BRDF LUT, equirect mip chain) and
 * deferred lighting (createDeferredLightingPass :442-556).
 * One hdsr_post per viewport size; its intermediate images live in the
 * handle, the inputs are the compositor's output views. */
typedef struct hdsr_post hdsr_post;

typedef struct hdsr_post_inputs {
  const void* color;        uint64_t color_pitch;     /* compositor colour, rgba16f or rgba32f */
  uint32_t color_format;    uint32_t _pad;            /* HDSR_COLOR_* */
  const float* depth;       uint64_t depth_pitch;     /* r32f NDC depth */
  const uint32_t* normal;   uint64_t normal_pitch;    /* r32u oct normal (source normals) */
  const uint32_t* material; uint64_t material_pitch;  /* rgba32u */
} hdsr_post_inputs;

/* Per-frame parameters; hdsr_post_default_params() fills the reference's
 * defaults (main.ts DEFAULT_SETTINGS :144-169, DEFAULT_GTAO_PARAMS,
 * DEFAULT_BLOOM_PARAMS, the constants of each pass's encode()). */
typedef struct hdsr_post_params {
  float view_proj_inverse[16];  /* mat4Inverse(lightingViewProj), column-major */
  float camera_pos[3];
  uint32_t normal_recovery_mode;/* 0 screen-space, 1 grazing recovery, 2 source normals */
  float grazing_start, grazing_end;   /* 0.45, 0.80 */
  float bilateral_spatial_sigma, bilateral_depth_sigma, bilateral_normal_sigma;  /* 3, 0.05, 1.5 */
  uint32_t bilateral_radius;          /* 3 (at most 8) */
  float proj[16];               /* projMatrix: GTAO projInfo */
  float view[16];               /* lightingViewMatrix: GTAO normal transform */
  float near_plane, far_plane;  /* 0.01, 100 */
  float ao_radius_world, ao_falloff_end, ao_intensity, ao_thickness;   /* 0.15, 1, 1.5, 1.81 */
  uint32_t ao_slices, ao_steps, frame_counter;                         /* 3, 4, 0 */
  float ao_denoise_strength;                                           /* 60 */
  float bloom_threshold, bloom_soft_knee;                              /* 0.8, 0.5 */
  float light_dir[3];
  float light_intensity, ambient_intensity;                            /* 3, 0.12 */
  uint32_t specular_only;
  float emissive_intensity, emissive_threshold;                        /* 3, 0.05 */
  float env_intensity, env_rotation, exposure;                         /* 1, 0, 1 */
  float fallback_roughness, fallback_metallic;                         /* 0.65, 0 (unused by the shader) */
} hdsr_post_params;

/* Intermediate images, readable with hdsr_post_get_buffer (dense rows). */
typedef enum hdsr_post_buffer_id {
  HDSR_POST_SCREEN_NORMALS = 0, /* u32 W*H: pack2x16float(oct), screen-space pass */
  HDSR_POST_NORMALS = 1,        /* u32 W*H: bilateral output (what GTAO and lighting read) */
  HDSR_POST_DEPTH_MIP0 = 2,     /* f32 W*H linear view depth */
  HDSR_POST_DEPTH_MIP1 = 3,     /* f32 ceil(W/2)*ceil(H/2), 2x2 min */
  HDSR_POST_DEPTH_MIP2 = 4,     /* f32 ceil(W/4)*ceil(H/4) */
  HDSR_POST_AO_RAW = 5,         /* rgba16f W*H: ao, bent-normal oct, 0 */
  HDSR_POST_AO = 6,             /* rgba16f W*H: denoised */
  HDSR_POST_BLOOM = 7,          /* rgba16f ceil(W/2)*ceil(H/2): after both blurs */
  HDSR_POST_BLOOM_H = 8,        /* rgba16f: after the horizontal blur */
  HDSR_POST_BRDF_LUT = 9,       /* u32 256*256: pack2x16float(scale, bias) */
  HDSR_POST_ENV = 10,           /* rgba16f equirect mip chain, level 0 first */
  HDSR_POST_CURVES = 11         /* u16 3*256: roughness, metalness, albedo LUTs (f16) */
} hdsr_post_buffer_id;

/* createGTAO / createBloom / createIBL / createMaterialCurves for one viewport.
 * Generates the BRDF LUT (ibl_brdf_lut.wgsl), the identity curves and the 1x1
 * placeholder environment (no IBL until hdsr_post_set_environment). */
hdsr_status hdsr_post_create(uint32_t width, uint32_t height, hdsr_post** out);
void hdsr_post_destroy(hdsr_post* p);
void hdsr_post_default_params(hdsr_post_params* params);
/* IBLResources.loadEquirectRGBA (ibl.ts:107-149): level 0 as rgba16f texels
 * (host memory, w*h*4 halves), the mip chain by 2x2 box filter
 * (ibl_mipgen.wgsl). width or height 0 restores the placeholder. */
hdsr_status hdsr_post_set_environment(hdsr_post* p, const uint16_t* rgba16f, uint32_t width, uint32_t height,
                                      void* stream);
/* MaterialCurves.update (materialCurves.ts:100-104): (contrast, brightness,
 * gamma) for roughness, metalness and albedo, generated on the host. */
hdsr_status hdsr_post_set_material_curves(hdsr_post* p, const float curves[9]);
/* The frame tail: normals -> bilateral -> GTAO (prefilter, main, denoise),
 * bloom on the handle's side stream, then lighting into `lit` (rgba16f,
 * lit_pitch bytes per row). Asynchronous on `stream`. */
hdsr_status hdsr_post_encode(hdsr_post* p, const hdsr_post_inputs* in, const hdsr_post_params* params,
                             void* lit, uint64_t lit_pitch, void* stream);
hdsr_status hdsr_post_get_buffer(hdsr_post* p, hdsr_post_buffer_id id, void** device_ptr, uint64_t* bytes);
/* With profiling on, passes run on one stream between CUDA events; times of
 * the last encode in ms: ss_normals, bilateral, gtao_prefilter, gtao_main,
 * gtao_denoise, bloom, lighting. */
hdsr_status hdsr_post_set_profiling(hdsr_post* p, int enable);
hdsr_status hdsr_post_pass_times(hdsr_post* p, float ms[7]);
const char* hdsr_post_last_error(const hdsr_post* p);

#ifdef __cplusplus
}
#endif
#endif /* HDSR_H */
