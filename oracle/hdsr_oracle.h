/*
 * hdsr_oracle.h — CPU restatement of the reference compute compositor.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path:
 * only the test suite, the smoke check and the benchmark's CPU-baseline leg
 * load it. The product never links or calls it, and it is not a fallback.
 *
 * What it restates (reference paths inside lyonsno/hybrid-differentiable-
 * deferred-splat-mesh-renderer):
 *   src/shaders/gpu_project_splats.wgsl:75-358          project_splats
 *   src/shaders/gpu_classify_large_splats.wgsl:33-66     classify_large_splats
 *   src/shaders/gpu_tile_splat_composite.wgsl:33-119     morton, count, scatter
 *   src/shaders/gpu_large_splat_scatter.wgsl:52-89       cooperative scatter
 *   src/shaders/gpu_prefix_sum.wgsl:14-85                3-pass exclusive scan
 *   src/shaders/gpu_tile_classify.wgsl:44-86             small / hot tile lists
 *   src/shaders/gpu_tile_depth_sort.wgsl:28-79           per-tile bitonic
 *   src/shaders/gpu_tile_bucket_sort.wgsl:41-144         hot-tile cascade
 *   src/shaders/gpu_tile_chunk_sort.wgsl:36-97           chunk sort
 *   src/shaders/gpu_tile_splat_composite.wgsl:162-370    composite
 *   src/gpuTileSplatCompositor.ts:109-139                 plan
 *   src/splatSort.ts:32-55,178-195                        CPU depth sort (baseline)
 *   src/gpuSortPrototype.ts:120-163                       sortedIndices order
 *
 * Parity status: the reference is TypeScript + WGSL executed by a browser's
 * WebGPU implementation, which cannot run on this machine. The CPU depth sort
 * and the compositor's constants are pinned against the reference's own unit
 * tests (tests/cpuDepthSort.test.ts, tests/renderer/
 * computeCompositorLifecycle.test.mjs); the compositor passes themselves
 * (tile counts, offsets, per-tile order, pixels) are "parity unpinned": no
 * reference test or fixture fixes them. This file is a transcription of the
 * shaders, checked three ways: by review against the shader text; by
 * independent NumPy restatements written from the same shaders, which the
 * CPU test suite compares with this file bit for bit (the projection cache
 * row and depth at SH degrees 0-3 with baked and detail normals, emissive and
 * material; the f32 composite's colour, alpha and G-buffer votes; the f16
 * composite's colour and alpha); and by property tests (known-answer
 * vectors, exp/log accuracy, Morton codes, bucket = k20 >> 13, the 4096/4097
 * hot-tile threshold, ties, near-plane depths, every tile in (depth, rank)
 * order, the FP64 twin). The projected covariance is also checked against
 * the reference's own EWA witness (rendererFidelityProbes/conicProjection.js).
 *
 * Canonical order. The reference bins with atomics, so its per-tile order is
 * not reproducible when keys tie. This restatement fixes every such choice
 * (each equals one of the orders the reference can produce):
 *   - small tiles (2..4096 entries): ascending (depth bits, sortRank);
 *   - hot tiles (>4096): entries in bucket order, within a bucket ascending
 *     (depth bits, sortRank) (the reference's atomic cursor leaves it open);
 *     packed greedily into 4096-entry chunks, each chunk ascending (depth
 *     bits, sortRank). Because this log is monotone over every positive
 *     float, the bucket is monotone in depth and the result equals ascending
 *     (depth bits, sortRank) over the whole tile; tiles with a negative,
 *     NaN or infinite depth, or a log range below 1e-10, put every entry in
 *     bucket 0 and reach the same order;
 *   - tile lists and chunk lists in ascending Morton order;
 *   - no caps: the reference's 65,535 large-splat cap, tile-ref budget drop,
 *     overflow-scratch skip and 1,024-chunk cap are reported as flags, not
 *     applied.
 *
 * Arithmetic. Compiled with -ffp-contract=off; every fused multiply-add is an
 * explicit fmaf(). exp/log are this project's own (orc_expf/orc_logf below),
 * because WGSL leaves their precision to the implementation.
 */
#ifndef HDSR_ORACLE_H
#define HDSR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference-cap flags reported in orc_frame.flags. */
#define ORC_FLAG_LARGE_SPLAT_CAP   1u  /* >65,535 large splats (classify_large_splats:52)  */
#define ORC_FLAG_REF_BUDGET_DROP   2u  /* total refs > maxTotalTileRefs (scatter_tile_refs:114)  */
#define ORC_FLAG_OVERFLOW_SKIP     4u  /* bucket scratch overflow skip (bucket_sort:54) */
#define ORC_FLAG_CHUNK_CAP         8u  /* >1,024 chunks (bucket_sort:126,138)           */
#define ORC_FLAG_BUCKET_KEY_MISMATCH 16u /* bucket != k20>>13 (must never happen)           */

typedef struct {
  uint32_t splat_count;
  uint32_t sh_degree;
  const float* positions;       /* N*3                                  */
  const float* scales;          /* N*3, log scale                       */
  const float* rotations;       /* N*4, wxyz                            */
  const float* opacities;       /* N, activated                         */
  const uint32_t* sorted_indices; /* N, back-to-front splat ids         */
  const uint32_t* material;     /* N, f16x2 (roughness, metalness)      */
  const float* normals;         /* normals_len floats or NULL           */
  uint64_t normals_len;
  const float* sh_data;         /* N*(6+3K): dc3 | sh 3K | emissive3    */
} orc_scene;

typedef struct {
  /* intermediates, caller-allocated */
  uint32_t* proj_cache;         /* N*14 (reference AoS layout)          */
  uint32_t* depth;              /* N                                    */
  uint32_t* tile_counts;        /* M                                    */
  uint32_t* tile_offsets;       /* M                                    */
  uint32_t* tile_entries;       /* entries_cap                          */
  uint64_t entries_cap;
  uint32_t* chunk_ranges;       /* 2*chunk_cap (start, count)           */
  uint32_t chunk_cap;
  /* results */
  uint64_t total_pairs;
  uint32_t small_tiles;
  uint32_t hot_tiles;
  uint32_t total_chunks;
  uint32_t large_splats;
  uint32_t flags;
  uint32_t composite_f16;       /* 1: the f16 composite variant (gpu_tile_splat_composite_f16.wgsl) */
  /* outputs, W*H pixels each (may be NULL to skip the composite) */
  uint16_t* out_color;          /* rgba16f, 4 halves per pixel           */
  float* out_depth;             /* r32f                                  */
  uint32_t* out_normal;         /* r32u: pack2x16float(oct)              */
  uint32_t* out_material;       /* rgba32u, 4 words per pixel            */
} orc_frame;

/* --- arithmetic ---------------------------------------------------------- */
float orc_expf(float x);
float orc_composite_expf(float x);       /* the deferred passes' weight exp */
float orc_splat_expf(float x);           /* the composites' exp (power in (-4, 0]) */
float orc_splat_exp_parts(float x, uint32_t* kb); /* its p and k << 23 */
float orc_logf(float x);
uint16_t orc_f32_to_f16_rne(float f);     /* pack2x16float rounding */
uint16_t orc_f64_to_f16_rne(double x);    /* binary16 round-to-nearest-even of a double */
float orc_f16_to_f32(uint16_t h);
uint16_t orc_f32_to_f16_trunc(float f);   /* splats.ts:431-442 f32ToF16 */
uint32_t orc_morton(uint32_t x, uint32_t y);

/* --- plan (gpuTileSplatCompositor.ts:109-139) ---------------------------- */
/* out: [W, H, tile, cols, rows, tileCount, M, N, maxTotalTileRefs] */
void orc_plan(uint32_t W, uint32_t H, uint32_t tile, uint32_t N, double mult, uint32_t out[9]);

/* --- passes --------------------------------------------------------------- */
void orc_project(const float* U, const orc_scene* s, uint32_t* proj_cache, uint32_t* depth,
                 int threads);
void orc_count_tile_refs(const float* U, uint32_t N, const uint32_t* proj_cache, uint32_t M,
                         uint32_t* tile_counts);
void orc_exclusive_scan(const uint32_t* in, uint32_t n, uint32_t* out);
/* Full canonical frame; returns 0, or -2 when entries_cap/chunk_cap are too
 * small (total_pairs/total_chunks are filled so the caller can retry). */
int orc_render_frame(const float* U, const orc_scene* s, orc_frame* f, int threads);
/* The 20-bit log-depth keys: for each tile in ascending Morton order, its
 * entries in ascending (k20, sortRank); keys[i] = morton<<20 | k20, where
 * k20 is the hot-tile bucket mapping scaled to 2^20 (bucket == k20 >> 13). */
int orc_sorted_keys20(const float* U, uint32_t N, const uint32_t* proj_cache,
                      const uint32_t* depth, uint64_t* keys, uint32_t* values, uint64_t cap,
                      uint64_t* total);
/* Composite only, from existing cache/entries (encodeCompositeOnly). */
void orc_composite(const float* U, const uint32_t* proj_cache, const uint32_t* depth,
                   const uint32_t* tile_counts, const uint32_t* tile_offsets,
                   const uint32_t* tile_entries, orc_frame* f, int threads);

/* --- FP64 accuracy judge: same passes and order, double arithmetic, no f16
 * quantisation of the cache. Writes rgba as 4 doubles per pixel. */
int orc_render_frame_f64(const float* U, const orc_scene* s, const uint32_t* tile_counts,
                         const uint32_t* tile_offsets, const uint32_t* tile_entries,
                         double* out_rgba, int threads);

/* Per sortRank, the FP64 screen-space parameters of the twin: cx, cy, ia,
 * ib, ic, opacity, r, g, b, visible (10 doubles). */
void orc_project_f64(const float* U, const orc_scene* s, double* out, int threads);

/* --- CPU depth sort baseline (splatSort.ts:32-55,178-195) ----------------
 * returns 0, -1 on a non-finite depth (the reference throws RangeError). */
int orc_sort_back_to_front(const float* positions, uint32_t n, const float* view,
                           uint32_t* order_out, int threads);
/* gpuSortPrototype order: f32 keys -viewZ, descending, ties by id. */
int orc_gpu_sort_prototype_order(const float* positions, uint32_t n, const float* view,
                                 uint32_t* order_out);

/* --- array helpers for tests -------------------------------------------- */
void orc_expf_n(const float* in, float* out, uint64_t n);
void orc_logf_n(const float* in, float* out, uint64_t n);
void orc_f16_rne_n(const float* in, uint16_t* out, uint64_t n);
void orc_f16_trunc_n(const float* in, uint16_t* out, uint64_t n);
void orc_f16_to_f32_n(const uint16_t* in, float* out, uint64_t n);
void orc_f64_to_f16_n(const double* in, uint16_t* out, uint64_t n);
void orc_composite_expf_n(const float* in, float* out, uint64_t n);
void orc_splat_expf_n(const float* in, float* out, uint64_t n);
void orc_splat_exp_parts_n(const float* in, float* p, uint32_t* kb, uint64_t n);

/* ---- deferred frame tail (hdsr_post_oracle.c) ---- */
typedef struct orp_inputs {
  int W, H;
  const float* color;        /* W*H*4, rgba as f32 (the compositor's f16 decoded) */
  const float* depth;        /* W*H */
  const uint32_t* normal;    /* W*H source oct normals */
  const uint32_t* material;  /* W*H*4 */
} orp_inputs;

/* the same fields, order and meaning as hdsr_post_params (include/hdsr.h) */
typedef struct orp_params {
  float view_proj_inverse[16];
  float camera_pos[3];
  uint32_t normal_recovery_mode;
  float grazing_start, grazing_end;
  float bilateral_spatial_sigma, bilateral_depth_sigma, bilateral_normal_sigma;
  uint32_t bilateral_radius;
  float proj[16];
  float view[16];
  float near_plane, far_plane;
  float ao_radius_world, ao_falloff_end, ao_intensity, ao_thickness;
  uint32_t ao_slices, ao_steps, frame_counter;
  float ao_denoise_strength;
  float bloom_threshold, bloom_soft_knee;
  float light_dir[3];
  float light_intensity, ambient_intensity;
  uint32_t specular_only;
  float emissive_intensity, emissive_threshold;
  float env_intensity, env_rotation, exposure;
  float fallback_roughness, fallback_metallic;
} orp_params;

typedef struct orp_env {
  const uint16_t* texels;    /* rgba16f mip chain, level 0 first */
  int w, h, levels;
  int lw[16], lh[16];
  uint32_t offset[16];       /* texel offset of each level */
} orp_env;

void orp_ss_normals(const orp_inputs* in, const orp_params* q, uint32_t* out);
void orp_bilateral(const orp_inputs* in, const orp_params* q, const uint32_t* ssn, uint32_t* out);
void orp_gtao_prefilter(const orp_inputs* in, const orp_params* q, float* mip0, float* mip1, float* mip2);
void orp_gtao_main(const orp_inputs* in, const orp_params* q, const float* mip0, const float* mip1,
                   const float* mip2, const uint32_t* normals, uint16_t* ao_raw);
void orp_gtao_denoise(const orp_inputs* in, const orp_params* q, const uint16_t* ao_raw, const float* mip0,
                      uint16_t* ao);
void orp_bloom_threshold(const orp_inputs* in, const orp_params* q, uint16_t* out);
void orp_bloom_blur(int hw, int hh, const uint16_t* src, uint16_t* dst, float dirx, float diry, float tx, float ty);
void orp_lighting(const orp_inputs* in, const orp_params* q, const uint32_t* normals, const uint16_t* ao,
                  const orp_env* env, const uint32_t* brdf, const uint16_t* bloom, const uint16_t* curves,
                  uint16_t* lit);
void orp_brdf_lut(int y0, int y1, uint32_t* out);
void orp_env_mip(const uint16_t* src, int sw, int sh, uint16_t* dst, int dw, int dh);
void orp_curve_lut(float contrast, float brightness, float gamma, uint16_t out[256]);
float orp_atan2(float y, float x);
float orp_asin(float x);
float orp_sin(float x);
float orp_cos(float x);
float orp_log2(float x);
float orp_pow(float x, float y);
void orc_morton_n(const uint32_t* x, const uint32_t* y, uint32_t* out, uint64_t n);
void orc_bucket_key20_n(const uint32_t* depth_bits, uint64_t n, uint32_t dmin, uint32_t dmax,
                        uint32_t* buckets, uint32_t* keys);

#ifdef __cplusplus
}
#endif
#endif
