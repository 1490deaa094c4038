/*
 * gs3d — GB300-native tiled Gaussian-splatting pass, C ABI.
 *
 * This library replaces the data path behind the reference's
 * TiledGaussianPipeline (src/renderer/pipeline/TiledGaussianPipeline.ts:39-484),
 * whose only caller is GaussianPass.updateBefore
 * (src/renderer/GaussianPass.ts:710-805). Every entry point below names the
 * reference interface it stands in for. The ABI uses plain C types and
 * pointers only: device buffers are CUDA device pointers, the stream is a
 * cudaStream_t passed as void*.
 *
 * Threading: a pipeline is used by one host thread at a time; all work is
 * enqueued asynchronously on the stream given to gs3d_pipeline_render and
 * never blocks the caller, except gs3d_pipeline_read_stats (a small
 * synchronous readback, the analogue of readStats()).
 *
 * Errors: every call returns a gs3d_status. No C++ exception crosses the ABI.
 * gs3d_pipeline_last_error() returns a message for the last failure.
 * Device-side conditions (intersection overflow, a bounded device wait that
 * expired) are reported through the 16-byte output state and the stats.
 */
#ifndef GS3D_H
#define GS3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GS3D_ABI_VERSION 4u

typedef enum gs3d_status {
  GS3D_OK = 0,
  /* TypeError in the reference: wrong formats, null pointers, bad enums. */
  GS3D_ERROR_INVALID_ARGUMENT = 1,
  /* RangeError in the reference (e.g. TiledGaussianPipeline.ts:294-296). */
  GS3D_ERROR_RANGE = 2,
  /* Error("must be prepared before rendering"), TiledGaussianPipeline.ts:324-329. */
  GS3D_ERROR_NOT_PREPARED = 3,
  /* "allocation-failed" output status (types.ts:209-233). */
  GS3D_ERROR_OUT_OF_MEMORY = 4,
  /* Any other CUDA runtime failure. */
  GS3D_ERROR_CUDA = 5,
  /* A bounded device-side wait (scan/sort look-back) gave up; the frame is invalid. */
  GS3D_ERROR_DEVICE_TIMEOUT = 6,
  /* The build does not support the requested option. */
  GS3D_ERROR_UNSUPPORTED = 7,
  /* Not an error: an asynchronous read-back has not landed yet. */
  GS3D_NOT_READY = 8
} gs3d_status;

/* DepthSortMode (types.ts:11). */
typedef enum gs3d_depth_sort_mode { GS3D_DEPTH_FLOAT32 = 0, GS3D_DEPTH_PACKED16 = 1 } gs3d_depth_sort_mode;
/* AntialiasMode (types.ts:12). */
typedef enum gs3d_antialias_mode { GS3D_ANTIALIAS_COMPENSATED = 0, GS3D_ANTIALIAS_CLASSIC = 1 } gs3d_antialias_mode;
/* GaussianBoundaryPolicy (types.ts:17). */
typedef enum gs3d_boundary_policy {
  GS3D_BOUNDARY_CLIP = 0,
  GS3D_BOUNDARY_REPEAT_X = 1,
  GS3D_BOUNDARY_REPEAT_Y = 2
} gs3d_boundary_policy;
/* Rasterizer arithmetic. FP32 is the reference's form. EXACT is FP32 with the
 * deterministic math library and no FMA contraction (bit-identical to the CPU
 * restatement). HALF2 evaluates each pixel's Gaussian exponent in packed
 * half2 (from the splat's Cholesky factor about the patch centre, two pixels
 * per instruction), with its threshold test, alpha clamp and exp2, the colour
 * stored in half; transmittance and colour accumulation stay FP32 (the
 * periodic-boundary variant keeps the exponent in FP32). The f16 exponent
 * relies on the screen-space low-pass filter: with filter_variance below
 * 0.05 a HALF2 render evaluates as FP32. */
/* Projection arithmetic. FP32 is the reference's (ProjectionStage.ts, bit-exact
 * with the CPU restatement). FP64 has no counterpart in the reference: it
 * evaluates the model-view mean transform in double (far-origin scenes) and
 * redoes the covariance -> determinant -> conic chain in double for splats
 * that are near-singular in FP32; results then follow the FP64 oracle, not the
 * FP32 restatement. */
typedef enum gs3d_projection_precision {
  GS3D_PROJECTION_FP32 = 0,
  GS3D_PROJECTION_FP64 = 1
} gs3d_projection_precision;

typedef enum gs3d_raster_precision {
  GS3D_RASTER_FP32 = 0,
  GS3D_RASTER_EXACT = 1,
  GS3D_RASTER_HALF2 = 2
} gs3d_raster_precision;
/* Colour target format: the reference's rgba16float texture, or rgba32float. */
typedef enum gs3d_color_format { GS3D_COLOR_RGBA16F = 0, GS3D_COLOR_RGBA32F = 1 } gs3d_color_format;

/* GaussianData packed buffers (src/renderer/GaussianData.ts:10-33,108-138),
 * compact geometry + rgb8e8 SH, as produced by the Rust backend's
 * encode_attributes (rust/gaussian-backend/src/engine.rs:1801-1891).
 * All pointers are device pointers owned by the caller (the Store); the
 * pipeline holds them like the reference's lease (GaussianData.retain) until
 * gs3d_pipeline_update_data or gs3d_pipeline_destroy. */
typedef struct gs3d_gaussian_data {
  uint32_t count;        /* slot capacity */
  uint32_t active_count; /* ordinals drawn; <= count */
  uint32_t sh_degree;    /* 0..3 */
  uint32_t reserved;
  const void* means;           /* float32[count][4]: xyz, objectId or -1 */
  const void* scales_opacity;  /* uint32[count][2]: f16 ln-scales + f16 opacity */
  const void* rotations;       /* uint32[count]: oct101012 */
  const void* sh_coefficients; /* uint32[count * (deg+1)^2 + count]: rgb8e8 + active-slot tail */
} gs3d_gaussian_data;

/* Constructor options of TiledGaussianPipeline (TiledGaussianPipeline.ts:65-85)
 * and the GaussianRenderDomain (types.ts:20-25). Zero-initialise, then call
 * gs3d_pipeline_desc_defaults() to get the reference's defaults. */
typedef struct gs3d_pipeline_desc {
  uint32_t abi_version;           /* GS3D_ABI_VERSION */
  int32_t device;                 /* CUDA device ordinal */
  uint32_t depth_sort_mode;       /* gs3d_depth_sort_mode, default float32 */
  uint32_t antialias_mode;        /* gs3d_antialias_mode, default compensated */
  uint64_t intersection_capacity; /* records; default 262,144 */
  float background[4];            /* default transparent black */
  uint32_t max_rasterized_splats_per_tile; /* 0 = null (uncapped) */
  uint32_t raster_chunk_size;     /* default 8192; 0 = null (single-block tiles) */
  uint32_t subpixel_sample_culling; /* default 1 */
  float raster_transmittance_threshold; /* default 1e-4, in (0,1) */
  float depth_alpha_threshold;    /* default 0.95, in [0,1] */
  float filter_variance;          /* default 0.3 */
  float invalid_depth_value;      /* default 1 */
  uint32_t boundary_policy;       /* gs3d_boundary_policy, default clip */
  uint32_t raster_precision;      /* gs3d_raster_precision, default FP32 */
  uint32_t depth_encoding;        /* 0: default device depth node; 1: raw alpha-weighted depth */
  uint32_t raster_stats;          /* rasterStats (types.ts:283): per-pixel work counters, default 0 */
  uint32_t projection_precision;  /* gs3d_projection_precision, default FP32 */
} gs3d_pipeline_desc;

/* Per-frame camera state: what FrameUniforms.update and ObjectFrameState.update
 * produce on the CPU (FrameUniforms.ts:41-58, ObjectFrameState.ts:78-119). */
typedef struct gs3d_camera {
  float projection[16];   /* column-major projectionMatrix */
  float view[16];         /* column-major matrixWorldInverse */
  float depth_near;       /* depthRange (defaults to camera near/far) */
  float depth_far;
  const float* object_table; /* HOST pointer: object_count x 40 floats */
  uint32_t object_count;
  uint32_t reserved;
} gs3d_camera;

/* Render targets: device pointers, row-major width x height pixels. */
typedef struct gs3d_targets {
  void* color;          /* rgba16f (uint16 x4) or rgba32f (float x4) */
  uint32_t color_format; /* gs3d_color_format */
  uint32_t reserved;
  float* depth;         /* float32 per pixel, or NULL (outputDepth = false) */
} gs3d_targets;

/* readStats() (IntersectionStage.ts:197-213, types.ts:94-103). */
typedef struct gs3d_stats {
  uint32_t visible_gaussian_count;
  uint32_t intersection_count;
  uint32_t requested_intersections; /* saturates at 0xffffffff */
  uint32_t overflow;
  uint64_t intersection_capacity;
  uint32_t device_error;            /* nonzero: a bounded device wait expired */
  uint32_t reserved;
  /* rasterStats counters (TileRasterizer.ts:904-927), zero unless enabled:
   * samples examined and blended by all pixels, in-bounds pixels of nonempty
   * tiles, and those whose transmittance fell below the threshold. */
  uint64_t raster_checked;
  uint64_t raster_blended;
  uint64_t raster_pixels;
  uint64_t raster_alpha_stopped;
  /* The 16-byte output state after the render (intersections.ts:114-133,
   * read back by GaussianPass.ts:1019-1079): attempt, version (the attempt
   * of the last complete image, 0 if none), demand, overflow. */
  uint32_t output_state[4];
} gs3d_stats;

/* getResources() (TiledGaussianPipeline.ts:391-406, types.ts:174-193).
 * Device pointers into the pipeline's workspaces, valid until the next
 * resize/update/destroy. Record buffers are structure-of-arrays here: the
 * reference's uvec2 (key, id) records are split into key and id arrays. */
typedef struct gs3d_resources {
  const float* projected_mean;     /* float4 per active ordinal: x, y, depth, opacity */
  const float* projected_conic;    /* float4: conic xyz, radiusX + 512 radiusY */
  const float* projected_color;    /* float4: rgb, bitcast(slot ^ 0x3f800000) */
  const uint32_t* tile_counts;
  const uint32_t* visible_offsets;
  const uint32_t* depth_sorted_keys; /* depth key per visible rank */
  const uint32_t* depth_sorted_ids;  /* active ordinal per visible rank */
  const uint32_t* depth_ordered_tile_counts;
  const uint32_t* intersection_offsets;
  const uint32_t* dispatch_state;    /* uvec4: count, total, radix blocks, overflow */
  const uint32_t* visible_state;     /* uvec4: visible, visible, radix blocks, 0 */
  const uint32_t* sorted_tile_ids;   /* tile id per sorted intersection */
  const uint32_t* sorted_gaussian_ids; /* active ordinal per sorted intersection */
  const uint32_t* tile_offsets;      /* tilesX*tilesY + 1 */
  const uint32_t* output_state;      /* uvec4: attempt, version, demand, overflow */
  uint32_t active_count;  /* items of the last render (a batch pads each view to 256) */
  uint32_t tiles_x;       /* prepared frame (single-view render) */
  uint32_t tiles_y;
  uint32_t total_tiles;   /* tiles of the last render over all views */
  uint64_t intersection_capacity;
} gs3d_resources;

typedef struct gs3d_pipeline gs3d_pipeline;

/* Library identity. */
uint32_t gs3d_abi_version(void);
const char* gs3d_status_string(gs3d_status status);

/* Fill *desc with the reference defaults (GaussianPass.ts:170-256). */
void gs3d_pipeline_desc_defaults(gs3d_pipeline_desc* desc);

/* new TiledGaussianPipeline(...) (TiledGaussianPipeline.ts:65-163). */
gs3d_status gs3d_pipeline_create(const gs3d_pipeline_desc* desc, const gs3d_gaussian_data* data,
                                 gs3d_pipeline** out);
/* dispose() (TiledGaussianPipeline.ts:408-425). Safe on NULL. */
void gs3d_pipeline_destroy(gs3d_pipeline* pipeline);

/* updateData(data) (TiledGaussianPipeline.ts:203-218). */
gs3d_status gs3d_pipeline_update_data(gs3d_pipeline* pipeline, const gs3d_gaussian_data* data);
/* resizeIntersections(capacity) (TiledGaussianPipeline.ts:220-231). */
gs3d_status gs3d_pipeline_resize_intersections(gs3d_pipeline* pipeline, uint64_t capacity);
/* prepareFrame(width, height) (TiledGaussianPipeline.ts:286-322): RANGE if a
 * tile axis exceeds 65,535. Camera state comes with each render call. */
gs3d_status gs3d_pipeline_prepare_frame(gs3d_pipeline* pipeline, uint32_t width, uint32_t height);
/* render(attempt, resetValid) (TiledGaussianPipeline.ts:324-341): enqueue the
 * whole pass on `stream`. NOT_PREPARED before prepare_frame. */
gs3d_status gs3d_pipeline_render(gs3d_pipeline* pipeline, const gs3d_camera* camera, uint32_t attempt,
                                 int reset_valid, const gs3d_targets* targets, void* stream);
/* One view of a batch: a scene, a camera, a size and its targets. */
typedef struct gs3d_view {
  const gs3d_gaussian_data* data;
  const gs3d_camera* camera;
  uint32_t width;
  uint32_t height;
  gs3d_targets targets;
} gs3d_view;

/* Launch-shape tuning (no counterpart in the reference, whose dispatch shape
 * is fixed). views_per_launch: a batch of more
 * views runs as consecutive launch sequences of at most that many views on the
 * same stream (0 = the whole batch at once); read_stats then reports their
 * totals (visible and intersection counts summed, requested = the largest
 * sequence's demand, overflow if any sequence overflowed), the output state
 * covers the whole batch, and get_resources and batch_layout describe the
 * last sequence. tile_digit_bits: the widest digit of the tile sort, 4..8.
 * work_order: 1 = rasterize tiles heaviest first, 0 = in tile order. None of
 * these three changes what a batch produces.
 * tile_size: pixels per tile side of batched renders (render_batch, captured
 * graphs, autotune): 8, 16 or 32, 0 = the reference's 16 (constants.ts:1).
 * The rasterizer's block follows the tile (one warp per 8x8 patch in the
 * FP32 and half2 forms, one thread per pixel in EXACT). The EXACT image does
 * not depend on it (the tile test is conservative for every pixel of the
 * tile); the tile ids, counts, intersection records and tile offsets do, and
 * so do the raster chunk split and maxRasterizedSplatsPerTile, which act per
 * tile, and the visible set, by splats that reach a tile only where it
 * extends past the image edge (they cover no pixel). Single-view
 * gs3d_pipeline_render always uses 16.
 * raster_pixels_per_lane: the FP32 and half2 rasterizers' block shape, 2 (a
 * warp per 8x8 patch of the tile, each lane two pixels of one column) or 4
 * (a warp per 8x16 patch, half the warps per tile; 8-pixel tiles keep 2);
 * 0 = 2. The EXACT form has one thread per pixel. The image of the fast
 * forms stays within their tolerance (their transmittance test runs per
 * group of 32 records of a warp's walk, which the patch regroups).
 * Setting a tuning releases captured graphs. */
typedef struct gs3d_tuning {
  uint32_t views_per_launch;       /* default 0 */
  uint32_t tile_digit_bits;        /* default 8 */
  uint32_t work_order;             /* default 1 */
  uint32_t tile_size;              /* default 0 (16) */
  uint32_t raster_pixels_per_lane; /* default 0 (2) */
  uint32_t reserved[3];
} gs3d_tuning;

gs3d_status gs3d_pipeline_set_tuning(gs3d_pipeline* pipeline, const gs3d_tuning* tuning);
gs3d_status gs3d_pipeline_get_tuning(gs3d_pipeline* pipeline, gs3d_tuning* tuning);

/* Times the batch under candidate tunings (coordinate descent: tile size 8
 * and 32 against 16, four pixels per lane against two, views per launch
 * halving from the batch size, tile digit width 7..4, then the work order; `trials` timed batches each after
 * one untimed one), keeps the fastest and returns it with its milliseconds
 * per batch. The views' targets receive the renders. GS3D_ERROR_RANGE if the
 * intersection capacity cannot hold the batch at 16-pixel tiles; a tile size
 * whose batch overflows the capacity is skipped. */
gs3d_status gs3d_pipeline_autotune(gs3d_pipeline* pipeline, const gs3d_view* views, uint32_t count, uint32_t trials,
                                   gs3d_tuning* best, double* best_ms, void* stream);

/* Batched rendering (an extension; the reference renders one camera per
 * pass): the views run through one launch sequence (or several, see
 * gs3d_tuning.views_per_launch). Views are
 * concatenated: view v owns items [item_base[v], item_base[v] + active) and
 * global tile ids [tile_base[v], tile_base[v+1]); each view's tiles hold
 * exactly the records, order and image a single-view render of that view
 * produces. The batch shares one intersection workspace: on overflow no view
 * is published and the output state reports the batch's demand. Consecutive
 * views whose gs3d_gaussian_data names the same buffers (means, shape,
 * rotations, SH) with the same counts and SH degree form a view group: the
 * projection decodes each splat once for the whole group, so order views by
 * scene. */
gs3d_status gs3d_pipeline_render_batch(gs3d_pipeline* pipeline, const gs3d_view* views, uint32_t count,
                                       uint32_t attempt, int reset_valid, void* stream);
/* Capture the batched pass for these views (scenes, sizes, targets and object
 * counts fixed) into CUDA graphs; gs3d_pipeline_launch_graph then replays it
 * with new cameras: one graph launch per frame instead of ~28 kernel launches
 * per launch sequence.
 * `stream` must be a non-default stream; profiling must be off. Any
 * update_data/resize_intersections drops the graphs. Two graph instances
 * alternate over two staging buffers, so the host prepares frame N+1 while
 * frame N runs. */
gs3d_status gs3d_pipeline_capture_graph(gs3d_pipeline* pipeline, const gs3d_view* views, uint32_t count,
                                        void* stream);
gs3d_status gs3d_pipeline_launch_graph(gs3d_pipeline* pipeline, const gs3d_camera* cameras, uint32_t count,
                                       uint32_t attempt, int reset_valid, void* stream);
/* item_base/tile_base of the last render (count + 1 entries each). */
gs3d_status gs3d_pipeline_batch_layout(gs3d_pipeline* pipeline, uint32_t* item_base, uint32_t* tile_base,
                                       uint32_t capacity, uint32_t* count);

/* readStats() (TiledGaussianPipeline.ts:353-366): synchronises the stream of
 * the last render. */
gs3d_status gs3d_pipeline_read_stats(gs3d_pipeline* pipeline, gs3d_stats* stats);
/* readStats() without blocking, the way GaussianPass reads its output state
 * (GaussianPass.ts:1019-1079: one read-back in flight, resolved when the GPU
 * has passed it). request_stats enqueues a copy of the last render's counters
 * into pinned memory owned by the pipeline, on `stream` (NULL: the last
 * render's stream) after the last render, and returns at once;
 * GS3D_ERROR_UNSUPPORTED if a read-back is already in flight. poll_stats
 * returns GS3D_NOT_READY while the copy is in flight (wait = 0), or waits
 * for it (wait != 0), then fills *stats exactly as read_stats does (including
 * GS3D_ERROR_DEVICE_TIMEOUT) and ends the read-back. */
gs3d_status gs3d_pipeline_request_stats(gs3d_pipeline* pipeline, void* stream);
gs3d_status gs3d_pipeline_poll_stats(gs3d_pipeline* pipeline, gs3d_stats* stats, int wait);

/* Failure detection (no counterpart in the reference, whose GPU waits cannot
 * hang: WebGPU has no inter-workgroup spin). The compaction and scan kernels
 * wait on their predecessors' look-back status words; a wait that spends
 * `polls` polls (with nanosleep back-off) on one word gives up, the frame
 * reports GS3D_ERROR_DEVICE_TIMEOUT through read_stats / poll_stats, nothing
 * is left running and the pipeline stays usable. 0 restores the default of
 * 4,194,304 polls (about one second). Releases captured graphs. */
gs3d_status gs3d_pipeline_set_wait_limit(gs3d_pipeline* pipeline, uint32_t polls);
/* Test hook for that path: the next render's visibility compaction never
 * scans its first chunk, so the look-back of the chunk after it waits on a
 * status word that nothing publishes until the wait limit runs out. The
 * render needs at least two compaction chunks (more than 256 active splats). */
gs3d_status gs3d_pipeline_debug_withhold_chunk(gs3d_pipeline* pipeline);
/* Test hook for the "allocation-failed" status (types.ts:209-233): the nth
 * device allocation the library makes from now on (1 = the next one) fails
 * as if the device were out of memory; 0 disarms. A failed workspace growth
 * returns GS3D_ERROR_OUT_OF_MEMORY and keeps the previous workspaces, so the
 * pipeline keeps rendering at its previous size. Process-wide. */
void gs3d_debug_fail_allocation(uint32_t nth);
/* getResources() (TiledGaussianPipeline.ts:391-406). */
gs3d_status gs3d_pipeline_get_resources(gs3d_pipeline* pipeline, gs3d_resources* resources);
/* Message of the last failed call on this pipeline ("" if none). */
const char* gs3d_pipeline_last_error(gs3d_pipeline* pipeline);
/* Kernel launches enqueued by the last render call. */
uint32_t gs3d_pipeline_last_launch_count(gs3d_pipeline* pipeline);

/* Kernel timing, the analogue of the reference's profileKernels option
 * (GaussianPass.ts:280-281; sandbox KernelTimingInspector). While enabled,
 * every render records CUDA events between its stages. */
typedef enum gs3d_stage {
  GS3D_STAGE_PROJECT = 0,     /* decode + project + cull + SH + tile count */
  GS3D_STAGE_COMPACT = 1,     /* visibility scan + compaction */
  GS3D_STAGE_DEPTH_SORT = 2,  /* radix sort of (depth key, ordinal) */
  GS3D_STAGE_SCAN = 3,        /* depth-ordered counts + intersection scan */
  GS3D_STAGE_EMIT = 4,        /* intersection emission */
  GS3D_STAGE_TILE_SORT = 5,   /* radix sort of (tile, ordinal) */
  GS3D_STAGE_RANGES = 6,      /* tile ranges */
  GS3D_STAGE_RASTER = 7,      /* tile rasterizer */
  GS3D_STAGE_COUNT = 8
} gs3d_stage;
gs3d_status gs3d_pipeline_set_profiling(gs3d_pipeline* pipeline, int enabled);
/* Mean stage durations in milliseconds over the renders profiled since the
 * last call (ms must hold GS3D_STAGE_COUNT floats); *renders receives how
 * many renders were averaged. Synchronises those renders' events. */
gs3d_status gs3d_pipeline_stage_times(gs3d_pipeline* pipeline, float* ms, uint32_t* renders);
const char* gs3d_stage_name(uint32_t stage);

/* Profiling diagnostics of the last launch sequence (the reference's
 * profile stats, ProfileDiagnosticsStage.ts:22-116, utils/profileStats.ts,
 * types.ts:105-148), computed on the device: tile loads over the tile
 * offsets, cap estimates at 2048/4096/8192 records per tile and at the
 * configured maxRasterizedSplatsPerTile, and the number of projected splats
 * whose subpixel footprint holds no pixel centre. Synchronises the stream. */
typedef struct gs3d_tile_load_stats {
  uint32_t max;
  uint32_t p95;
  uint32_t p99;
  uint32_t tiles_over_256;
  uint32_t tiles_over_512;
  uint32_t tiles_over_1024;
  uint32_t tiles_over_2048;
  uint32_t max_batches;      /* 256-record raster batches of the heaviest tile */
  double mean;
  double median;
  uint64_t total_batches;    /* 256-record raster batches over all tiles */
} gs3d_tile_load_stats;

typedef struct gs3d_tile_cap_stats {
  uint32_t cap;
  uint32_t affected_tiles;
  uint64_t rasterized_intersections;
  uint64_t dropped_intersections;
  double dropped_fraction;
  uint64_t total_batches;
  uint32_t max_batches;
  uint32_t reserved;
} gs3d_tile_cap_stats;

typedef struct gs3d_profile_stats {
  gs3d_tile_load_stats tile_loads;
  gs3d_tile_cap_stats cap_estimates[3]; /* caps 2048, 4096, 8192 */
  gs3d_tile_cap_stats applied_cap;      /* valid when has_applied_cap */
  uint32_t has_applied_cap;
  uint32_t zero_pixel_subpixel_splats;
} gs3d_profile_stats;

gs3d_status gs3d_pipeline_read_profile(gs3d_pipeline* pipeline, gs3d_profile_stats* out);

/* On-device compact packer (the reference packs on the CPU:
 * rust/gaussian-backend/src/engine.rs:1801-1891 encode_attributes with the
 * compact layout, spark-lib splat_encode.rs:127-136,234-252, pack_sh
 * engine.rs:1940-1949). Writes slots [first_slot, first_slot + count) of a
 * store's packed buffers (device pointers; `capacity` = the store's slot
 * count): means (x, y, z, object_id), compact scalesOpacity (f16 ln-scales,
 * f16 opacity), oct101012 rotations, rgb8e8 SH (slot * C words; the DC word
 * from (rgb - 0.5) / SH_C0). The active-slot tail is left to the caller.
 * Inputs are device arrays: centers and scales (linear) count x 3, opacity
 * count, quaternions count x 4 (xyzw, normalised here), rgb count x 3,
 * sh_rest count x (C - 1) x 3 (null at degree 0). Asynchronous on `stream`. */
typedef struct gs3d_splat_source {
  const float* centers;
  const float* scales;
  const float* opacity;
  const float* quaternions;
  const float* rgb;
  const float* sh_rest;
  uint32_t count;
  uint32_t sh_degree;
  uint32_t object_id;
  uint32_t reserved;
} gs3d_splat_source;

gs3d_status gs3d_pack_splats(const gs3d_splat_source* source, uint32_t first_slot, float* means,
                             uint32_t* scales_opacity, uint32_t* rotations, uint32_t* sh_coefficients,
                             uint32_t capacity, void* stream);

/* Visibility compaction with no device allocation. This entry point has no
 * counterpart in the reference. It serves callers that cannot call cudaMalloc
 * where they enqueue work: hosts that route all device memory through their
 * own arena or allocator (and must not see allocations they did not make),
 * and real-time loops that must not stall on the driver's allocator. The
 * caller passes every input and output; the kernel's scratch is a static
 * device array of about 41 KB per GPU, held until the process exits.
 *   keys[n]            per-ordinal depth key, 0xffffffff = not visible
 *   visible_offsets[n] exclusive count of visible ordinals before each one
 *   keys_out/ids_out   (key, ordinal) of the visible ordinals, in ordinal order
 *   result[2]          device words: visible count, error flags (nonzero: a
 *                      bounded device wait expired)
 * n must not exceed GS3D_STATIC_COMPACT_MAX_ITEMS (else GS3D_ERROR_RANGE);
 * keys must be 4-byte aligned. The first call on a device looks up the static
 * array's device address and the SM count. All calls share the array, which
 * keeps the previous call's contents (each call clears what must start at
 * zero): calls that overlap on the GPU race, so order them on one stream. */
#define GS3D_STATIC_COMPACT_MAX_ITEMS 16777216u
gs3d_status gs3d_compact_visible_static(const uint32_t* keys, uint32_t n, uint32_t* visible_offsets,
                                        uint32_t* keys_out, uint32_t* ids_out, uint32_t* result, void* stream);

/* IntersectionCapacityPolicy.next(current, demand)
 * (src/renderer/pipeline/IntersectionCapacityPolicy.ts:90-100): the capacity
 * to grow to, or 0 for null (demand above maximum). */
uint64_t gs3d_capacity_next(uint64_t maximum, double growth, double headroom, uint64_t current,
                            uint64_t demand);

#ifdef __cplusplus
}
#endif

#endif /* GS3D_H */
