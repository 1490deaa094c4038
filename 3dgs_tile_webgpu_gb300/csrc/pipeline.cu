// Host side of the C ABI (include/gs3d.h): workspace ownership, validation
// with the reference's error semantics, and the per-frame launch sequence of
// TiledGaussianPipeline.render (src/renderer/pipeline/TiledGaussianPipeline.ts:324-341).
#include <cuda_runtime.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <new>
#include <string>
#include <vector>

#include "../../include/gs3d.h"
#include "pass_common.cuh"

using namespace gs;

namespace {

constexpr uint32_t kObjectRing = 4;  // pinned batch-table staging slots
constexpr uint32_t kMaxViews = 4096;
constexpr uint32_t kStageEvents = GS3D_STAGE_COUNT + 1;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

// Totals of a batch rendered as several launch sequences (views per launch
// below the batch size): every launch sequence zeroes and refills the control
// block, so its counts are added here before the next one starts.
struct BatchSummary {
  uint32_t visible, intersections, requested, overflow;
  uint32_t error, prev_version, chunks, pad;
  unsigned long long raster[4];
};

namespace {

__global__ void k_summary_begin(BatchSummary* s, const uint32_t* output_state) {
  s->visible = s->intersections = s->requested = s->overflow = 0u;
  s->error = s->chunks = s->pad = 0u;
  s->prev_version = output_state[1];
  for (int i = 0; i < 4; ++i) s->raster[i] = 0ull;
}

// Adds one launch sequence's counts; after the last one, writes the batch's
// output state (attempt, version, demand, overflow): the version advances
// only if no launch sequence overflowed, and the demand is the largest of the
// sequences (they share one intersection buffer).
__global__ void k_summary_add(BatchSummary* s, const Control* c, const uint32_t* frame_params,
                              uint32_t* output_state, int last) {
  s->visible += c->visible_state[0];
  s->intersections += c->state[0];
  s->requested = max(s->requested, c->state[1]);
  s->overflow |= c->state[3];
  s->error |= c->error;
  for (int i = 0; i < 4; ++i) s->raster[i] += c->raster_stats[i];
  s->chunks += 1u;
  if (last) {
    const uint32_t attempt = frame_params[0];
    const uint32_t last_version = frame_params[1] ? 0u : s->prev_version;
    output_state[0] = attempt;
    output_state[1] = s->overflow ? last_version : attempt;
    output_state[2] = s->requested;
    output_state[3] = s->overflow ? 1u : 0u;
  }
}

}  // namespace

struct gs3d_pipeline {
  gs3d_pipeline_desc desc{};
  gs3d_gaussian_data data{};
  int device = 0;
  int sms = 148;
  std::string error;
  // Per-slot workspaces (sized by data.count).
  uint32_t slot_cap = 0;
  float4* mean = nullptr;
  float4* rec = nullptr;   // packed raster records, two float4 per slot
  float4* erec = nullptr;  // emission records, two float4 per slot
  float4* conic = nullptr;
  float4* color = nullptr;
  uint32_t* counts = nullptr;
  uint32_t* keys = nullptr;
  uint32_t* vis_off = nullptr;
  uint32_t* dk[2] = {nullptr, nullptr};
  uint32_t* dv[2] = {nullptr, nullptr};
  uint32_t* ordered = nullptr;
  uint32_t* ioff = nullptr;
  // Intersection workspaces (sized by capacity).
  uint64_t capacity = 0;
  uint32_t* tk[2] = {nullptr, nullptr};
  uint32_t* tv[2] = {nullptr, nullptr};
  // Tiles.
  uint32_t tile_cap = 0;
  uint32_t* tile_offsets = nullptr;
  uint32_t* tile_order = nullptr;
  // Control, output state, look-back status.
  Control* ctl = nullptr;
  uint32_t* output_state = nullptr;
  unsigned long long* status = nullptr;
  size_t status_words = 0;
  // Per-(chunk, digit) counts of the chunked sort passes.
  uint32_t* chunk_counts = nullptr;
  uint32_t epoch = 0;
  // Batch-table staging (bases, view descriptors, object tables), a ring of
  // pinned host buffers each mirrored by a device buffer.
  size_t stage_cap = 0;
  unsigned char* stage_dev[kObjectRing] = {};
  unsigned char* stage_pinned[kObjectRing] = {};
  cudaEvent_t stage_ev[kObjectRing] = {};
  bool stage_ev_used[kObjectRing] = {};
  uint32_t frame_index = 0;
  // Layout of the last batch.
  std::vector<uint32_t> item_bases, tile_bases;
  uint32_t total_items = 0, total_tiles = 0;
  // Device epoch counter of the look-back protocol and frames since the last
  // status reset.
  uint32_t* epoch_dev = nullptr;
  uint64_t frames_since_reset = 0;
  // Captured CUDA graphs (two, alternating staging buffers).
  cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
  unsigned char* graph_pinned[2] = {nullptr, nullptr};
  unsigned char* graph_dev[2] = {nullptr, nullptr};
  cudaEvent_t graph_ev[2] = {nullptr, nullptr};
  bool graph_ev_used[2] = {false, false};
  size_t graph_stage_bytes = 0;
  std::vector<gs3d_view> graph_views;
  std::vector<gs3d_camera> graph_cameras;
  uint32_t graph_launches = 0;
  uint32_t graph_next = 0;
  uint32_t graph_tile = kTileSize;
  // Tuning (gs3d_pipeline_set_tuning / autotune) and the device summary of a
  // batch rendered as several launch sequences.
  gs3d_tuning tuning{0u, 8u, 1u, 0u, 0u, {0u, 0u, 0u}};  // tile_size 0: the reference's 16; 2 pixels per lane
  BatchSummary* summary = nullptr;
  uint32_t last_chunks = 1;
  BatchView last_bv{};  // batch table of the last launch sequence (device pointers)
  // Profiling diagnostics scratch: tile-load sums, load histogram, zero-pixel count.
  TileLoadSums* profile_sums = nullptr;
  uint32_t* profile_hist = nullptr;
  uint32_t* profile_zero = nullptr;
  struct GraphChunk {
    uint32_t first, count;
    size_t offset;
  };
  std::vector<GraphChunk> graph_chunks;
  // Frame.
  bool prepared = false;
  uint32_t width = 0, height = 0, tiles_x = 0, tiles_y = 0;
  cudaStream_t last_stream = nullptr;
  uint32_t last_launches = 0;
  // Final buffers of the two sorts (after ping-pong).
  int depth_final = 0;
  int tile_final = 0;
  // Asynchronous stats read-back (gs3d_pipeline_request_stats / poll_stats):
  // pinned copy of the counters, its completion event, and the layout of the
  // render it describes.
  unsigned char* rb_pinned = nullptr;
  cudaEvent_t rb_event = nullptr;
  bool rb_pending = false;
  uint32_t rb_chunks = 1;
  // Polls a look-back wait may spend on one status word (0: the default),
  // and the test hook that withholds the compaction's first chunk.
  uint32_t wait_limit = 0;
  bool withhold_first_chunk = false;
  // Kernel timing: one set of GS3D_STAGE_COUNT + 1 events per profiled render.
  bool profiling = false;
  std::vector<cudaEvent_t> events;  // pool, in sets of kStageEvents
  uint32_t profiled = 0;            // sets recorded since the last read
};

namespace {

gs3d_status fail(gs3d_pipeline* p, gs3d_status s, const std::string& msg) {
  if (p) p->error = msg;
  return s;
}

gs3d_status cuda_fail(gs3d_pipeline* p, cudaError_t e, const char* what) {
  cudaGetLastError();
  gs3d_status s = e == cudaErrorMemoryAllocation ? GS3D_ERROR_OUT_OF_MEMORY : GS3D_ERROR_CUDA;
  return fail(p, s, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
void dfree(T*& ptr) {
  if (ptr) cudaFree((void*)ptr);
  ptr = nullptr;
}

// Allocation-failure injection (gs3d_debug_fail_allocation): the countdown
// reaches zero on the device allocation that is made to fail.
std::atomic<int64_t> g_fail_countdown{0};

cudaError_t device_malloc(void** ptr, size_t bytes) {
  if (g_fail_countdown.load() > 0 && g_fail_countdown.fetch_sub(1) == 1) {
    *ptr = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(ptr, bytes);
}

template <typename T>
cudaError_t dalloc(T*& ptr, size_t count) {
  dfree(ptr);
  if (count == 0) count = 1;
  return device_malloc((void**)&ptr, count * sizeof(T));
}

// Tiles covering `px` pixels with tiles of `tile` pixels per side.
uint32_t tiles_for(uint32_t px, uint32_t tile = kTileSize) { return (px + tile - 1u) / tile; }

// Pixels per tile side of a batched render: the tuning's, or the reference's 16.
uint32_t batch_tile(const gs3d_pipeline* p) { return p->tuning.tile_size ? p->tuning.tile_size : kTileSize; }

uint32_t ceil_log2(uint64_t v) {
  uint32_t b = 0;
  while ((1ull << b) < v) ++b;
  return b;
}

gs3d_status validate_desc(gs3d_pipeline* p, const gs3d_pipeline_desc& d) {
  if (d.abi_version != GS3D_ABI_VERSION) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "abi_version mismatch");
  if (d.depth_sort_mode > 1) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "depthSortMode must be float32 or packed16");
  if (d.antialias_mode > 1) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "antialiasMode must be compensated or classic");
  if (d.boundary_policy > 2) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "boundaryPolicy must be clip, repeat-x or repeat-y");
  if (d.raster_precision > 2) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "unknown raster precision");
  if (d.depth_encoding > 1) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "unknown depth encoding");
  if (d.projection_precision > 1) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "unknown projection precision");
  // GaussianPass.ts:178-192,231-255
  if (d.intersection_capacity == 0 || d.intersection_capacity > 0x7fffffffull)
    return fail(p, GS3D_ERROR_RANGE, "intersectionCapacity must be a positive integer below 2^31");
  if (!(d.raster_transmittance_threshold > 0.0f && d.raster_transmittance_threshold < 1.0f))
    return fail(p, GS3D_ERROR_RANGE, "rasterTransmittanceThreshold must be finite and in (0, 1)");
  if (!(d.depth_alpha_threshold >= 0.0f && d.depth_alpha_threshold <= 1.0f))
    return fail(p, GS3D_ERROR_RANGE, "depthAlphaThreshold must be finite and in [0, 1]");
  // rasterChunks.ts:208-227 (the 65,535-task bound is a WebGPU dispatch limit
  // and does not apply to this implementation).
  if (d.raster_chunk_size != 0 && (d.raster_chunk_size < 256 || d.raster_chunk_size % 256 != 0))
    return fail(p, GS3D_ERROR_RANGE, "rasterChunkSize must be a multiple of 256 and at least 256");
  if (!isfinite(d.filter_variance) || d.filter_variance < 0.0f)
    return fail(p, GS3D_ERROR_RANGE, "filterVariance must be finite and non-negative");
  return GS3D_OK;
}

gs3d_status validate_data(gs3d_pipeline* p, const gs3d_gaussian_data* d) {
  if (!d) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "GaussianData is null");
  // GaussianData.ts:76-167
  if (d->count == 0) return fail(p, GS3D_ERROR_RANGE, "GaussianData count must be a positive integer");
  if (d->sh_degree > 3) return fail(p, GS3D_ERROR_RANGE, "GaussianData shDegree must be 0, 1, 2, or 3");
  if (d->active_count > d->count) return fail(p, GS3D_ERROR_RANGE, "active count exceeds slot count");
  if (!d->means || !d->scales_opacity || !d->rotations || !d->sh_coefficients)
    return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "Invalid compact Gaussian shape attribute");
  if (((uintptr_t)d->means & 15u) || ((uintptr_t)d->scales_opacity & 7u) || ((uintptr_t)d->rotations & 3u) ||
      ((uintptr_t)d->sh_coefficients & 15u))
    return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "packed buffers must be naturally aligned (SH to 16 bytes)");
  return GS3D_OK;
}

// Look-back status words of the compaction and the ordered-count scan: one
// per chunk, at most one chunk per 256 items.
size_t status_words_needed(uint32_t slots, uint64_t capacity) {
  (void)capacity;
  return (slots + 255u) / 256u + 1;
}

gs3d_status ensure_status(gs3d_pipeline* p) {
  const size_t need = status_words_needed(p->slot_cap, p->capacity);
  if (need <= p->status_words) return GS3D_OK;
  unsigned long long* fresh = nullptr;
  cudaError_t e = dalloc(fresh, need);
  if (e == cudaSuccess) e = cudaMemset(fresh, 0, need * sizeof(unsigned long long));
  if (e != cudaSuccess) {
    dfree(fresh);
    return cuda_fail(p, e, "allocating look-back status");
  }
  dfree(p->status);
  p->status = fresh;
  p->status_words = need;
  p->epoch = 0;
  return GS3D_OK;
}

// Grows every buffer of `bufs` to its new element count, or none of them: on
// a failed allocation the new buffers are released and the old ones kept, so
// the pipeline stays usable at its previous size ("allocation-failed" leaves
// the previous resources in place, GaussianPass.ts:808-826).
struct Grow {
  void** slot;
  size_t bytes;
};
cudaError_t grow_all(Grow* bufs, size_t n) {
  std::vector<void*> fresh(n, nullptr);
  cudaError_t e = cudaSuccess;
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) e = device_malloc(&fresh[i], std::max<size_t>(bufs[i].bytes, 1));
  if (e != cudaSuccess) {
    for (void* q : fresh)
      if (q) cudaFree(q);
    return e;
  }
  for (size_t i = 0; i < n; ++i) {
    if (*bufs[i].slot) cudaFree(*bufs[i].slot);
    *bufs[i].slot = fresh[i];
  }
  return cudaSuccess;
}

gs3d_status ensure_slots(gs3d_pipeline* p, uint32_t count) {
  if (count <= p->slot_cap) return GS3D_OK;
  // AttributePool.grow semantics: at least double.
  const uint32_t cap = std::max(count, p->slot_cap * 2u);
  const size_t f4 = (size_t)cap * sizeof(float4), u = (size_t)cap * sizeof(uint32_t);
  Grow bufs[] = {{(void**)&p->mean, f4},    {(void**)&p->conic, f4},   {(void**)&p->color, f4},
                 {(void**)&p->rec, 2 * f4}, {(void**)&p->erec, 2 * f4}, {(void**)&p->counts, u},
                 {(void**)&p->keys, u},     {(void**)&p->vis_off, u}, {(void**)&p->dk[0], u},
                 {(void**)&p->dk[1], u},    {(void**)&p->dv[0], u},   {(void**)&p->dv[1], u},
                 {(void**)&p->ordered, u},  {(void**)&p->ioff, u}};
  cudaError_t e = grow_all(bufs, sizeof(bufs) / sizeof(bufs[0]));
  if (e != cudaSuccess) return cuda_fail(p, e, "allocating per-Gaussian workspaces");
  cudaMemset(p->conic, 0, f4);
  cudaMemset(p->color, 0, f4);
  p->slot_cap = cap;
  return ensure_status(p);
}

gs3d_status ensure_capacity(gs3d_pipeline* p, uint64_t capacity) {
  const size_t u = (size_t)capacity * sizeof(uint32_t);
  Grow bufs[] = {{(void**)&p->tk[0], u}, {(void**)&p->tk[1], u}, {(void**)&p->tv[0], u}, {(void**)&p->tv[1], u}};
  cudaError_t e = grow_all(bufs, 4);
  if (e != cudaSuccess) return cuda_fail(p, e, "allocating intersection workspaces");
  p->capacity = capacity;
  return ensure_status(p);
}

gs3d_status ensure_stage(gs3d_pipeline* p, size_t bytes) {
  if (bytes <= p->stage_cap) return GS3D_OK;
  const size_t cap = std::max(bytes, std::max<size_t>(16384, p->stage_cap * 2));
  p->stage_cap = 0;  // until every slot is regrown
  for (uint32_t i = 0; i < kObjectRing; ++i) {
    if (p->stage_ev_used[i]) cudaEventSynchronize(p->stage_ev[i]);
    dfree(p->stage_dev[i]);
    if (p->stage_pinned[i]) cudaFreeHost(p->stage_pinned[i]);
    p->stage_pinned[i] = nullptr;
    cudaError_t e = dalloc(p->stage_dev[i], cap);
    if (e != cudaSuccess) return cuda_fail(p, e, "allocating the batch table");
    e = cudaMallocHost((void**)&p->stage_pinned[i], cap);
    if (e != cudaSuccess) return cuda_fail(p, e, "allocating the pinned batch table");
  }
  p->stage_cap = cap;
  return GS3D_OK;
}

// Tile offsets (tiles + 1 words) and the raster work list (tiles words), grown
// together to the next power of two (TiledGaussianPipeline.ts:306-318).
gs3d_status ensure_tiles(gs3d_pipeline* p, uint64_t tiles) {
  if (tiles + 1 <= p->tile_cap && p->tile_offsets && p->tile_order) return GS3D_OK;
  if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  uint64_t cap = 1;
  while (cap < tiles + 1) cap <<= 1;
  cudaError_t e = dalloc(p->tile_offsets, cap);
  if (e == cudaSuccess) e = dalloc(p->tile_order, cap);
  if (e != cudaSuccess) {
    p->tile_cap = 0;
    return cuda_fail(p, e, "allocating tile offsets");
  }
  cudaMemset(p->tile_offsets, 0, (size_t)cap * sizeof(uint32_t));
  p->tile_cap = (uint32_t)cap;
  return GS3D_OK;
}

// Status words hold 30-bit epochs and every frame consumes kEpochsPerFrame of
// them; well before the counter wraps, clear the words and the counter
// (stream-ordered, outside any captured graph).
void maybe_reset_epochs(gs3d_pipeline* p, cudaStream_t st) {
  if (++p->frames_since_reset < (1ull << 25)) return;
  cudaMemsetAsync(p->status, 0, p->status_words * sizeof(unsigned long long), st);
  cudaMemsetAsync(p->epoch_dev, 0, sizeof(uint32_t), st);
  p->frames_since_reset = 1;
}

// Event marking the start of `stage` (stage == GS3D_STAGE_COUNT: end) of the
// current profiled render.
void mark(gs3d_pipeline* p, uint32_t stage, cudaStream_t st) {
  if (!p->profiling) return;
  const size_t idx = (size_t)p->profiled * kStageEvents + stage;
  while (p->events.size() <= idx) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    p->events.push_back(e);
  }
  cudaEventRecord(p->events[idx], st);
}

void release_graphs(gs3d_pipeline* p) {
  for (int g = 0; g < 2; ++g) {
    if (p->graph_ev_used[g]) cudaEventSynchronize(p->graph_ev[g]);
    if (p->graph_exec[g]) cudaGraphExecDestroy(p->graph_exec[g]);
    p->graph_exec[g] = nullptr;
    if (p->graph_pinned[g]) cudaFreeHost(p->graph_pinned[g]);
    p->graph_pinned[g] = nullptr;
    dfree(p->graph_dev[g]);
    if (p->graph_ev[g]) cudaEventDestroy(p->graph_ev[g]);
    p->graph_ev[g] = nullptr;
    p->graph_ev_used[g] = false;
  }
  p->graph_views.clear();
  p->graph_cameras.clear();
}

void release_all(gs3d_pipeline* p) {
  release_graphs(p);
  if (p->rb_event) {
    cudaEventSynchronize(p->rb_event);
    cudaEventDestroy(p->rb_event);
  }
  if (p->rb_pinned) cudaFreeHost(p->rb_pinned);
  p->rb_event = nullptr;
  p->rb_pinned = nullptr;
  for (cudaEvent_t e : p->events) cudaEventDestroy(e);
  p->events.clear();
  for (uint32_t i = 0; i < kObjectRing; ++i) {
    if (p->stage_ev_used[i]) cudaEventSynchronize(p->stage_ev[i]);
    if (p->stage_ev[i]) cudaEventDestroy(p->stage_ev[i]);
    dfree(p->stage_dev[i]);
    if (p->stage_pinned[i]) cudaFreeHost(p->stage_pinned[i]);
  }
  dfree(p->mean); dfree(p->rec); dfree(p->erec); dfree(p->conic); dfree(p->color); dfree(p->counts); dfree(p->keys); dfree(p->vis_off);
  dfree(p->dk[0]); dfree(p->dk[1]); dfree(p->dv[0]); dfree(p->dv[1]); dfree(p->ordered); dfree(p->ioff);
  dfree(p->tk[0]); dfree(p->tk[1]); dfree(p->tv[0]); dfree(p->tv[1]);
  dfree(p->tile_offsets); dfree(p->tile_order); dfree(p->ctl); dfree(p->epoch_dev); dfree(p->output_state); dfree(p->status);
  dfree(p->chunk_counts);
  dfree(p->summary); dfree(p->profile_sums); dfree(p->profile_hist); dfree(p->profile_zero);
}

}  // namespace

extern "C" {

uint32_t gs3d_abi_version(void) { return GS3D_ABI_VERSION; }

const char* gs3d_status_string(gs3d_status s) {
  switch (s) {
    case GS3D_OK: return "ok";
    case GS3D_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case GS3D_ERROR_RANGE: return "out of range";
    case GS3D_ERROR_NOT_PREPARED: return "pipeline must be prepared before rendering";
    case GS3D_ERROR_OUT_OF_MEMORY: return "allocation failed";
    case GS3D_ERROR_CUDA: return "CUDA error";
    case GS3D_ERROR_DEVICE_TIMEOUT: return "device wait expired";
    case GS3D_ERROR_UNSUPPORTED: return "unsupported option";
    case GS3D_NOT_READY: return "not ready";
  }
  return "unknown status";
}

void gs3d_pipeline_desc_defaults(gs3d_pipeline_desc* d) {
  if (!d) return;
  memset(d, 0, sizeof(*d));
  d->abi_version = GS3D_ABI_VERSION;
  d->device = 0;
  d->depth_sort_mode = GS3D_DEPTH_FLOAT32;
  d->antialias_mode = GS3D_ANTIALIAS_COMPENSATED;
  d->intersection_capacity = 262144;  // IntersectionCapacityPolicy.ts:71-74
  d->max_rasterized_splats_per_tile = 0;
  d->raster_chunk_size = 8192;        // constants.ts:3
  d->subpixel_sample_culling = 1;
  d->raster_transmittance_threshold = 1e-4f;
  d->depth_alpha_threshold = 0.95f;
  d->filter_variance = 0.3f;
  d->invalid_depth_value = 1.0f;
  d->boundary_policy = GS3D_BOUNDARY_CLIP;
  d->raster_precision = GS3D_RASTER_FP32;
  d->depth_encoding = 0;
  d->projection_precision = GS3D_PROJECTION_FP32;
}

gs3d_status gs3d_pipeline_create(const gs3d_pipeline_desc* desc, const gs3d_gaussian_data* data,
                                 gs3d_pipeline** out) {
  if (!desc || !out) return GS3D_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  gs3d_pipeline* p = new (std::nothrow) gs3d_pipeline();
  if (!p) return GS3D_ERROR_OUT_OF_MEMORY;
  gs3d_status s;
  if ((s = validate_desc(p, *desc)) != GS3D_OK || (s = validate_data(p, data)) != GS3D_OK) {
    delete p;
    return s;
  }
  p->desc = *desc;
  p->data = *data;
  p->device = desc->device;
  cudaError_t e = cudaSetDevice(p->device);
  if (e != cudaSuccess) {
    delete p;
    return GS3D_ERROR_CUDA;
  }
  cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device);
  for (uint32_t i = 0; i < kObjectRing; ++i) cudaEventCreateWithFlags(&p->stage_ev[i], cudaEventDisableTiming);
  if ((e = dalloc(p->ctl, 1)) || (e = dalloc(p->output_state, 4)) || (e = dalloc(p->epoch_dev, 1)) ||
      (e = dalloc(p->summary, 1)) ||
      (e = dalloc(p->chunk_counts, (size_t)kChunkBlocksPerSm * (size_t)p->sms * 256u))) {
    s = cuda_fail(p, e, "allocating control block");
    release_all(p);
    delete p;
    return s;
  }
  cudaMemset(p->output_state, 0, 4 * sizeof(uint32_t));
  cudaMemset(p->ctl, 0, sizeof(Control));
  cudaMemset(p->epoch_dev, 0, sizeof(uint32_t));
  cudaMemset(p->summary, 0, sizeof(BatchSummary));
  prepare_sort_kernels();
  if ((s = ensure_slots(p, data->count)) != GS3D_OK || (s = ensure_capacity(p, desc->intersection_capacity)) != GS3D_OK ||
      (s = ensure_stage(p, 16384)) != GS3D_OK) {
    release_all(p);
    delete p;
    return s;
  }
  *out = p;
  return GS3D_OK;
}

void gs3d_pipeline_destroy(gs3d_pipeline* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  release_all(p);
  delete p;
}

gs3d_status gs3d_pipeline_update_data(gs3d_pipeline* p, const gs3d_gaussian_data* data) {
  if (!p) return GS3D_ERROR_INVALID_ARGUMENT;
  gs3d_status s = validate_data(p, data);
  if (s != GS3D_OK) return s;
  cudaSetDevice(p->device);
  if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  release_graphs(p);
  if ((s = ensure_slots(p, data->count)) != GS3D_OK) return s;
  p->data = *data;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_resize_intersections(gs3d_pipeline* p, uint64_t capacity) {
  if (!p) return GS3D_ERROR_INVALID_ARGUMENT;
  if (capacity == 0 || capacity > 0x7fffffffull)
    return fail(p, GS3D_ERROR_RANGE, "intersection capacity must be a positive integer below 2^31");
  cudaSetDevice(p->device);
  if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  release_graphs(p);
  return ensure_capacity(p, capacity);
}

gs3d_status gs3d_pipeline_prepare_frame(gs3d_pipeline* p, uint32_t width, uint32_t height) {
  if (!p) return GS3D_ERROR_INVALID_ARGUMENT;
  if (width == 0 || height == 0) return fail(p, GS3D_ERROR_RANGE, "render size must be positive");
  const uint32_t tx = tiles_for(width), ty = tiles_for(height);
  // TiledGaussianPipeline.ts:294-296
  if (tx > 65535u || ty > 65535u) return fail(p, GS3D_ERROR_RANGE, "Render size exceeds WebGPU's tile dispatch limit");
  cudaSetDevice(p->device);
  const uint32_t ntile = tx * ty;
  gs3d_status s = ensure_tiles(p, ntile);
  if (s != GS3D_OK) return s;
  p->width = width;
  p->height = height;
  p->tiles_x = tx;
  p->tiles_y = ty;
  p->prepared = true;
  return GS3D_OK;
}

}  // extern "C"

namespace {

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

struct Plan {
  uint32_t n = 0, ngroups = 0;
  uint32_t tile = kTileSize;  // pixels per tile side
  bool any_depth = false;
  uint32_t items = 0, tiles = 0, blocks = 0;
  size_t objects = 0;
  size_t views_off = 0, objects_off = 0, stage_bytes = 0;
};

// Byte layout of a staged batch table of n views holding `objects` object
// rows: frame parameters and the four base arrays, view descriptors, object
// rows.
void layout_plan(Plan* pl, uint32_t n, size_t objects) {
  const size_t header = 16 + align16(4 * (size_t)(n + 1) * sizeof(uint32_t));
  pl->views_off = header;
  pl->objects_off = align16(header + (size_t)n * sizeof(ViewDesc));
  pl->stage_bytes = pl->objects_off + objects * 40 * sizeof(float);
}

// Consecutive views of a batch that render the same packed scene (same
// buffers, counts and SH degree) form a view group: the projection decodes
// each splat once for the whole group.
bool same_scene(const gs3d_view& a, const gs3d_view& b) {
  const gs3d_gaussian_data& x = *a.data;
  const gs3d_gaussian_data& y = *b.data;
  return x.means == y.means && x.scales_opacity == y.scales_opacity && x.rotations == y.rotations &&
         x.sh_coefficients == y.sh_coefficients && x.count == y.count && x.active_count == y.active_count &&
         x.sh_degree == y.sh_degree;
}

// Validate a batch, grow every workspace it needs and lay out its batch
// table. Not capturable (it may allocate).
gs3d_status plan_batch(gs3d_pipeline* p, const gs3d_view* views, uint32_t n, Plan* out, uint32_t tile) {
  if (n == 0 || n > kMaxViews) return fail(p, GS3D_ERROR_RANGE, "a batch holds 1 to 4096 views");
  uint64_t items = 0, tiles = 0, blocks = 0;
  uint32_t ngroups = 0;
  bool any_depth = false;
  size_t objects = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const gs3d_view& v = views[i];
    gs3d_status s = validate_data(p, v.data);
    if (s != GS3D_OK) return s;
    if (!v.camera || !v.targets.color) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "camera and color target required");
    if (v.targets.color_format > 1) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "unknown color format");
    if (v.camera->object_count > 0 && !v.camera->object_table)
      return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "object table is null");
    if (!(v.camera->depth_near >= 0.0f) || !(v.camera->depth_far > v.camera->depth_near))
      return fail(p, GS3D_ERROR_RANGE, "depth range must satisfy 0 <= near < far");
    if (v.width == 0 || v.height == 0) return fail(p, GS3D_ERROR_RANGE, "render size must be positive");
    any_depth = any_depth || v.targets.depth != nullptr;
    const uint32_t tx = tiles_for(v.width, tile), ty = tiles_for(v.height, tile);
    // TiledGaussianPipeline.ts:294-296
    if (tx > 65535u || ty > 65535u) return fail(p, GS3D_ERROR_RANGE, "Render size exceeds WebGPU's tile dispatch limit");
    const uint64_t b = ((uint64_t)v.data->active_count + kBlock - 1) / kBlock;
    if (i == 0 || !same_scene(views[i - 1], v)) {
      blocks += b;
      ++ngroups;
    }
    items += b * kBlock;
    tiles += (uint64_t)tx * ty;
    objects += v.camera->object_count;
  }
  if (items >= 0xffffffffull || tiles >= 0x7fffffffull) return fail(p, GS3D_ERROR_RANGE, "batch too large");
  // Workspaces (grow only; synchronise before freeing buffers a queued frame may use).
  if (items > p->slot_cap || tiles + 1 > p->tile_cap ||
      status_words_needed((uint32_t)items, p->capacity) > p->status_words) {
    if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  }
  gs3d_status s = ensure_slots(p, (uint32_t)items);
  if (s != GS3D_OK) return s;
  if ((s = ensure_status(p)) != GS3D_OK) return s;
  if ((s = ensure_tiles(p, tiles)) != GS3D_OK) return s;
  out->n = n;
  out->tile = tile;
  out->ngroups = ngroups;
  out->any_depth = any_depth;
  out->items = (uint32_t)items;
  out->tiles = (uint32_t)tiles;
  out->blocks = (uint32_t)blocks;
  out->objects = objects;
  layout_plan(out, n, objects);
  return GS3D_OK;
}

// Fill a host copy of the batch table whose device copy will live at `dev`:
// frame parameters, the item/tile base arrays, the view-group arrays, view
// descriptors, object tables.
void stage_batch(gs3d_pipeline* p, const gs3d_view* views, const Plan& pl, uint32_t attempt, int reset_valid,
                 unsigned char* host, unsigned char* dev) {
  const uint32_t n = pl.n;
  uint32_t* params = (uint32_t*)host;
  params[0] = attempt;
  params[1] = reset_valid ? 1u : 0u;
  params[2] = params[3] = 0u;
  uint32_t* h_item = params + 4;
  uint32_t* h_tile = h_item + (n + 1);
  uint32_t* h_gblock = h_tile + (n + 1);
  uint32_t* h_gview = h_gblock + (n + 1);
  uint32_t ngroups = 0;
  ViewDesc* h_views = (ViewDesc*)(host + pl.views_off);
  float* h_obj = (float*)(host + pl.objects_off);
  uint32_t item = 0, tile = 0, block = 0;
  size_t obj = 0;
  p->item_bases.assign(n + 1, 0);
  p->tile_bases.assign(n + 1, 0);
  for (uint32_t i = 0; i < n; ++i) {
    const gs3d_view& v = views[i];
    const gs3d_gaussian_data& d = *v.data;
    ViewDesc& w = h_views[i];
    memset(&w, 0, sizeof(w));
    w.means = (const float4*)d.means;
    w.shape = (const uint2*)d.scales_opacity;
    w.rot = (const uint32_t*)d.rotations;
    w.sh = (const uint32_t*)d.sh_coefficients;
    w.objects = (const float*)(dev + pl.objects_off) + obj * 40;
    w.color = v.targets.color;
    w.depth = v.targets.depth;
    w.count = d.count;
    w.active = d.active_count;
    w.degree = d.sh_degree;
    w.C = (d.sh_degree + 1) * (d.sh_degree + 1);
    w.object_count = v.camera->object_count;
    w.color_half = v.targets.color_format == GS3D_COLOR_RGBA16F ? 1u : 0u;
    w.tiles_x = tiles_for(v.width, pl.tile);
    w.tiles_y = tiles_for(v.height, pl.tile);
    w.item_base = item;
    w.tile_base = tile;
    memcpy(w.P, v.camera->projection, sizeof(w.P));
    w.vw = (float)v.width;
    w.vh = (float)v.height;
    w.vnear = v.camera->depth_near;
    w.vfar = v.camera->depth_far;
    if (v.camera->object_count)
      memcpy(h_obj + obj * 40, v.camera->object_table, (size_t)v.camera->object_count * 40 * sizeof(float));
    h_item[i] = item;
    h_tile[i] = tile;
    p->item_bases[i] = item;
    p->tile_bases[i] = tile;
    const uint32_t b = (d.active_count + kBlock - 1) / kBlock;
    if (i == 0 || !same_scene(views[i - 1], v)) {
      h_gblock[ngroups] = block;
      h_gview[ngroups] = i;
      ++ngroups;
      block += b;
    }
    item += b * kBlock;
    tile += w.tiles_x * w.tiles_y;
    obj += v.camera->object_count;
  }
  h_item[n] = item;
  h_tile[n] = tile;
  for (uint32_t g = ngroups; g <= n; ++g) {
    h_gblock[g] = block;
    h_gview[g] = n;
  }
  p->item_bases[n] = item;
  p->tile_bases[n] = tile;
  p->total_items = item;
  p->total_tiles = tile;
}

// Enqueue the pass over a staged batch table at `dev` (capturable: launches
// and memsets only).
void record_batch(gs3d_pipeline* p, const Plan& pl, unsigned char* dev, cudaStream_t st) {
  const uint32_t n = pl.n;
  BatchView bv;
  bv.frame_params = (const uint32_t*)dev;
  bv.item_base = bv.frame_params + 4;
  bv.tile_base = bv.item_base + (n + 1);
  bv.group_block = bv.tile_base + (n + 1);
  bv.group_view = bv.group_block + (n + 1);
  bv.ngroups = pl.ngroups;
  bv.views = (const ViewDesc*)(dev + pl.views_off);
  bv.nviews = n;
  bv.total_items = pl.items;
  bv.total_tiles = pl.tiles;
  bv.total_blocks = pl.blocks;
  p->last_bv = bv;

  PassOptions o;
  memset(&o, 0, sizeof(o));
  o.filter = p->desc.filter_variance;
  o.axis = p->desc.boundary_policy;
  o.antialias = p->desc.antialias_mode;
  o.subpixel = p->desc.subpixel_sample_culling ? 1u : 0u;
  o.depth_mode = p->desc.depth_sort_mode;
  o.chunk = p->desc.raster_chunk_size;
  o.max_per_tile = p->desc.max_rasterized_splats_per_tile;
  o.depth_encoding = p->desc.depth_encoding;
  o.proj_fp64 = p->desc.projection_precision == GS3D_PROJECTION_FP64 ? 1u : 0u;
  o.any_depth = pl.any_depth ? 1u : 0u;
  o.tile = pl.tile;
  o.tile_px = (float)pl.tile;
  o.tile_inv = 1.0f / (float)pl.tile;
  o.pixels_per_lane = p->tuning.raster_pixels_per_lane == 4u ? 4u : 2u;
  memcpy(o.background, p->desc.background, sizeof(o.background));
  o.t_threshold = p->desc.raster_transmittance_threshold;
  o.depth_alpha_threshold = p->desc.depth_alpha_threshold;
  o.invalid_depth = p->desc.invalid_depth_value;

  const uint32_t N = pl.items;
  const uint32_t tile = pl.tiles;
  uint32_t launches = 0;
  Control* ctl = p->ctl;
  uint32_t ep = 0;  // look-back launch index within the frame
  auto epoch = [&]() { return Epoch{p->epoch_dev, ++ep, p->wait_limit}; };
  launch_epoch_begin(p->epoch_dev, st);
  cudaMemsetAsync(ctl, 0, sizeof(Control), st);
  launches += 1;
  if (p->withhold_first_chunk) {
    // Test hook (gs3d_pipeline_debug_withhold_chunk): the compaction's ticket
    // counter starts at 1, so no block scans chunk 0 and the look-back of
    // chunk 1 waits on a status word that is never published.
    launch_skip_ticket(ctl, kTicketCompact, st);
    p->withhold_first_chunk = false;
    ++launches;
  }

  // K1: projection.
  mark(p, GS3D_STAGE_PROJECT, st);
  const bool exact = p->desc.raster_precision == GS3D_RASTER_EXACT;
  launch_project(bv, o, p->mean, p->conic, p->color, p->counts, p->keys, exact ? nullptr : p->rec, p->erec, st);
  launches += pl.blocks ? 1 : 0;
  // Visibility compaction.
  mark(p, GS3D_STAGE_COMPACT, st);
  const int depth_passes = p->desc.depth_sort_mode == GS3D_DEPTH_FLOAT32 ? 4 : 2;
  const uint32_t scan_grid = scan_chunks(N, p->sms);
  launch_compact(p->keys, N, p->vis_off, p->dk[0], p->dv[0], ctl, p->status, epoch(), scan_grid, st);
  ++launches;
  // Depth sort.
  mark(p, GS3D_STAGE_DEPTH_SORT, st);
  int cur = 0;
  const uint32_t depth_chunks = chunk_pass_chunks(N, p->sms);
  for (int pass = 0; pass < depth_passes; ++pass) {
    launch_chunk_pass(8, p->dk[cur], p->dv[cur], p->dk[cur ^ 1], p->dv[cur ^ 1], &ctl->visible_state[0], 8 * pass,
                      ctl->depth_hist[pass], depth_chunks, p->chunk_counts, &ctl->error, st);
    cur ^= 1;
    launches += 3;
  }
  p->depth_final = cur;
  // Ordered counts + saturating scan + dispatch/output state.
  mark(p, GS3D_STAGE_SCAN, st);
  const uint32_t cap32 = (uint32_t)p->capacity;
  launch_scan_counts(p->dv[cur], p->counts, p->ordered, p->ioff, ctl, p->status, epoch(), cap32, bv.frame_params,
                     p->output_state, scan_grid, st);
  ++launches;
  // Emission + tile-sort histograms.
  mark(p, GS3D_STAGE_EMIT, st);
  // Fewest passes with digits of at most tuning.tile_digit_bits, then the
  // narrowest digit; never more than the 4 passes the digit histograms hold
  // (the digit then widens past the tuning, up to 8 bits for 32-bit ids).
  const uint32_t tile_bits = std::max(1u, ceil_log2((uint64_t)tile + 1));
  const uint32_t max_digit = p->tuning.tile_digit_bits;
  const int tile_passes = (int)std::min<uint32_t>(kMaxSortPasses, (tile_bits + max_digit - 1) / max_digit);
  const int digit_bits = (int)((tile_bits + tile_passes - 1) / tile_passes);
  launch_emit(p->dv[cur], N, p->erec, p->ordered, p->ioff, bv, o, ctl, cap32, p->tk[0], p->tv[0], st);
  launches += N ? 1 : 0;
  // Tile sort.
  mark(p, GS3D_STAGE_TILE_SORT, st);
  int tcur = 0;
  const uint32_t tile_chunks = chunk_pass_chunks(cap32, p->sms);
  for (int pass = 0; pass < tile_passes; ++pass) {
    launch_chunk_pass(digit_bits, p->tk[tcur], p->tv[tcur], p->tk[tcur ^ 1], p->tv[tcur ^ 1], &ctl->state[0],
                      digit_bits * pass, ctl->tile_hist[pass], tile_chunks, p->chunk_counts, &ctl->error, st);
    tcur ^= 1;
    launches += 3;
  }
  p->tile_final = tcur;
  // Tile ranges and the raster work list.
  mark(p, GS3D_STAGE_RANGES, st);
  launch_tile_ranges(p->tk[tcur], ctl, tile, cap32, p->tile_offsets, st);
  ++launches;
  const bool ordered_tiles = p->tuning.work_order != 0u;
  if (ordered_tiles) {
    launch_tile_order(p->tile_offsets, tile, ctl, p->tile_order, p->sms, st);
    launches += 2;
  }
  // Raster.
  mark(p, GS3D_STAGE_RASTER, st);
  launch_raster((int)p->desc.raster_precision, p->tile_offsets, ordered_tiles ? p->tile_order : nullptr, p->tv[tcur],
                p->mean, p->conic,
                p->color, p->rec, bv, o, ctl, p->desc.raster_stats != 0, st);
  ++launches;
  mark(p, GS3D_STAGE_COUNT, st);
  if (p->profiling) ++p->profiled;
  p->last_launches = launches;
}

// The whole pass of TiledGaussianPipeline.render (TiledGaussianPipeline.ts:324-341)
// for every view of a batch in one launch sequence.
gs3d_status enqueue(gs3d_pipeline* p, const gs3d_view* views, uint32_t n, uint32_t attempt, int reset_valid,
                    cudaStream_t st, uint32_t tile, const uint32_t** frame_params = nullptr) {
  Plan pl;
  gs3d_status s = plan_batch(p, views, n, &pl, tile);
  if (s != GS3D_OK) return s;
  if ((s = ensure_stage(p, pl.stage_bytes)) != GS3D_OK) return s;
  const uint32_t slot = p->frame_index++ % kObjectRing;
  if (p->stage_ev_used[slot]) cudaEventSynchronize(p->stage_ev[slot]);
  stage_batch(p, views, pl, attempt, reset_valid, p->stage_pinned[slot], p->stage_dev[slot]);
  maybe_reset_epochs(p, st);
  cudaMemcpyAsync(p->stage_dev[slot], p->stage_pinned[slot], pl.stage_bytes, cudaMemcpyHostToDevice, st);
  record_batch(p, pl, p->stage_dev[slot], st);
  cudaEventRecord(p->stage_ev[slot], st);
  p->stage_ev_used[slot] = true;
  p->last_stream = st;
  if (frame_params) *frame_params = (const uint32_t*)p->stage_dev[slot];
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(p, e, "launching the pass");
  return GS3D_OK;
}

uint32_t views_per_launch(const gs3d_pipeline* p, uint32_t n) {
  const uint32_t v = p->tuning.views_per_launch;
  return v == 0u || v >= n ? n : v;
}

// A batch as launch sequences of at most tuning.views_per_launch views, one
// after another on the stream (they share the workspaces), with the batch's
// counts and output state summed up on the device.
gs3d_status enqueue_batch(gs3d_pipeline* p, const gs3d_view* views, uint32_t n, uint32_t attempt, int reset_valid,
                          cudaStream_t st) {
  const uint32_t per = views_per_launch(p, n);
  if (per >= n) {
    p->last_chunks = 1;
    return enqueue(p, views, n, attempt, reset_valid, st, batch_tile(p));
  }
  // Grow every workspace for the largest launch first, so no launch
  // sequence is queued on buffers that a later one reallocates.
  for (uint32_t k = 0; k < n; k += per) {
    Plan pl;
    gs3d_status s = plan_batch(p, views + k, std::min(per, n - k), &pl, batch_tile(p));
    if (s != GS3D_OK) return s;
    if ((s = ensure_stage(p, pl.stage_bytes)) != GS3D_OK) return s;
  }
  k_summary_begin<<<1, 1, 0, st>>>(p->summary, p->output_state);
  uint32_t launches = 1;
  for (uint32_t k = 0; k < n; k += per) {
    const uint32_t m = std::min(per, n - k);
    const uint32_t* params = nullptr;
    gs3d_status s = enqueue(p, views + k, m, attempt, reset_valid, st, batch_tile(p), &params);
    if (s != GS3D_OK) return s;
    launches += p->last_launches + 1;
    k_summary_add<<<1, 1, 0, st>>>(p->summary, p->ctl, params, p->output_state, k + m >= n ? 1 : 0);
  }
  p->last_chunks = (n + per - 1) / per;
  p->last_launches = launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(p, e, "launching the batch");
  return GS3D_OK;
}

}  // namespace

extern "C" {

gs3d_status gs3d_pipeline_render(gs3d_pipeline* p, const gs3d_camera* cam, uint32_t attempt, int reset_valid,
                                 const gs3d_targets* targets, void* stream) {
  if (!p) return GS3D_ERROR_INVALID_ARGUMENT;
  // TiledGaussianPipeline.ts:324-329
  if (!p->prepared) return fail(p, GS3D_ERROR_NOT_PREPARED, "TiledGaussianPipeline must be prepared before rendering");
  if (!cam || !targets) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "camera and color target required");
  cudaSetDevice(p->device);
  gs3d_view v;
  v.data = &p->data;
  v.camera = cam;
  v.width = p->width;
  v.height = p->height;
  v.targets = *targets;
  p->last_chunks = 1;
  // A single-view render keeps the reference's 16-pixel tiles, so every
  // buffer getResources() exposes is the reference's.
  return enqueue(p, &v, 1, attempt, reset_valid, (cudaStream_t)stream, kTileSize);
}

gs3d_status gs3d_pipeline_render_batch(gs3d_pipeline* p, const gs3d_view* views, uint32_t count, uint32_t attempt,
                                       int reset_valid, void* stream) {
  if (!p || !views) return GS3D_ERROR_INVALID_ARGUMENT;
  cudaSetDevice(p->device);
  p->prepared = true;
  return enqueue_batch(p, views, count, attempt, reset_valid, (cudaStream_t)stream);
}

gs3d_status gs3d_pipeline_capture_graph(gs3d_pipeline* p, const gs3d_view* views, uint32_t count, void* stream) {
  if (!p || !views) return GS3D_ERROR_INVALID_ARGUMENT;
  if (p->profiling) return fail(p, GS3D_ERROR_UNSUPPORTED, "disable profiling before capturing a graph");
  cudaSetDevice(p->device);
  cudaStream_t st = (cudaStream_t)stream;
  if (!st) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "graph capture needs a non-default stream");
  if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  release_graphs(p);
  // One staged batch table per launch sequence, back to back in one buffer;
  // every workspace is grown for the largest sequence before capturing.
  const uint32_t per = views_per_launch(p, count);
  std::vector<Plan> plans;
  p->graph_chunks.clear();
  size_t total = 0;
  for (uint32_t k = 0; k < count; k += per) {
    Plan pl;
    gs3d_status s = plan_batch(p, views + k, std::min(per, count - k), &pl, batch_tile(p));
    if (s != GS3D_OK) return s;
    plans.push_back(pl);
    p->graph_chunks.push_back({k, pl.n, total});
    total = align16(total + pl.stage_bytes);
  }
  const bool chunked = plans.size() > 1;
  uint32_t launches = chunked ? 1u : 0u;
  for (int g = 0; g < 2; ++g) {
    cudaError_t e = cudaMallocHost((void**)&p->graph_pinned[g], total);
    if (e == cudaSuccess) e = dalloc(p->graph_dev[g], total);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->graph_ev[g], cudaEventDisableTiming);
    if (e != cudaSuccess) {
      release_graphs(p);
      return cuda_fail(p, e, "allocating graph staging");
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      release_graphs(p);
      return cuda_fail(p, e, "beginning stream capture");
    }
    if (chunked) k_summary_begin<<<1, 1, 0, st>>>(p->summary, p->output_state);
    for (size_t c = 0; c < plans.size(); ++c) {
      unsigned char* dev = p->graph_dev[g] + p->graph_chunks[c].offset;
      record_batch(p, plans[c], dev, st);
      if (g == 0) launches += p->last_launches + (chunked ? 1u : 0u);
      if (chunked)
        k_summary_add<<<1, 1, 0, st>>>(p->summary, p->ctl, (const uint32_t*)dev, p->output_state,
                                       c + 1 == plans.size() ? 1 : 0);
    }
    e = cudaStreamEndCapture(st, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->graph_exec[g], graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      release_graphs(p);
      return cuda_fail(p, e, "capturing the pass");
    }
  }
  p->graph_stage_bytes = total;
  p->graph_tile = batch_tile(p);
  p->prepared = true;
  p->graph_views.assign(views, views + count);
  p->graph_cameras.resize(count);
  p->graph_launches = launches;
  p->graph_next = 0;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_launch_graph(gs3d_pipeline* p, const gs3d_camera* cameras, uint32_t count,
                                       uint32_t attempt, int reset_valid, void* stream) {
  if (!p || !cameras) return GS3D_ERROR_INVALID_ARGUMENT;
  if (!p->graph_exec[0]) return fail(p, GS3D_ERROR_NOT_PREPARED, "no captured graph");
  if (count != p->graph_views.size()) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "camera count differs from the capture");
  cudaSetDevice(p->device);
  cudaStream_t st = (cudaStream_t)stream;
  for (uint32_t i = 0; i < count; ++i) {
    if (cameras[i].object_count != p->graph_views[i].camera->object_count)
      return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "object count differs from the capture");
    p->graph_cameras[i] = cameras[i];
    p->graph_views[i].camera = &p->graph_cameras[i];
  }
  const int g = (int)(p->graph_next++ & 1u);
  if (p->graph_ev_used[g]) cudaEventSynchronize(p->graph_ev[g]);
  for (const auto& ch : p->graph_chunks) {
    Plan pl;
    pl.n = ch.count;
    pl.tile = p->graph_tile;
    size_t objects = 0;
    for (uint32_t i = 0; i < ch.count; ++i) objects += cameras[ch.first + i].object_count;
    layout_plan(&pl, ch.count, objects);
    stage_batch(p, p->graph_views.data() + ch.first, pl, attempt, reset_valid, p->graph_pinned[g] + ch.offset,
                p->graph_dev[g] + ch.offset);
  }
  maybe_reset_epochs(p, st);
  cudaMemcpyAsync(p->graph_dev[g], p->graph_pinned[g], p->graph_stage_bytes, cudaMemcpyHostToDevice, st);
  cudaError_t e = cudaGraphLaunch(p->graph_exec[g], st);
  cudaEventRecord(p->graph_ev[g], st);
  p->graph_ev_used[g] = true;
  p->last_stream = st;
  p->last_launches = p->graph_launches;
  p->last_chunks = (uint32_t)p->graph_chunks.size();
  if (e != cudaSuccess) return cuda_fail(p, e, "launching the graph");
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_set_tuning(gs3d_pipeline* p, const gs3d_tuning* t) {
  if (!p || !t) return GS3D_ERROR_INVALID_ARGUMENT;
  if (t->tile_digit_bits < 4 || t->tile_digit_bits > 8)
    return fail(p, GS3D_ERROR_RANGE, "tile_digit_bits must be in [4, 8]");
  if (t->work_order > 1) return fail(p, GS3D_ERROR_INVALID_ARGUMENT, "work_order must be 0 or 1");
  if (t->tile_size != 0 && t->tile_size != 8 && t->tile_size != 16 && t->tile_size != 32)
    return fail(p, GS3D_ERROR_RANGE, "tile_size must be 8, 16 or 32 (0: 16)");
  if (t->raster_pixels_per_lane != 0 && t->raster_pixels_per_lane != 2 && t->raster_pixels_per_lane != 4)
    return fail(p, GS3D_ERROR_RANGE, "raster_pixels_per_lane must be 2 or 4 (0: 2)");
  if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  release_graphs(p);  // captured graphs follow the tuning they were captured with
  p->tuning = *t;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_get_tuning(gs3d_pipeline* p, gs3d_tuning* t) {
  if (!p || !t) return GS3D_ERROR_INVALID_ARGUMENT;
  *t = p->tuning;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_autotune(gs3d_pipeline* p, const gs3d_view* views, uint32_t count, uint32_t trials,
                                   gs3d_tuning* best, double* best_ms, void* stream) {
  if (!p || !views || count == 0) return GS3D_ERROR_INVALID_ARGUMENT;
  if (trials == 0) trials = 3;
  cudaSetDevice(p->device);
  cudaStream_t st = (cudaStream_t)stream;
  if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  release_graphs(p);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // Milliseconds per batch with tuning t (one untimed render first, which
  // also grows the workspaces); an overflowing batch is an error, except for
  // a tile-size candidate (smaller tiles make more intersections), which is
  // then skipped (*ms stays infinite).
  auto measure = [&](const gs3d_tuning& t, double* ms) -> gs3d_status {
    p->tuning = t;
    *ms = HUGE_VAL;
    gs3d_status s = enqueue_batch(p, views, count, 1, 0, st);
    if (s != GS3D_OK) return s;
    gs3d_stats stats;
    if ((s = gs3d_pipeline_read_stats(p, &stats)) != GS3D_OK) return s;
    if (stats.overflow) {
      if (t.tile_size != 0 && t.tile_size != kTileSize) return GS3D_OK;
      return fail(p, GS3D_ERROR_RANGE, "intersection capacity too small for the batch");
    }
    cudaEventRecord(e0, st);
    for (uint32_t i = 0; i < trials; ++i)
      if ((s = enqueue_batch(p, views, count, 1, 0, st)) != GS3D_OK) return s;
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float f = 0.0f;
    cudaEventElapsedTime(&f, e0, e1);
    *ms = (double)f / trials;
    return GS3D_OK;
  };
  gs3d_tuning cur{0u, 8u, 1u, 0u, 0u, {0u, 0u, 0u}};
  double cur_ms = 0.0;
  gs3d_status s = measure(cur, &cur_ms);
  // Coordinate descent: tile size (8 and 32 against the reference's 16; the
  // raster block follows the tile), the fast rasterizers' pixels per lane
  // (the block shape), views per launch (halving), widest tile-sort digit,
  // then the raster work order.
  for (uint32_t ts : {8u, 32u}) {
    if (s != GS3D_OK) break;
    gs3d_tuning t = cur;
    t.tile_size = ts;
    double ms = 0.0;
    if ((s = measure(t, &ms)) == GS3D_OK && ms < cur_ms) { cur = t; cur_ms = ms; }
  }
  if (s == GS3D_OK && p->desc.raster_precision != GS3D_RASTER_EXACT) {
    gs3d_tuning t = cur;
    t.raster_pixels_per_lane = 4u;
    double ms = 0.0;
    if ((s = measure(t, &ms)) == GS3D_OK && ms < cur_ms) { cur = t; cur_ms = ms; }
  }
  for (uint32_t v = count / 2; s == GS3D_OK && v >= 1; v /= 2) {
    gs3d_tuning t = cur;
    t.views_per_launch = v;
    double ms = 0.0;
    if ((s = measure(t, &ms)) == GS3D_OK && ms < cur_ms) { cur = t; cur_ms = ms; }
    if (v == 1) break;
  }
  const gs3d_tuning by_views = cur;
  for (uint32_t d = 7; s == GS3D_OK && d >= 4; --d) {
    gs3d_tuning t = by_views;
    t.tile_digit_bits = d;
    double ms = 0.0;
    if ((s = measure(t, &ms)) == GS3D_OK && ms < cur_ms) { cur = t; cur_ms = ms; }
  }
  if (s == GS3D_OK) {
    gs3d_tuning t = cur;
    t.work_order = 0u;
    double ms = 0.0;
    if ((s = measure(t, &ms)) == GS3D_OK && ms < cur_ms) { cur = t; cur_ms = ms; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  p->tuning = cur;
  if (s != GS3D_OK) return s;
  if (best) *best = cur;
  if (best_ms) *best_ms = cur_ms;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_batch_layout(gs3d_pipeline* p, uint32_t* item_base, uint32_t* tile_base,
                                       uint32_t capacity, uint32_t* count) {
  if (!p || !count) return GS3D_ERROR_INVALID_ARGUMENT;
  const uint32_t n = p->item_bases.empty() ? 0u : (uint32_t)p->item_bases.size() - 1u;
  *count = n;
  for (uint32_t i = 0; i <= n && i < capacity; ++i) {
    if (item_base) item_base[i] = p->item_bases[i];
    if (tile_base) tile_base[i] = p->tile_bases[i];
  }
  return GS3D_OK;
}

}  // extern "C"

namespace {

// The counters of a finished render: the part of the control block from
// visible_state to raster_stats, and the batch summary (used when the batch
// ran as several launch sequences).
constexpr size_t kCountersOffset = offsetof(Control, visible_state);
constexpr size_t kCountersBytes = offsetof(Control, order_hist) - offsetof(Control, visible_state);
constexpr size_t kReadbackBytes = kCountersBytes + sizeof(BatchSummary) + 4 * sizeof(uint32_t);

gs3d_status fill_stats(gs3d_pipeline* p, const unsigned char* counters, const BatchSummary* summary, uint32_t chunks,
                       const uint32_t* output_state, gs3d_stats* out) {
  Control c;
  memcpy((unsigned char*)&c + kCountersOffset, counters, kCountersBytes);
  if (chunks > 1) {
    // A batch of several launch sequences: the totals of all of them.
    const BatchSummary& b = *summary;
    c.visible_state[0] = b.visible;
    c.state[0] = b.intersections;
    c.state[1] = b.requested;
    c.state[3] = b.overflow;
    c.error = b.error;
    for (int i = 0; i < 4; ++i) c.raster_stats[i] = b.raster[i];
  }
  memset(out, 0, sizeof(*out));
  out->visible_gaussian_count = c.visible_state[0];
  out->intersection_count = c.state[0];
  out->requested_intersections = c.state[1];
  out->overflow = c.state[3];
  out->intersection_capacity = p->capacity;
  out->device_error = c.error;
  out->raster_checked = c.raster_stats[0];
  out->raster_blended = c.raster_stats[1];
  out->raster_pixels = c.raster_stats[2];
  out->raster_alpha_stopped = c.raster_stats[3];
  for (int i = 0; i < 4; ++i) out->output_state[i] = output_state[i];
  if (c.error) return fail(p, GS3D_ERROR_DEVICE_TIMEOUT, "a device-side look-back wait expired");
  return GS3D_OK;
}

}  // namespace

extern "C" {

gs3d_status gs3d_pipeline_read_stats(gs3d_pipeline* p, gs3d_stats* out) {
  if (!p || !out) return GS3D_ERROR_INVALID_ARGUMENT;
  cudaSetDevice(p->device);
  cudaError_t e = cudaStreamSynchronize(p->last_stream);
  if (e != cudaSuccess) return cuda_fail(p, e, "synchronising the render stream");
  unsigned char counters[kCountersBytes];
  BatchSummary b{};
  e = cudaMemcpy(counters, (const unsigned char*)p->ctl + kCountersOffset, kCountersBytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(p, e, "reading the pass state");
  if (p->last_chunks > 1) {
    e = cudaMemcpy(&b, p->summary, sizeof(b), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(p, e, "reading the batch summary");
  }
  uint32_t output_state[4];
  e = cudaMemcpy(output_state, p->output_state, sizeof(output_state), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(p, e, "reading the output state");
  return fill_stats(p, counters, &b, p->last_chunks, output_state, out);
}

gs3d_status gs3d_pipeline_request_stats(gs3d_pipeline* p, void* stream) {
  if (!p) return GS3D_ERROR_INVALID_ARGUMENT;
  if (p->rb_pending) return fail(p, GS3D_ERROR_UNSUPPORTED, "a stats read-back is already in flight");
  cudaSetDevice(p->device);
  cudaError_t e = cudaSuccess;
  if (!p->rb_pinned && (e = cudaMallocHost((void**)&p->rb_pinned, kReadbackBytes)) != cudaSuccess) {
    p->rb_pinned = nullptr;
    return cuda_fail(p, e, "allocating the pinned read-back buffer");
  }
  if (!p->rb_event && (e = cudaEventCreateWithFlags(&p->rb_event, cudaEventDisableTiming)) != cudaSuccess) {
    p->rb_event = nullptr;
    return cuda_fail(p, e, "creating the read-back event");
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : p->last_stream;
  if (st != p->last_stream && p->last_stream) {
    // Order the copies after the last render's stream.
    if ((e = cudaEventRecord(p->rb_event, p->last_stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(st, p->rb_event, 0)) != cudaSuccess)
      return cuda_fail(p, e, "ordering the read-back after the render");
  }
  p->rb_chunks = p->last_chunks;
  if ((e = cudaMemcpyAsync(p->rb_pinned, (const unsigned char*)p->ctl + kCountersOffset, kCountersBytes,
                           cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (p->rb_chunks > 1 && (e = cudaMemcpyAsync(p->rb_pinned + kCountersBytes, p->summary, sizeof(BatchSummary),
                                                cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
      (e = cudaMemcpyAsync(p->rb_pinned + kCountersBytes + sizeof(BatchSummary), p->output_state,
                           4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaEventRecord(p->rb_event, st)) != cudaSuccess)
    return cuda_fail(p, e, "enqueueing the stats read-back");
  p->rb_pending = true;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_poll_stats(gs3d_pipeline* p, gs3d_stats* out, int wait) {
  if (!p || !out) return GS3D_ERROR_INVALID_ARGUMENT;
  if (!p->rb_pending) return fail(p, GS3D_ERROR_NOT_PREPARED, "no stats read-back was requested");
  cudaSetDevice(p->device);
  cudaError_t e = wait ? cudaEventSynchronize(p->rb_event) : cudaEventQuery(p->rb_event);
  if (e == cudaErrorNotReady) return GS3D_NOT_READY;
  p->rb_pending = false;
  if (e != cudaSuccess) return cuda_fail(p, e, "waiting for the stats read-back");
  return fill_stats(p, p->rb_pinned, (const BatchSummary*)(p->rb_pinned + kCountersBytes), p->rb_chunks,
                    (const uint32_t*)(p->rb_pinned + kCountersBytes + sizeof(BatchSummary)), out);
}

gs3d_status gs3d_pipeline_set_wait_limit(gs3d_pipeline* p, uint32_t polls) {
  if (!p) return GS3D_ERROR_INVALID_ARGUMENT;
  if (p->last_stream) cudaStreamSynchronize(p->last_stream);
  release_graphs(p);  // captured graphs hold the limit they were captured with
  p->wait_limit = polls;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_debug_withhold_chunk(gs3d_pipeline* p) {
  if (!p) return GS3D_ERROR_INVALID_ARGUMENT;
  p->withhold_first_chunk = true;
  return GS3D_OK;
}

void gs3d_debug_fail_allocation(uint32_t nth) { g_fail_countdown.store((int64_t)nth); }

gs3d_status gs3d_pipeline_get_resources(gs3d_pipeline* p, gs3d_resources* r) {
  if (!p || !r) return GS3D_ERROR_INVALID_ARGUMENT;
  if (!p->prepared) return fail(p, GS3D_ERROR_NOT_PREPARED, "TiledGaussianPipeline must be prepared first");
  memset(r, 0, sizeof(*r));
  r->projected_mean = (const float*)p->mean;
  r->projected_conic = (const float*)p->conic;
  r->projected_color = (const float*)p->color;
  r->tile_counts = p->counts;
  r->visible_offsets = p->vis_off;
  r->depth_sorted_keys = p->dk[p->depth_final];
  r->depth_sorted_ids = p->dv[p->depth_final];
  r->depth_ordered_tile_counts = p->ordered;
  r->intersection_offsets = p->ioff;
  r->dispatch_state = p->ctl->state;
  r->visible_state = p->ctl->visible_state;
  r->sorted_tile_ids = p->tk[p->tile_final];
  r->sorted_gaussian_ids = p->tv[p->tile_final];
  r->tile_offsets = p->tile_offsets;
  r->output_state = p->output_state;
  r->active_count = p->total_items;
  r->tiles_x = p->tiles_x;
  r->tiles_y = p->tiles_y;
  r->total_tiles = p->total_tiles;
  r->intersection_capacity = p->capacity;
  return GS3D_OK;
}

const char* gs3d_pipeline_last_error(gs3d_pipeline* p) { return p ? p->error.c_str() : ""; }

uint32_t gs3d_pipeline_last_launch_count(gs3d_pipeline* p) { return p ? p->last_launches : 0u; }

gs3d_status gs3d_pipeline_set_profiling(gs3d_pipeline* p, int enabled) {
  if (!p) return GS3D_ERROR_INVALID_ARGUMENT;
  p->profiling = enabled != 0;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_stage_times(gs3d_pipeline* p, float* ms, uint32_t* renders) {
  if (!p || !ms) return GS3D_ERROR_INVALID_ARGUMENT;
  cudaSetDevice(p->device);
  for (uint32_t s = 0; s < GS3D_STAGE_COUNT; ++s) ms[s] = 0.0f;
  const uint32_t n = p->profiled;
  for (uint32_t r = 0; r < n; ++r) {
    cudaEvent_t* ev = p->events.data() + (size_t)r * kStageEvents;
    cudaError_t e = cudaEventSynchronize(ev[GS3D_STAGE_COUNT]);
    if (e != cudaSuccess) return cuda_fail(p, e, "waiting for profiled render");
    for (uint32_t s = 0; s < GS3D_STAGE_COUNT; ++s) {
      float t = 0.0f;
      cudaEventElapsedTime(&t, ev[s], ev[s + 1]);
      ms[s] += t;
    }
  }
  if (n)
    for (uint32_t s = 0; s < GS3D_STAGE_COUNT; ++s) ms[s] /= (float)n;
  if (renders) *renders = n;
  p->profiled = 0;
  return GS3D_OK;
}

gs3d_status gs3d_pipeline_read_profile(gs3d_pipeline* p, gs3d_profile_stats* out) {
  if (!p || !out) return GS3D_ERROR_INVALID_ARGUMENT;
  if (!p->prepared) return fail(p, GS3D_ERROR_NOT_PREPARED, "render a frame before reading the profile");
  cudaSetDevice(p->device);
  cudaError_t e = cudaSuccess;
  if (!p->profile_sums &&
      ((e = dalloc(p->profile_sums, 1)) || (e = dalloc(p->profile_hist, 65536)) || (e = dalloc(p->profile_zero, 1))))
    return cuda_fail(p, e, "allocating profile scratch");
  cudaStream_t st = p->last_stream;
  const uint32_t ntile = p->total_tiles, n = p->total_items;
  cudaMemsetAsync(p->profile_sums, 0, sizeof(TileLoadSums), st);
  cudaMemsetAsync(p->profile_hist, 0, 65536 * sizeof(uint32_t), st);
  cudaMemsetAsync(p->profile_zero, 0, sizeof(uint32_t), st);
  // PROFILE_TILE_CAPS (utils/profileStats.ts:7) and the configured cap.
  const uint32_t caps[4] = {2048u, 4096u, 8192u, p->desc.max_rasterized_splats_per_tile};
  launch_profile(p->mean, p->conic, p->last_bv, n, p->tile_offsets, ntile, caps, p->profile_sums, p->profile_hist,
                 p->profile_zero, st);
  TileLoadSums sums;
  std::vector<uint32_t> hist(65536);
  uint32_t zero = 0;
  if ((e = cudaMemcpyAsync(&sums, p->profile_sums, sizeof(sums), cudaMemcpyDeviceToHost, st)) ||
      (e = cudaMemcpyAsync(hist.data(), p->profile_hist, 65536 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) ||
      (e = cudaMemcpyAsync(&zero, p->profile_zero, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) ||
      (e = cudaStreamSynchronize(st)))
    return cuda_fail(p, e, "reading the profile");
  memset(out, 0, sizeof(*out));
  out->zero_pixel_subpixel_splats = zero;
  gs3d_tile_load_stats& L = out->tile_loads;
  if (ntile) {
    // The k-th smallest load from the histogram; loads past its last bin are
    // read back exactly from the tile offsets.
    std::vector<uint32_t> exact;
    auto kth = [&](uint64_t k) -> uint32_t {
      uint64_t run = 0;
      for (uint32_t b = 0; b < 65535u; ++b) {
        run += hist[b];
        if (k < run) return b;
      }
      if (exact.empty()) {
        std::vector<uint32_t> off(ntile + 1);
        cudaMemcpy(off.data(), p->tile_offsets, (ntile + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        for (uint32_t t = 0; t < ntile; ++t)
          if (off[t + 1] > off[t] && off[t + 1] - off[t] >= 65535u) exact.push_back(off[t + 1] - off[t]);
        std::sort(exact.begin(), exact.end());
      }
      return exact.empty() ? 65535u : exact[std::min<uint64_t>(k - run, exact.size() - 1)];
    };
    L.max = sums.max;
    L.mean = (double)sums.total / (double)ntile;
    const uint32_t mid = ntile / 2;
    L.median = (ntile % 2) ? (double)kth(mid) : ((double)kth(mid - 1) + (double)kth(mid)) * 0.5;
    const auto pct = [&](double f) { return kth((uint64_t)std::max<int64_t>(0, (int64_t)std::ceil(ntile * f) - 1)); };
    L.p95 = pct(0.95);
    L.p99 = pct(0.99);
    L.tiles_over_256 = sums.over[0];
    L.tiles_over_512 = sums.over[1];
    L.tiles_over_1024 = sums.over[2];
    L.tiles_over_2048 = sums.over[3];
    L.total_batches = sums.batches;
    L.max_batches = sums.max_batches;
  }
  auto cap_stats = [&](int k, gs3d_tile_cap_stats* c) {
    c->cap = caps[k];
    c->rasterized_intersections = sums.cap_rasterized[k];
    c->dropped_intersections = sums.cap_dropped[k];
    const uint64_t emitted = sums.cap_rasterized[k] + sums.cap_dropped[k];
    c->dropped_fraction = emitted == 0 ? 0.0 : (double)sums.cap_dropped[k] / (double)emitted;
    c->affected_tiles = sums.cap_affected[k];
    c->total_batches = sums.cap_batches[k];
    c->max_batches = sums.cap_max_batches[k];
  };
  for (int k = 0; k < 3; ++k) cap_stats(k, &out->cap_estimates[k]);
  out->has_applied_cap = caps[3] != 0u;
  if (out->has_applied_cap) cap_stats(3, &out->applied_cap);
  return GS3D_OK;
}

const char* gs3d_stage_name(uint32_t stage) {
  static const char* names[GS3D_STAGE_COUNT] = {"project", "compact", "depth_sort", "scan",
                                                "emit", "tile_sort", "ranges", "raster"};
  return stage < GS3D_STAGE_COUNT ? names[stage] : "unknown";
}

uint64_t gs3d_capacity_next(uint64_t maximum, double growth, double headroom, uint64_t current, uint64_t demand) {
  // IntersectionCapacityPolicy.ts:90-100
  if (demand > maximum) return 0;
  const double a = ceil((double)demand * headroom);
  const double b = ceil((double)current * growth);
  const double desired = a > b ? a : b;
  const double rounded = ceil(desired / 256.0) * 256.0;
  return (uint64_t)(rounded < (double)maximum ? rounded : (double)maximum);
}

}  // extern "C"
