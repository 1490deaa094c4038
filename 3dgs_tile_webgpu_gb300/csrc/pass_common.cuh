// Shared definitions of the CUDA pass: kernel parameter blocks, the per-frame
// control block, and the decoupled look-back protocol used by the compaction
// and scan kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gs {

constexpr int kBlock = 256;  // threads per block for the linear kernels
constexpr uint32_t kTileSize = 16;  // the reference's pixels per tile side (src/renderer/pipeline/constants.ts:1)

// One view of a batch: a scene (packed GaussianData buffers), a camera
// (FrameUniforms.ts:18-58 + the object table), a viewport and its targets.
// Views are concatenated: view v owns items [item_base, item_base + active)
// (item_base is a multiple of kBlock so every projection block belongs to one
// view) and global tile ids [tile_base, tile_base + tiles_x * tiles_y).
struct ViewDesc {
  const float4* means;     // count
  const uint2* shape;      // count
  const uint32_t* rot;     // count
  const uint32_t* sh;      // count * C + count (active tail at count * C)
  const float* objects;    // object_count * 40
  void* color;             // rgba16f or rgba32f, width * height
  float* depth;            // width * height or null
  uint32_t count, active, degree, C;
  uint32_t object_count, color_half;
  uint32_t tiles_x, tiles_y;
  uint32_t item_base, tile_base, pad0, pad1;
  float P[16];             // projection, column-major
  float vw, vh, vnear, vfar;
};

// Pass options shared by every view (TiledGaussianPipeline constructor options).
struct PassOptions {
  float filter;
  uint32_t axis;           // boundary axis 0/1/2
  uint32_t antialias;      // 0 compensated, 1 classic
  uint32_t subpixel;       // subpixel sample culling
  uint32_t depth_mode;     // 0 float32, 1 packed16
  uint32_t chunk;          // raster chunk size, 0 = none
  uint32_t max_per_tile;   // 0 = uncapped
  uint32_t depth_encoding; // 0 device depth, 1 raw
  float background[4];
  float t_threshold;
  float depth_alpha_threshold;
  float invalid_depth;
  uint32_t proj_fp64;      // 1: FP64 far-origin mean transform and near-singular conic
  uint32_t any_depth;      // some view of the launch has a depth target
  uint32_t tile;           // pixels per tile side: 16 (the reference's), or 8 / 32 in tuned batches
  float tile_px;           // the same as a float
  float tile_inv;          // its reciprocal (exact: a power of two)
  uint32_t pixels_per_lane;  // fast raster forms: 2 (a warp per 8x8 patch) or 4 (per 8x16)
};

// The batch table in device memory: the per-frame parameters (attempt,
// reset_valid), four ascending arrays (nviews + 1 entries each), then the view
// descriptors. Consecutive views that render the same packed scene form a view
// group, projected together (group_block: first projection block of each
// group; group_view: first view of each group; ngroups + 1 entries used).
struct BatchView {
  const uint32_t* item_base;
  const uint32_t* tile_base;
  const uint32_t* group_block;
  const uint32_t* group_view;
  const ViewDesc* views;
  const uint32_t* frame_params;  // attempt, reset_valid
  uint32_t nviews;
  uint32_t ngroups;
  uint32_t total_items;
  uint32_t total_tiles;
  uint32_t total_blocks;         // projection blocks over the groups
};

// Index of the view whose [base[v], base[v+1]) range holds x.
__device__ __forceinline__ uint32_t find_view(const uint32_t* base, uint32_t nviews, uint32_t x) {
  uint32_t lo = 0, hi = nviews;  // base[lo] <= x < base[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(base + mid) <= x) lo = mid; else hi = mid;
  }
  return lo;
}

constexpr uint32_t kMaxSortPasses = 4;  // digit histograms held per sort
// Persistent blocks per SM of the chunked look-back scans (compaction and
// ordered-count scan); scan_chunks() = their grid for n_max items.
constexpr uint32_t kScanBlocksPerSm = 4;
uint32_t scan_chunks(uint32_t n_max, int sms);

// Per-frame control block, zeroed before each render.
struct Control {
  uint32_t tickets[2];           // dynamic tile ids of the look-back kernels (Ticket)
  uint32_t depth_hist[kMaxSortPasses][256];  // digit histograms of the depth sort (its count kernels)
  uint32_t tile_hist[kMaxSortPasses][256];   // digit histograms of the tile sort (its count kernels)
  uint32_t visible_state[4];     // visible, visible, radix blocks, 0
  uint32_t state[4];             // count, total, radix blocks, overflow
  uint32_t error;                // bit 0: look-back wait expired; bit 2: a sort tile copy never landed
  uint32_t pad[3];
  unsigned long long raster_stats[4];  // checked, blended, pixels, alpha-stopped
  uint32_t order_hist[34];       // raster work-list buckets (tile load classes)
  uint32_t order_fill[34];
};

enum Ticket { kTicketCompact = 0, kTicketScan = 1 };

// ---------------------------------------------------------------------------
// Decoupled look-back status words: [63:34] epoch, [33:32] flag, [31:0] value.
// A word whose epoch differs from the launch's epoch is "not yet published",
// so the status array never needs clearing between launches. A frame's
// launches use epochs base + 1 .. base + kEpochsPerFrame, where base is a
// device-side counter advanced by k_epoch_begin at the start of every frame,
// so a replayed CUDA graph never reuses an epoch.
constexpr uint32_t kEpochsPerFrame = 16;

constexpr uint32_t kSpinLimit = 1u << 22;  // default polls before a wait is declared expired (about 1 s)

// The epoch of look-back launch `add` of the current frame, and how many
// polls a wait of that launch may spend on one status word.
struct Epoch {
  const uint32_t* base;  // device counter
  uint32_t add;
  uint32_t spin_limit;   // 0: kSpinLimit
  __device__ __forceinline__ uint32_t get() const { return *base + add; }
  __device__ __forceinline__ uint32_t limit() const { return spin_limit ? spin_limit : kSpinLimit; }
};
constexpr unsigned long long kFlagAggregate = 1ull;
constexpr unsigned long long kFlagInclusive = 2ull;

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long pack_status(uint32_t epoch, unsigned long long flag, uint32_t value) {
  return ((unsigned long long)epoch << 34) | (flag << 32) | (unsigned long long)value;
}
__device__ __forceinline__ uint32_t sat_add(uint32_t a, uint32_t b) { return a + min(b, 0xffffffffu - a); }

// Wait (bounded) until *p carries this launch's epoch. On expiry the error
// word gets bit 0 and the caller treats the word as an inclusive zero, so the
// kernel always finishes and the host sees the error.
__device__ __forceinline__ unsigned long long wait_status(const unsigned long long* p, unsigned long long v,
                                                          uint32_t epoch, uint32_t limit, uint32_t* err,
                                                          bool* expired) {
  uint32_t polls = 0, backoff = 8;
  while ((uint32_t)(v >> 34) != epoch) {
    if (++polls >= limit) {
      atomicOr(err, 1u);
      *expired = true;
      return 0;
    }
    __nanosleep(backoff);
    backoff = backoff < 256 ? backoff * 2 : 256;
    v = ld_acquire(p);
  }
  return v;
}

// Warp-wide decoupled look-back for a single value per tile: every lane
// requests K predecessors at once (lane l reads tile end - 32 k - l), so one
// round trip covers 32 K tiles; the sub-windows are then resolved nearest
// first, waiting only on the ones needed before an inclusive prefix turns up.
// Returns the exclusive prefix of `tile` in every lane. All 32 lanes of the
// warp must call it.
template <bool SATURATE, int K = 4>
__device__ __forceinline__ uint32_t warp_lookback(const unsigned long long* status, uint32_t tile, uint32_t epoch,
                                                  uint32_t limit, uint32_t* err) {
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t excl = 0;
  int64_t end = (int64_t)tile - 1;
  while (end >= 0) {
    unsigned long long v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int64_t idx = end - 32 * k - (int64_t)lane;
      v[k] = idx >= 0 ? ld_acquire(status + idx) : 0ull;
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (end - 32 * k < 0) return excl;  // no predecessors left
      const int64_t idx = end - 32 * k - (int64_t)lane;
      bool incl = true, expired = false;
      uint32_t val = 0;
      if (idx >= 0) {
        const unsigned long long w = wait_status(status + idx, v[k], epoch, limit, err, &expired);
        incl = expired || ((w >> 32) & 3ull) == kFlagInclusive;
        val = expired ? 0u : (uint32_t)w;
      }
      const uint32_t inc_mask = __ballot_sync(0xffffffffu, incl);
      const uint32_t stop = inc_mask ? (uint32_t)(__ffs(inc_mask) - 1) : 31u;  // nearest inclusive lane
      uint32_t x = lane <= stop ? val : 0u;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, o);
        x = SATURATE ? sat_add(x, y) : x + y;
      }
      excl = SATURATE ? sat_add(excl, x) : excl + x;
      if (inc_mask) return excl;
    }
    end -= 32 * K;
  }
  return excl;
}

// ---------------------------------------------------------------------------
// Block-wide exclusive scan of one value per thread (256 threads).
template <bool SATURATE>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x = SATURATE ? sat_add(y, x) : y + x;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < (kBlock / 32) ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w = SATURATE ? sat_add(y, w) : y + w;
    }
    if (lane < (kBlock / 32)) s_warp[lane] = w;
  }
  __syncthreads();
  uint32_t warp_prefix = warp == 0 ? 0u : s_warp[warp - 1];
  uint32_t incl = SATURATE ? sat_add(warp_prefix, x) : warp_prefix + x;
  *total = s_warp[kBlock / 32 - 1];
  // Exclusive value = the previous thread's inclusive value (exact for the
  // saturating form too, since saturating addition is associative).
  uint32_t prev = __shfl_up_sync(0xffffffffu, incl, 1);
  uint32_t excl = lane == 0 ? warp_prefix : prev;
  __syncthreads();
  return excl;
}

// Launch wrappers implemented in the .cu files.
// Packed raster record of a visible splat, read by the fast raster forms with
// one 32-byte gather (two float4, 32-byte aligned):
//   [0] cx, cy, -a/2 log2 e, -b log2 e
//   [1] -c/2 log2 e, log2 opacity, half2(r, g) bits, half2(b, min(log2 opacity, log2 0.99)) bits
// where (a, b, c) is the conic. Written by the projection when `rec` is not null.
// rec: packed raster records of the fast forms (null for EXACT); erec: the
// emission records, two float4 per item: (cx, cy, conic a, conic b),
// (conic c, log(opacity * 255), rx + 512 ry, 0), written for visible items.
void launch_project(const BatchView& b, const PassOptions& o, float4* mean, float4* conic, float4* color,
                    uint32_t* counts, uint32_t* keys, float4* rec, float4* erec, cudaStream_t st);
void launch_epoch_begin(uint32_t* epoch_base, cudaStream_t st);
// Advance ticket counter `ticket` of the control block by one (a test hook:
// the chunk of ticket 0 is then never scanned, so its successor's look-back
// wait runs out).
void launch_skip_ticket(Control* ctl, uint32_t ticket, cudaStream_t st);
void launch_compact(const uint32_t* keys, uint32_t n, uint32_t* vis_off, uint32_t* keys_out, uint32_t* vals_out,
                    Control* ctl, unsigned long long* status, Epoch epoch, uint32_t chunks, cudaStream_t st);
void launch_scan_counts(const uint32_t* sorted_ids, const uint32_t* tile_counts, uint32_t* ordered,
                        uint32_t* offsets, Control* ctl, unsigned long long* status, Epoch epoch,
                        uint32_t capacity, const uint32_t* frame_params, uint32_t* output_state, uint32_t chunks,
                        cudaStream_t st);
void launch_emit(const uint32_t* sorted_ids, uint32_t n_max, const float4* erec, const uint32_t* ordered,
                 const uint32_t* offsets, const BatchView& b, const PassOptions& o, Control* ctl, uint32_t capacity,
                 uint32_t* tile_keys, uint32_t* tile_vals, cudaStream_t st);
void launch_tile_ranges(const uint32_t* sorted_tile_keys, Control* ctl, uint32_t ntile, uint32_t n_max,
                        uint32_t* tile_offsets, cudaStream_t st);
constexpr uint32_t kSortTile = 4096;  // items per sort tile
// Chunked LSD pass (reduce, scan, scatter; no look-back chain): `chunks`
// blocks, each walking a contiguous run of 4096-item tiles. counts holds
// chunks x 2^bits words; hist (2^bits words, zero on entry) receives the
// pass's digit histogram. n is read from *n_ptr on the device.
constexpr uint32_t kChunkBlocksPerSm = 3;
uint32_t chunk_pass_chunks(uint32_t n_max, int sms);
// err: the control block's error word (bit 2: a tile copy of the scatter
// never landed).
void launch_chunk_pass(int bits, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                       uint32_t* vals_out, const uint32_t* n_ptr, int shift, uint32_t* hist, uint32_t chunks,
                       uint32_t* counts, uint32_t* err, cudaStream_t st);
// Opt every sort-scatter instantiation into its shared-memory size (once per
// device; call before any stream capture).
void prepare_sort_kernels();
// Raster work list: every tile of the batch, heaviest load class first.
void launch_tile_order(const uint32_t* tile_offsets, uint32_t ntile, Control* ctl, uint32_t* order, int sms,
                       cudaStream_t st);
// Rasterizer over every tile of the batch (precision: 0 fp32, 1 exact, 2 half2).
void launch_raster(int precision, const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* sorted_ids,
                   const float4* mean, const float4* conic, const float4* color, const float4* rec,
                   const BatchView& b, const PassOptions& o, Control* ctl, bool stats, cudaStream_t st);
// Profiling diagnostics: tile-load sums (caps: up to four, 0 = unused) and
// the zero-pixel subpixel splat count (ProfileDiagnosticsStage.ts:22-116).
struct TileLoadSums {
  unsigned long long total, batches;
  uint32_t max, max_batches, over[4];
  unsigned long long cap_rasterized[4], cap_dropped[4], cap_batches[4];
  uint32_t cap_affected[4], cap_max_batches[4];
};
void launch_profile(const float4* mean, const float4* conic, const BatchView& b, uint32_t n,
                    const uint32_t* tile_offsets, uint32_t ntile, const uint32_t caps[4], TileLoadSums* sums,
                    uint32_t* hist, uint32_t* zero_count, cudaStream_t st);
void launch_raster_exact(const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* sorted_ids,
                         const float4* mean, const float4* conic, const float4* color, const BatchView& b,
                         const PassOptions& o, Control* ctl, bool stats, cudaStream_t st);

}  // namespace gs
