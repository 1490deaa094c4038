// Onesweep-style stable LSD radix sort pass over (uint32 key, uint32 value).
//
// Replaces the reference's 4-bit, 5-dispatch-per-pass radix sort
// (src/renderer/kernels/radix.ts:10-263, src/renderer/pipeline/RadixSorter.ts:50-322),
// which is a stable LSD sort; stability is the property the pass depends on
// (records enter in ordinal order for the depth sort and in depth-rank order
// for the tile sort, TiledGaussianPipeline.ts:144,442-446).
//
// One pass = one kernel. The digit histograms of every pass were accumulated
// by the kernel that produced the keys, so each block only:
//   1. takes the next tile id from an atomic ticket (tiles are processed in
//      launch order, which keeps the look-back deadlock-free);
//   2. ranks its 4096 keys per digit with __match_any_sync (warp-striped
//      layout: item j*32+lane of each warp's 512-item segment, so ranks follow
//      index order and the sort is stable);
//   3. publishes its per-digit counts and resolves its global per-digit base
//      with decoupled look-back (one thread per digit, bounded waits);
//   4. stages keys and values in shared memory in block-sorted order and
//      writes each digit's run contiguously to global memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pass_common.cuh"

namespace gs {

constexpr int kSortWarps = 8;
constexpr int kSortItems = 16;  // kSortTile = 8 warps * 32 lanes * 16 items

template <int BITS>
__global__ void __launch_bounds__(kBlock, 2)
    k_onesweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
               uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, const uint32_t* __restrict__ n_ptr,
               int shift, const uint32_t* __restrict__ hist, unsigned long long* __restrict__ status,
               uint32_t* __restrict__ ticket, uint32_t epoch, uint32_t* __restrict__ err) {
  constexpr uint32_t RADIX = 1u << BITS;
  constexpr uint32_t MASK = RADIX - 1u;
  constexpr uint32_t INVALID = 0xffffu;
  __shared__ uint32_t s_warp_hist[kSortWarps][RADIX];
  __shared__ uint32_t s_block_excl[RADIX];
  __shared__ uint32_t s_global_base[RADIX];
  __shared__ uint32_t s_hist_excl[RADIX];
  __shared__ uint32_t s_keys[kSortTile];
  __shared__ uint32_t s_vals[kSortTile];
  __shared__ uint32_t s_scan[kBlock / 32];
  __shared__ uint32_t s_tile;

  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(ticket, 1u);
  for (uint32_t i = tid; i < kSortWarps * RADIX; i += kBlock) (&s_warp_hist[0][0])[i] = 0u;
  __syncthreads();
  const uint32_t n = *n_ptr;
  const uint32_t tile = s_tile;
  const uint32_t base = tile * kSortTile;
  if (base >= n) return;

  // Exclusive scan of the pass's global digit histogram.
  {
    uint32_t h = tid < RADIX ? hist[tid] : 0u;
    uint32_t tot;
    uint32_t e = block_exclusive_scan<false>(h, s_scan, &tot);
    if (tid < RADIX) s_hist_excl[tid] = e;
  }

  // Load (warp-striped) and rank.
  const uint32_t wbase = base + warp * 32u * kSortItems;
  uint32_t k[kSortItems], v[kSortItems], rank[kSortItems];
  uint32_t d[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    const bool ok = idx < n;
    k[j] = ok ? keys_in[idx] : 0u;
    v[j] = ok ? vals_in[idx] : 0u;
    d[j] = ok ? (k[j] >> shift) & MASK : INVALID;
  }
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t peers = __match_any_sync(0xffffffffu, d[j]);
    const uint32_t leader = __ffs(peers) - 1u;
    const uint32_t before = __popc(peers & lt);
    uint32_t cnt = 0;
    if (d[j] != INVALID) cnt = s_warp_hist[warp][d[j]];
    rank[j] = cnt + before;
    __syncwarp();
    if (lane == leader && d[j] != INVALID) s_warp_hist[warp][d[j]] = cnt + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Per digit: exclusive offsets across warps and the block count.
  uint32_t block_count = 0;
  if (tid < RADIX) {
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = s_warp_hist[w][tid];
      s_warp_hist[w][tid] = block_count;
      block_count += c;
    }
    unsigned long long* mine = status + (size_t)tile * RADIX + tid;
    st_release(mine, pack_status(epoch, tile == 0 ? kFlagInclusive : kFlagAggregate, block_count));
  }
  {
    uint32_t tot;
    const uint32_t e = block_exclusive_scan<false>(tid < RADIX ? block_count : 0u, s_scan, &tot);
    if (tid < RADIX) s_block_excl[tid] = e;
  }
  if (tid < RADIX) {
    uint32_t prefix = 0;
    if (tile > 0) {
      prefix = lookback<false>(status + tid, RADIX, tile, epoch, err);
      st_release(status + (size_t)tile * RADIX + tid, pack_status(epoch, kFlagInclusive, prefix + block_count));
    }
    s_global_base[tid] = s_hist_excl[tid] + prefix;
  }
  __syncthreads();

  // Stage in block-sorted order.
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    if (d[j] != INVALID) {
      const uint32_t pos = s_block_excl[d[j]] + s_warp_hist[warp][d[j]] + rank[j];
      s_keys[pos] = k[j];
      s_vals[pos] = v[j];
    }
  }
  __syncthreads();

  // Scatter: consecutive positions of one digit go to consecutive addresses.
  const uint32_t count = min(kSortTile, n - base);
  for (uint32_t i = tid; i < count; i += kBlock) {
    const uint32_t key = s_keys[i];
    const uint32_t dig = (key >> shift) & MASK;
    const uint32_t dst = s_global_base[dig] + (i - s_block_excl[dig]);
    keys_out[dst] = key;
    vals_out[dst] = s_vals[i];
  }
}

void launch_onesweep(int bits, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                     uint32_t* vals_out, const uint32_t* n_ptr, uint32_t n_max, int shift, const uint32_t* hist,
                     unsigned long long* status, uint32_t* ticket, uint32_t epoch, uint32_t* err, cudaStream_t st) {
  const uint32_t grid = n_max == 0 ? 1u : (uint32_t)(((uint64_t)n_max + kSortTile - 1) / kSortTile);
#define GS_SWEEP(B)                                                                                         \
  case B:                                                                                                   \
    k_onesweep<B><<<grid, kBlock, 0, st>>>(keys_in, vals_in, keys_out, vals_out, n_ptr, shift, hist, status, \
                                           ticket, epoch, err);                                             \
    break;
  switch (bits) {
    GS_SWEEP(1)
    GS_SWEEP(2)
    GS_SWEEP(3)
    GS_SWEEP(4)
    GS_SWEEP(5)
    GS_SWEEP(6)
    GS_SWEEP(7)
    default:
      GS_SWEEP(8)
  }
#undef GS_SWEEP
}

}  // namespace gs
