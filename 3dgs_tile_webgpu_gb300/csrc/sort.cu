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
//   2. ranks its 4096 keys per digit within each warp by ballot bit-splitting
//      (warp-striped layout: item j*32+lane of each warp's 512-item segment,
//      so ranks follow index order and the sort is stable), while the values
//      stream into shared memory with cp.async;
//   3. publishes its per-digit counts and resolves its global per-digit base
//      with decoupled look-back (one thread per digit, bounded waits);
//   4. stages keys and values in shared memory in block-sorted order and
//      writes each digit's run contiguously to global memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pass_common.cuh"

namespace gs {

constexpr int kSortWarps = 8;
constexpr int kSortWindow = 8;  // predecessor tiles requested per look-back round trip, per digit
constexpr int kSortItems = 16;  // kSortTile = 8 warps * 32 lanes * 16 items

// Lanes of the warp holding the same BITS-bit digit, by ballot bit-splitting.
template <int BITS>
__device__ __forceinline__ uint32_t match_digit(uint32_t d, uint32_t valid_mask) {
  uint32_t peers = valid_mask;
#pragma unroll
  for (int b = 0; b < BITS; ++b) {
    const bool bit = (d >> b) & 1u;
    const uint32_t bal = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? bal : ~bal;
  }
  return peers;
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit_wait() {
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_all;" ::: "memory");
}

template <int BITS>
__global__ void __launch_bounds__(kBlock, 3)
    k_onesweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
               uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, const uint32_t* __restrict__ n_ptr,
               int shift, const uint32_t* __restrict__ hist, unsigned long long* __restrict__ status,
               uint32_t* __restrict__ ticket, Epoch ep, uint32_t* __restrict__ err) {
  constexpr uint32_t RADIX = 1u << BITS;
  constexpr uint32_t MASK = RADIX - 1u;
  __shared__ uint32_t s_warp_hist[kSortWarps][RADIX];
  __shared__ uint32_t s_block_excl[RADIX];
  __shared__ uint32_t s_global_base[RADIX];
  __shared__ uint32_t s_hist_excl[RADIX];
  extern __shared__ uint4 s_dyn[];  // keys, values, raw values: 3 x kSortTile words
  uint32_t* s_keys = reinterpret_cast<uint32_t*>(s_dyn);
  uint32_t* s_vals = s_keys + kSortTile;
  uint32_t* s_vraw = s_vals + kSortTile;
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
  const uint32_t epoch = ep.get();
  const uint32_t wbase = base + warp * 32u * kSortItems;

  // Keys into registers (warp-striped: item j*32+lane of the warp's
  // segment); values into shared memory asynchronously, in the same order.
  uint32_t k[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    k[j] = idx < n ? keys_in[idx] : 0u;
  }
  uint32_t* vraw = s_vraw + warp * 32u * kSortItems;
  for (uint32_t c = lane; c < 8u * kSortItems; c += 32u) {
    const uint32_t first = wbase + 4u * c;
    if (first + 4u <= n) {
      cp_async16(vraw + 4u * c, vals_in + first);
    } else {
      for (uint32_t e = 0; e < 4u; ++e)
        if (first + e < n) vraw[4u * c + e] = vals_in[first + e];
    }
  }

  // Exclusive scan of the pass's global digit histogram.
  {
    const uint32_t h = tid < RADIX ? hist[tid] : 0u;
    uint32_t tot;
    const uint32_t e = block_exclusive_scan<false>(h, s_scan, &tot);
    if (tid < RADIX) s_hist_excl[tid] = e;
  }

  // Rank: position among equal digits of this warp, in index order.
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t rank[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    const bool ok = idx < n;
    const uint32_t valid = __ballot_sync(0xffffffffu, ok);
    const uint32_t d = (k[j] >> shift) & MASK;
    const uint32_t peers = match_digit<BITS>(d, valid);
    const uint32_t before = __popc(peers & lt);
    uint32_t cnt = 0;
    if (ok) cnt = s_warp_hist[warp][d];
    rank[j] = cnt + before;
    __syncwarp();
    if (ok && before == 0) s_warp_hist[warp][d] = cnt + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Per digit: exclusive offsets across warps and the block count; publish.
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
  cp_async_commit_wait();
  __syncthreads();

  // Stage keys and values in block-sorted order (block-local prefixes only),
  // so the keys and ranks leave registers before the look-back.
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    if (idx < n) {
      const uint32_t d = (k[j] >> shift) & MASK;
      const uint32_t pos = s_block_excl[d] + s_warp_hist[warp][d] + rank[j];
      s_keys[pos] = k[j];
      s_vals[pos] = vraw[(uint32_t)j * 32u + lane];
    }
  }

  // Global base of every digit: decoupled look-back over the predecessors.
  if (tid < RADIX) {
    uint32_t prefix = 0;
    if (tile > 0) {
      prefix = window_lookback<kSortWindow>(status + tid, RADIX, tile, epoch, err);
      st_release(status + (size_t)tile * RADIX + tid, pack_status(epoch, kFlagInclusive, prefix + block_count));
    }
    s_global_base[tid] = s_hist_excl[tid] + prefix;
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

constexpr size_t kSortDynSmem = 3 * kSortTile * sizeof(uint32_t);

template <int B>
void launch_bits(uint32_t grid, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                 uint32_t* vals_out, const uint32_t* n_ptr, int shift, const uint32_t* hist,
                 unsigned long long* status, uint32_t* ticket, Epoch epoch, uint32_t* err, cudaStream_t st) {
  k_onesweep<B><<<grid, kBlock, kSortDynSmem, st>>>(keys_in, vals_in, keys_out, vals_out, n_ptr, shift, hist, status,
                                                    ticket, epoch, err);
}

template <int B>
void configure_bits() {
  cudaFuncSetAttribute(k_onesweep<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSortDynSmem);
}

void prepare_sort_kernels() {
  configure_bits<1>(); configure_bits<2>(); configure_bits<3>(); configure_bits<4>();
  configure_bits<5>(); configure_bits<6>(); configure_bits<7>(); configure_bits<8>();
}

void launch_onesweep(int bits, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                     uint32_t* vals_out, const uint32_t* n_ptr, uint32_t n_max, int shift, const uint32_t* hist,
                     unsigned long long* status, uint32_t* ticket, Epoch epoch, uint32_t* err, cudaStream_t st) {
  const uint32_t grid = n_max == 0 ? 1u : (uint32_t)(((uint64_t)n_max + kSortTile - 1) / kSortTile);
#define GS_SWEEP(B)                                                                                      \
  case B:                                                                                                \
    launch_bits<B>(grid, keys_in, vals_in, keys_out, vals_out, n_ptr, shift, hist, status, ticket, epoch, \
                   err, st);                                                                             \
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
