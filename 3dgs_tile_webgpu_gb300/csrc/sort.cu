// Stable LSD radix sort pass over (uint32 key, uint32 value).
//
// Replaces the reference's 4-bit, 5-dispatch-per-pass radix sort
// (src/renderer/kernels/radix.ts:10-263, src/renderer/pipeline/RadixSorter.ts:50-322),
// which is a stable LSD sort; stability is the property the pass depends on
// (records enter in ordinal order for the depth sort and in depth-rank order
// for the tile sort, TiledGaussianPipeline.ts:144,442-446).
//
// One pass = reduce, scan, scatter with no look-back chain (a single-kernel
// decoupled look-back pass settles only a window of tiles per L2 round trip,
// which bounds it far below HBM speed on passes of tens of millions of keys).
// The items split into `chunks` contiguous runs of whole 4096-item tiles (one
// split, derived from the device-side count, shared by the three kernels):
//   k_chunk_count   keys of every (chunk, digit), by shared-memory atomics,
//                   also summed into the pass's global digit histogram;
//   k_chunk_offsets per digit, the exclusive prefix over chunks plus the
//                   digit's global base from that histogram;
//   k_chunk_scatter one block per chunk walks its tiles in order with running
//                   per-digit offsets: tile t+1 streams into shared memory by
//                   two bulk copies (cp.async.bulk, 16 KB of keys and 16 KB
//                   of values, completion counted on an mbarrier) while tile
//                   t is ranked per digit within each warp by ballot
//                   bit-splitting (warp-striped layout: item j*32+lane of
//                   each warp's 512-item segment, so ranks follow index
//                   order), staged in place in block-sorted order, and
//                   written out with each digit's run contiguous.
// Stable: tiles in index order within a chunk, chunks in index order, ranks in
// index order within a tile.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "pass_common.cuh"

namespace gs {

constexpr int kSortWarps = 8;
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

// Tiles [t0, t1) of chunk c when n items split over `chunks` chunks.
__device__ __forceinline__ void chunk_tiles(uint32_t n, uint32_t chunks, uint32_t c, uint32_t* t0, uint32_t* t1) {
  const uint32_t tiles = (uint32_t)(((uint64_t)n + kSortTile - 1) / kSortTile);
  const uint32_t per = (tiles + chunks - 1) / chunks;
  *t0 = min(c * per, tiles);
  *t1 = min(*t0 + per, tiles);
}

template <int BITS>
__global__ void __launch_bounds__(kBlock) k_chunk_count(const uint32_t* __restrict__ keys,
                                                        const uint32_t* __restrict__ n_ptr, int shift,
                                                        uint32_t chunks, uint32_t* __restrict__ counts,
                                                        uint32_t* __restrict__ hist) {
  constexpr uint32_t RADIX = 1u << BITS;
  constexpr uint32_t MASK = RADIX - 1u;
  __shared__ uint32_t s_hist[kSortWarps][RADIX];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  for (uint32_t i = tid; i < kSortWarps * RADIX; i += kBlock) (&s_hist[0][0])[i] = 0u;
  __syncthreads();
  const uint32_t n = *n_ptr;
  uint32_t t0, t1;
  chunk_tiles(n, chunks, blockIdx.x, &t0, &t1);
  const uint32_t begin = (uint32_t)min((uint64_t)t0 * kSortTile, (uint64_t)n);
  const uint32_t end = (uint32_t)min((uint64_t)t1 * kSortTile, (uint64_t)n);
  // Each warp takes 512-key runs: four 16-byte loads per lane in flight
  // before any counting (begin is a multiple of 4096, so they are aligned).
  constexpr uint32_t kRun = 512u;
  for (uint32_t s = begin + warp * kRun; s < end; s += kSortWarps * kRun) {
    uint32_t kk[16];
#pragma unroll
    for (uint32_t q = 0; q < 4u; ++q) {
      const uint32_t i0 = s + q * 128u + 4u * lane;
      if (i0 + 4u <= end) {
        const uint4 v = *reinterpret_cast<const uint4*>(keys + i0);
        kk[4 * q] = v.x; kk[4 * q + 1] = v.y; kk[4 * q + 2] = v.z; kk[4 * q + 3] = v.w;
      } else {
#pragma unroll
        for (uint32_t e = 0; e < 4u; ++e) kk[4 * q + e] = i0 + e < end ? keys[i0 + e] : 0u;
      }
    }
#pragma unroll
    for (uint32_t q = 0; q < 16u; ++q) {
      const bool ok = s + (q >> 2) * 128u + 4u * lane + (q & 3u) < end;
      const uint32_t d = (kk[q] >> shift) & MASK;
      const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
      if (__all_sync(0xffffffffu, ok && d == d0)) {
        if (lane == 0u) atomicAdd(&s_hist[warp][d0], 32u);
      } else if (ok) {
        atomicAdd(&s_hist[warp][d], 1u);
      }
    }
  }
  __syncthreads();
  for (uint32_t d = tid; d < RADIX; d += kBlock) {
    uint32_t sum = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) sum += s_hist[w][d];
    counts[(size_t)blockIdx.x * RADIX + d] = sum;
    if (sum) atomicAdd(hist + d, sum);
  }
}

// One block per digit; counts[c][d] becomes the global position of the first
// key of digit d in chunk c.
template <int BITS>
__global__ void __launch_bounds__(kBlock) k_chunk_offsets(const uint32_t* __restrict__ hist, uint32_t chunks,
                                                          uint32_t* __restrict__ counts) {
  constexpr uint32_t RADIX = 1u << BITS;
  __shared__ uint32_t s_scan[kBlock / 32];
  const uint32_t tid = threadIdx.x, d = blockIdx.x;
  uint32_t base;
  block_exclusive_scan<false>(tid < d ? hist[tid] : 0u, s_scan, &base);  // keys of the digits below d
  const uint32_t per = (chunks + kBlock - 1) / kBlock;
  const uint32_t c0 = min(tid * per, chunks), c1 = min(c0 + per, chunks);
  uint32_t local = 0;
  for (uint32_t c = c0; c < c1; ++c) local += counts[(size_t)c * RADIX + d];
  uint32_t total;
  uint32_t run = base + block_exclusive_scan<false>(local, s_scan, &total);
  for (uint32_t c = c0; c < c1; ++c) {
    const uint32_t v = counts[(size_t)c * RADIX + d];
    counts[(size_t)c * RADIX + d] = run;
    run += v;
  }
}

// Two tile buffers (keys and values each): tile t+1 streams in while tile t
// is ranked and scattered.
constexpr size_t kChunkDynSmem = 2 * 2 * kSortTile * sizeof(uint32_t);

template <int BITS>
struct ScatterShared {
  uint32_t warp_hist[kSortWarps][1u << BITS];
  uint32_t block_excl[1u << BITS];
  uint32_t run[1u << BITS];  // global position of the next key of each digit
  uint32_t scan[kBlock / 32];
  unsigned long long bar[2];  // bulk-copy completion of each tile buffer
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Bulk copies of one tile's keys and values (items base .. min(base + 4096,
// n)) into kb/vb, issued by thread 0 and counted on the buffer's mbarrier;
// the last n % 4 items of a ragged tile (a bulk copy moves whole 16-byte
// units) come by plain loads, visible after the next block barrier.
__device__ __forceinline__ void load_tile_bulk(const uint32_t* __restrict__ keys_in,
                                               const uint32_t* __restrict__ vals_in, uint32_t base, uint32_t n,
                                               uint32_t* kb, uint32_t* vb, uint32_t bar) {
  const uint32_t items = min(kSortTile, n - base);
  const uint32_t whole = items & ~3u;  // items moved by the bulk copies
  if (threadIdx.x == 0) {
    const uint32_t bytes = whole * 4u;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(2u * bytes) : "memory");
    if (bytes) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the buffer's previous reads come first
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_addr(kb)),
                   "l"(keys_in + base), "r"(bytes), "r"(bar)
                   : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_addr(vb)),
                   "l"(vals_in + base), "r"(bytes), "r"(bar)
                   : "memory");
    }
  }
  for (uint32_t e = whole + threadIdx.x; e < items; e += kBlock) {
    kb[e] = keys_in[base + e];
    vb[e] = vals_in[base + e];
  }
}

// Bounded wait for phase `parity` of the mbarrier (about a second of polls).
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
  uint32_t backoff = 16;
  for (uint32_t polls = 0; polls < kSpinLimit; ++polls) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    __nanosleep(backoff);
    backoff = backoff < 256 ? backoff * 2 : 256;
  }
  return false;
}

// Ranks the tile held in kb/vb (items base .. base + 4096, those below n),
// stages it in place in block-sorted order and writes each digit's run to its
// global position. FULL: every item of the tile is below n. Leaves warp_hist
// zeroed and run advanced past the tile.
template <int BITS, bool FULL>
__device__ __forceinline__ void scatter_tile(ScatterShared<BITS>& sm, uint32_t* kb, uint32_t* vb, uint32_t base,
                                             uint32_t n, int shift, uint32_t* __restrict__ keys_out,
                                             uint32_t* __restrict__ vals_out) {
  constexpr uint32_t RADIX = 1u << BITS;
  constexpr uint32_t MASK = RADIX - 1u;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t wofs = warp * 32u * kSortItems;  // warp-striped: item j*32+lane of the warp's segment
  uint32_t k[kSortItems], rank[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) k[j] = kb[wofs + (uint32_t)j * 32u + lane];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const bool ok = FULL || base + wofs + (uint32_t)j * 32u + lane < n;
    const uint32_t valid = FULL ? 0xffffffffu : __ballot_sync(0xffffffffu, ok);
    const uint32_t d = (k[j] >> shift) & MASK;
    const uint32_t peers = match_digit<BITS>(d, valid);
    const uint32_t before = __popc(peers & lt);
    uint32_t cnt = 0;
    if (ok) cnt = sm.warp_hist[warp][d];
    rank[j] = cnt + before;
    __syncwarp();
    if (ok && before == 0) sm.warp_hist[warp][d] = cnt + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  uint32_t block_count = 0;
  if (tid < RADIX) {
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = sm.warp_hist[w][tid];
      sm.warp_hist[w][tid] = block_count;
      block_count += c;
    }
  }
  {
    uint32_t tot;
    const uint32_t e = block_exclusive_scan<false>(tid < RADIX ? block_count : 0u, sm.scan, &tot);
    if (tid < RADIX) sm.block_excl[tid] = e;
  }
  __syncthreads();

  // Keys first (every raw key is already in registers), then the values
  // (read raw into registers, then written once every thread has read).
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    if (FULL || base + wofs + (uint32_t)j * 32u + lane < n) {
      const uint32_t d = (k[j] >> shift) & MASK;
      rank[j] += sm.block_excl[d] + sm.warp_hist[warp][d];
      kb[rank[j]] = k[j];
    }
  }
  uint32_t v[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) v[j] = vb[wofs + (uint32_t)j * 32u + lane];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kSortItems; ++j)
    if (FULL || base + wofs + (uint32_t)j * 32u + lane < n) vb[rank[j]] = v[j];
  __syncthreads();

  const uint32_t count = FULL ? kSortTile : min(kSortTile, n - base);
#pragma unroll 4
  for (uint32_t i = tid; i < count; i += kBlock) {
    const uint32_t key = kb[i];
    const uint32_t dig = (key >> shift) & MASK;
    const uint32_t dst = sm.run[dig] + (i - sm.block_excl[dig]);
    keys_out[dst] = key;
    vals_out[dst] = vb[i];
  }
  for (uint32_t i = tid; i < kSortWarps * RADIX; i += kBlock) (&sm.warp_hist[0][0])[i] = 0u;
  __syncthreads();
  if (tid < RADIX) sm.run[tid] += block_count;
}

template <int BITS>
__global__ void __launch_bounds__(kBlock, kChunkBlocksPerSm)
    k_chunk_scatter(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                    const uint32_t* __restrict__ n_ptr, int shift, uint32_t chunks,
                    const uint32_t* __restrict__ offsets, uint32_t* __restrict__ err) {
  constexpr uint32_t RADIX = 1u << BITS;
  __shared__ ScatterShared<BITS> sm;
  extern __shared__ uint4 s_dyn[];
  uint32_t* s_buf = reinterpret_cast<uint32_t*>(s_dyn);

  const uint32_t tid = threadIdx.x;
  const uint32_t n = *n_ptr;
  uint32_t t0, t1;
  chunk_tiles(n, chunks, blockIdx.x, &t0, &t1);
  if (t0 >= t1) return;
  if (tid < 2u) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&sm.bar[tid])) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();
  uint32_t phases = 0;  // parity of the next phase of each buffer's barrier
  load_tile_bulk(keys_in, vals_in, t0 * kSortTile, n, s_buf, s_buf + kSortTile, smem_addr(&sm.bar[0]));
  if (tid < RADIX) sm.run[tid] = offsets[(size_t)blockIdx.x * RADIX + tid];
  for (uint32_t i = tid; i < kSortWarps * RADIX; i += kBlock) (&sm.warp_hist[0][0])[i] = 0u;

  for (uint32_t t = t0; t < t1; ++t) {
    const uint32_t k = (t - t0) & 1u;
    uint32_t* kb = s_buf + k * 2u * kSortTile;
    uint32_t* vb = kb + kSortTile;
    if (t + 1u < t1) {
      uint32_t* nb = s_buf + (k ^ 1u) * 2u * kSortTile;
      load_tile_bulk(keys_in, vals_in, (t + 1u) * kSortTile, n, nb, nb + kSortTile, smem_addr(&sm.bar[k ^ 1u]));
    }
    const bool landed = bar_wait(smem_addr(&sm.bar[k]), (phases >> k) & 1u);
    phases ^= 1u << k;
    if (!__syncthreads_and(landed)) {
      // A copy never landed: flag the frame and leave, after the other
      // buffer's copy (if one was issued) had its own bounded wait.
      if (tid == 0) atomicOr(err, 4u);
      if (t + 1u < t1) bar_wait(smem_addr(&sm.bar[k ^ 1u]), (phases >> (k ^ 1u)) & 1u);
      return;
    }
    const uint32_t base = t * kSortTile;
    if ((uint64_t)base + kSortTile <= n)
      scatter_tile<BITS, true>(sm, kb, vb, base, n, shift, keys_out, vals_out);
    else
      scatter_tile<BITS, false>(sm, kb, vb, base, n, shift, keys_out, vals_out);
  }
}

template <int B>
void launch_chunk_bits(uint32_t chunks, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                       uint32_t* vals_out, const uint32_t* n_ptr, int shift, uint32_t* hist, uint32_t* counts,
                       uint32_t* err, cudaStream_t st) {
  k_chunk_count<B><<<chunks, kBlock, 0, st>>>(keys_in, n_ptr, shift, chunks, counts, hist);
  k_chunk_offsets<B><<<1u << B, kBlock, 0, st>>>(hist, chunks, counts);
  k_chunk_scatter<B><<<chunks, kBlock, kChunkDynSmem, st>>>(keys_in, vals_in, keys_out, vals_out, n_ptr, shift,
                                                           chunks, counts, err);
}

template <int B>
void configure_bits() {
  cudaFuncSetAttribute(k_chunk_scatter<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kChunkDynSmem);
}

void prepare_sort_kernels() {
  configure_bits<1>(); configure_bits<2>(); configure_bits<3>(); configure_bits<4>();
  configure_bits<5>(); configure_bits<6>(); configure_bits<7>(); configure_bits<8>();
}

uint32_t chunk_pass_chunks(uint32_t n_max, int sms) {
  const uint64_t tiles = ((uint64_t)n_max + kSortTile - 1) / kSortTile;
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)kChunkBlocksPerSm * (uint64_t)sms));
}

void launch_chunk_pass(int bits, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                       uint32_t* vals_out, const uint32_t* n_ptr, int shift, uint32_t* hist, uint32_t chunks,
                       uint32_t* counts, uint32_t* err, cudaStream_t st) {
#define GS_CHUNK(B)                                                                                             \
  case B:                                                                                                       \
    launch_chunk_bits<B>(chunks, keys_in, vals_in, keys_out, vals_out, n_ptr, shift, hist, counts, err, st);    \
    break;
  switch (bits) {
    GS_CHUNK(1)
    GS_CHUNK(2)
    GS_CHUNK(3)
    GS_CHUNK(4)
    GS_CHUNK(5)
    GS_CHUNK(6)
    GS_CHUNK(7)
    default:
      GS_CHUNK(8)
  }
#undef GS_CHUNK
}

}  // namespace gs
