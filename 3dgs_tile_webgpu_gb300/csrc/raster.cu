// The fast raster forms (FP32 and packed half2) of the reference's direct tile
// rasterizer (src/renderer/pipeline/TileRasterizer.ts:414-805), built with
// multiply-add contraction, and the raster work list.
#include "raster_half2.cuh"
#include "raster_impl.cuh"

namespace gs {

// Load class of a tile: 0 when empty, else 1 + floor(log2(samples)).
__device__ __forceinline__ uint32_t load_class(uint32_t samples) { return samples == 0 ? 0u : 32u - __clz(samples); }

__global__ void __launch_bounds__(kBlock) k_order_count(const uint32_t* __restrict__ off, uint32_t ntile,
                                                        Control* __restrict__ ctl) {
  __shared__ uint32_t s_hist[34];
  if (threadIdx.x < 34) s_hist[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
  if (t < ntile) atomicAdd(&s_hist[load_class(off[t + 1] - off[t])], 1u);
  __syncthreads();
  if (threadIdx.x < 34 && s_hist[threadIdx.x]) atomicAdd(&ctl->order_hist[threadIdx.x], s_hist[threadIdx.x]);
}

// Tiles of class c go after every tile of a heavier class; within a class the
// order is whatever the atomics give (tiles are independent, so the image
// does not depend on it).
__global__ void __launch_bounds__(kBlock) k_order_scatter(const uint32_t* __restrict__ off, uint32_t ntile,
                                                          Control* __restrict__ ctl, uint32_t* __restrict__ order) {
  __shared__ uint32_t s_start[34], s_count[34], s_base[34];
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int c = 33; c >= 0; --c) {
      s_start[c] = run;
      run += ctl->order_hist[c];
    }
  }
  if (threadIdx.x < 34) s_count[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
  uint32_t c = 0, local = 0;
  if (t < ntile) {
    c = load_class(off[t + 1] - off[t]);
    local = atomicAdd(&s_count[c], 1u);
  }
  __syncthreads();
  if (threadIdx.x < 34 && s_count[threadIdx.x])
    s_base[threadIdx.x] = atomicAdd(&ctl->order_fill[threadIdx.x], s_count[threadIdx.x]);
  __syncthreads();
  if (t < ntile) order[s_start[c] + s_base[c] + local] = t;
}

void launch_tile_order(const uint32_t* tile_offsets, uint32_t ntile, Control* ctl, uint32_t* order, int sms,
                       cudaStream_t st) {
  (void)sms;
  if (ntile == 0) return;
  const uint32_t grid = (ntile + kBlock - 1) / kBlock;
  k_order_count<<<grid, kBlock, 0, st>>>(tile_offsets, ntile, ctl);
  k_order_scatter<<<grid, kBlock, 0, st>>>(tile_offsets, ntile, ctl, order);
}

void launch_raster(int precision, const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* ids,
                   const float4* mean, const float4* conic, const float4* color, const float4* rec,
                   const BatchView& b, const PassOptions& o, Control* ctl, bool stats, cudaStream_t st) {
  if (precision == 1) {
    launch_raster_exact(tile_offsets, order, ids, mean, conic, color, b, o, ctl, stats, st);
    return;
  }
  if (precision == 2) {
    launch_raster_pairs(true, tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
    return;
  }
  launch_raster_pairs(false, tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
}

}  // namespace gs
