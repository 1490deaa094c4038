// FP32 rasterizer with hardware exp/log and multiply-add contraction: the
// production form of the reference's direct tile rasterizer
// (src/renderer/pipeline/TileRasterizer.ts:414-805).
#include "raster_impl.cuh"

namespace gs {

void launch_raster(int precision, const uint32_t* tile_offsets, const uint32_t* ids, const float4* mean,
                   const float4* conic, const float4* color, const BatchView& b, const PassOptions& o,
                   const Control* ctl, cudaStream_t st) {
  if (precision == 1) {
    launch_raster_exact(tile_offsets, ids, mean, conic, color, b, o, ctl, st);
    return;
  }
  if (b.total_tiles == 0) return;
  k_raster<FastMath><<<b.total_tiles, kBlock, 0, st>>>(tile_offsets, ids, mean, conic, color, b, o, ctl);
}

}  // namespace gs
