// FP32 rasterizer with hardware exp/log and multiply-add contraction: the
// production form of the reference's direct tile rasterizer
// (src/renderer/pipeline/TileRasterizer.ts:414-805).
#include "raster_impl.cuh"

namespace gs {

void launch_raster(int precision, const uint32_t* tile_offsets, const uint32_t* ids, const float4* mean,
                   const float4* conic, const float4* color, const FrameView& f, const Control* ctl,
                   void* color_out, int color_half, float* depth_out, cudaStream_t st) {
  if (precision == 1) {
    launch_raster_exact(tile_offsets, ids, mean, conic, color, f, ctl, color_out, color_half, depth_out, st);
    return;
  }
  const uint32_t grid = f.tiles_x * f.tiles_y;
  if (color_half)
    k_raster<FastMath, true><<<grid, kBlock, 0, st>>>(tile_offsets, ids, mean, conic, color, f, ctl, color_out,
                                                      depth_out);
  else
    k_raster<FastMath, false><<<grid, kBlock, 0, st>>>(tile_offsets, ids, mean, conic, color, f, ctl, color_out,
                                                       depth_out);
}

}  // namespace gs
