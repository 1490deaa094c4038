// Front-to-back tile rasterizer body (src/renderer/pipeline/TileRasterizer.ts:414-805,
// storeFinalPixel :930-964, finalizeGaussianDepth.ts:18-68, chunk split
// rasterChunks.ts:3-99 and composite TileRasterizer.ts:807-902).
//
// One 256-thread block per 16x16 tile, one pixel per thread (lane -> pixel in
// the reference's compact Morton order, rasterHelpers.ts:3-12, so a warp
// covers an 8x4 patch). Each batch of 256 sorted records is gathered into
// shared memory once and read by every pixel; the block leaves the tile as
// soon as no pixel is still accumulating (__syncthreads_or).
//
// Tiles holding more than `chunk` samples are evaluated as the reference's
// exact chunks: every chunk starts at transmittance 1 and its partial
// (colour, transmittance, depth) is composited in order. The block runs the
// chunks of its tile one after another and stops compositing once the
// composite transmittance falls below the threshold, which yields exactly the
// composite the reference's parallel chunk tasks produce.
//
// The MATH policy supplies exp/log: deterministic (bit-identical to the CPU
// restatement when the translation unit is built with --fmad=false) or the
// hardware fast path.
#pragma once

#include <cuda_fp16.h>

#include "detmath.h"
#include "pass_common.cuh"

namespace gs {

struct ExactMath {
  static __device__ __forceinline__ float exp(float x) { return gsdm::expf_(x); }
  static __device__ __forceinline__ float log(float x) { return gsdm::logf_(x); }
};
struct FastMath {
  static __device__ __forceinline__ float exp(float x) { return __expf(x); }
  static __device__ __forceinline__ float log(float x) { return __logf(x); }
};

__device__ __forceinline__ uint32_t morton_compact(uint32_t v) {
  uint32_t r = v & 0x55555555u;
  r = (r | (r >> 1)) & 0x33333333u;
  r = (r | (r >> 2)) & 0x0f0f0f0fu;
  r = (r | (r >> 4)) & 0x00ff00ffu;
  r = (r | (r >> 8)) & 0x0000ffffu;
  return r;
}

__device__ __forceinline__ float rclamp(float x, float lo, float hi) {
  float y = x < lo ? lo : x;
  return y > hi ? hi : y;
}

// tileContribution.ts:66-82 gaussian_boundary_delta.
__device__ __forceinline__ void boundary_delta(float pxc, float pyc, float4 m, float4 c, const FrameView& f,
                                               float* dx, float* dy) {
  if (f.axis == 0u) {
    *dx = pxc - m.x;
    *dy = pyc - m.y;
    return;
  }
  float ccx = m.x, ccy = m.y;
  if (f.axis == 1u) ccx = ccx - floorf(m.x / f.vw) * f.vw;
  if (f.axis == 2u) ccy = ccy - floorf(m.y / f.vh) * f.vh;
  float ddx = pxc - ccx, ddy = pyc - ccy;
  if (f.axis == 1u) {
    float opt = (-c.y * ddy) / c.x;
    ddx = ddx - floorf((ddx - opt) / f.vw + 0.5f) * f.vw;
  } else {
    float opt = (-c.y * ddx) / c.z;
    ddy = ddy - floorf((ddy - opt) / f.vh + 0.5f) * f.vh;
  }
  *dx = ddx;
  *dy = ddy;
}

struct PixelAcc {
  float r, g, b, t, d;
};

// Blend samples [s0, s1) of the tile into `a` (block-cooperative; every thread
// of the block must call it). `done` marks pixels that take no more samples.
template <class M>
__device__ __forceinline__ void blend_range(uint32_t begin, uint32_t source_count, uint32_t raster_count,
                                            uint32_t s0, uint32_t s1, bool capped, const uint32_t* __restrict__ ids,
                                            const float4* __restrict__ mean, const float4* __restrict__ conic,
                                            const float4* __restrict__ color, const FrameView& f, float pxc,
                                            float pyc, bool done, PixelAcc& a, float4* s_mean, float4* s_conic,
                                            float4* s_color) {
  const uint32_t t = threadIdx.x;
  for (uint32_t b = s0; b < s1; b += kBlock) {
    if (!__syncthreads_or(!done)) break;
    uint32_t i = b + t;
    if (i < s1) {
      uint32_t src = i;
      if (capped) src = (uint32_t)floorf((((float)i + 0.5f) * (float)source_count) / (float)raster_count);
      uint32_t g = __ldg(ids + begin + src);
      float4 m = __ldg(mean + g);
      float4 c = __ldg(conic + g);
      s_mean[t] = m;
      s_conic[t] = make_float4(c.x, c.y, c.z, M::log(m.w * 255.0f));
      s_color[t] = __ldg(color + g);
    }
    __syncthreads();
    if (!done) {
      uint32_t n = min((uint32_t)kBlock, s1 - b);
      for (uint32_t j = 0; j < n; ++j) {
        float4 m = s_mean[j];
        float4 c = s_conic[j];
        float dx, dy;
        boundary_delta(pxc, pyc, m, c, f, &dx, &dy);
        float power = ((c.x * (dx * dx) + ((c.y * 2.0f) * dx) * dy) + c.z * (dy * dy)) * -0.5f;
        if (power > 0.0f || power < -c.w) continue;
        float alpha = rclamp(m.w * M::exp(power), 0.0f, 0.99f);
        if (alpha < (float)(1.0 / 255.0)) continue;
        float4 col = s_color[j];
        float contrib = a.t * alpha;
        a.r = a.r + col.x * contrib;
        a.g = a.g + col.y * contrib;
        a.b = a.b + col.z * contrib;
        a.d = a.d + m.z * contrib;
        a.t = a.t * (1.0f - alpha);
        if (a.t < f.t_threshold) {
          done = true;
          break;
        }
      }
    }
  }
  __syncthreads();  // shared batch buffers are free again
}

__device__ __forceinline__ bool finite_r(float v) { return v == v && fabsf(v) <= 3.402823e+38f; }

// finalizeGaussianDepth.ts:18-68 with the default nodes (GaussianContextNodes.ts:127-132).
__device__ __forceinline__ float finalize_depth(float wd, float trans, const FrameView& f) {
  float a = 1.0f - trans;
  float out = 0.0f;
  if (a > 0.0f) out = wd / a;
  bool scalar_valid = a > 0.0f && finite_r(wd) && finite_r(out) && out > 0.0f;
  bool valid = scalar_valid && a > f.depth_alpha_threshold;
  float dev = f.invalid_depth;
  if (valid) {
    float enc;
    if (f.depth_encoding == 0u) {
      float vz = -out;
      enc = rclamp(((f.vnear + vz) * f.vfar) / ((f.vfar - f.vnear) * vz), 0.0f, 1.0f);
    } else {
      enc = out;
    }
    if (finite_r(enc)) dev = enc;
  }
  return dev;
}

template <class M, bool HALF_OUT>
__global__ void __launch_bounds__(kBlock) k_raster(const uint32_t* __restrict__ tile_offsets,
                                                   const uint32_t* __restrict__ ids,
                                                   const float4* __restrict__ mean,
                                                   const float4* __restrict__ conic,
                                                   const float4* __restrict__ color, FrameView f,
                                                   const Control* __restrict__ ctl, void* __restrict__ out,
                                                   float* __restrict__ depth_out) {
  // Overflow: the reference zeroes the raster dispatch, so nothing is written.
  if (ctl->state[3] != 0u) return;
  __shared__ float4 s_mean[kBlock];
  __shared__ float4 s_conic[kBlock];
  __shared__ float4 s_color[kBlock];
  const uint32_t tile = blockIdx.x;
  const uint32_t tx = tile % f.tiles_x, ty = tile / f.tiles_x;
  const uint32_t lx = morton_compact(threadIdx.x), ly = morton_compact(threadIdx.x >> 1);
  const uint32_t px = tx * kTileSize + lx, py = ty * kTileSize + ly;
  const uint32_t W = (uint32_t)f.vw, H = (uint32_t)f.vh;
  const bool active = px < W && py < H;
  const uint32_t begin = tile_offsets[tile], end = tile_offsets[tile + 1];
  const uint32_t source_count = end - begin;
  const bool capped = f.max_per_tile != 0u;
  const uint32_t raster_count = capped ? min(source_count, f.max_per_tile) : source_count;
  const bool chunked = f.chunk != 0u && raster_count > f.chunk;
  const float pxc = (float)px + 0.5f, pyc = (float)py + 0.5f;
  PixelAcc a = {0.0f, 0.0f, 0.0f, 1.0f, 0.0f};
  if (!chunked) {
    blend_range<M>(begin, source_count, raster_count, 0, raster_count, capped, ids, mean, conic, color, f, pxc,
                   pyc, !active, a, s_mean, s_conic, s_color);
  } else {
    const uint32_t nchunk = (raster_count + f.chunk - 1) / f.chunk;
    bool finished = !active;
    for (uint32_t ch = 0; ch < nchunk; ++ch) {
      if (!__syncthreads_or(!finished)) break;
      const uint32_t s0 = ch * f.chunk;
      const uint32_t s1 = min(s0 + f.chunk, raster_count);
      PixelAcc p = {0.0f, 0.0f, 0.0f, 1.0f, 0.0f};
      blend_range<M>(begin, source_count, raster_count, s0, s1, capped, ids, mean, conic, color, f, pxc, pyc,
                     finished, p, s_mean, s_conic, s_color);
      if (!finished) {
        a.r = a.r + p.r * a.t;
        a.g = a.g + p.g * a.t;
        a.b = a.b + p.b * a.t;
        a.d = a.d + p.d * a.t;
        a.t = a.t * p.t;
        if (a.t < f.t_threshold) finished = true;
      }
    }
  }
  if (!active) return;
  const float bga = rclamp(f.background[3], 0.0f, 1.0f);
  float r = a.r + (f.background[0] * a.t) * bga;
  float g = a.g + (f.background[1] * a.t) * bga;
  float b = a.b + (f.background[2] * a.t) * bga;
  float alpha = 1.0f - a.t * (1.0f - bga);
  const size_t o = (size_t)py * W + px;
  if (HALF_OUT) {
    __half2 lo = __floats2half2_rn(r, g);
    __half2 hi = __floats2half2_rn(b, alpha);
    uint2 w;
    w.x = *reinterpret_cast<uint32_t*>(&lo);
    w.y = *reinterpret_cast<uint32_t*>(&hi);
    reinterpret_cast<uint2*>(out)[o] = w;
  } else {
    reinterpret_cast<float4*>(out)[o] = make_float4(r, g, b, alpha);
  }
  if (depth_out) depth_out[o] = finalize_depth(a.d, a.t, f);
}

}  // namespace gs
