// Front-to-back tile rasterizer body (src/renderer/pipeline/TileRasterizer.ts:414-805,
// storeFinalPixel :930-964, finalizeGaussianDepth.ts:18-68, chunk split
// rasterChunks.ts:3-99 and composite TileRasterizer.ts:807-902).
//
// One 256-thread block per 16x16 tile, one pixel per thread, lanes mapped to
// pixels in the reference's compact Morton order (rasterHelpers.ts:3-12), so
// warp w owns an 8x4 patch of the tile. Blocks take tiles from a work list
// ordered heaviest first, so long tiles start early and do not form a tail.
// Each batch of 256 sorted records is gathered into shared memory once.
// While staging, the thread that loads a record also tests the splat's
// support box against the eight warp patches and stores an 8-bit mask; each
// warp then walks only the records whose bit is set (ballot + find-first-set,
// ascending, so front-to-back order holds). The culling is conservative: a
// skipped (pixel, splat) pair is one where the per-pixel test rejects the
// splat anyway, so the result is unchanged. The block leaves the tile when no
// pixel is still accumulating (__syncthreads_or), a warp leaves a batch when
// all its pixels are done (__all_sync).
//
// Tiles holding more than `chunk` samples are evaluated as the reference's
// exact chunks: every chunk starts at transmittance 1 and its partial
// (colour, transmittance, depth) is composited in order; the block runs the
// chunks of its tile one after another and stops once the composite
// transmittance falls below the threshold, which yields exactly the composite
// of the reference's parallel chunk tasks.
//
// Arithmetic: the reference's expressions and tests in their order, with the
// deterministic exp/log (ExactMath); bit-identical to the CPU restatement when
// the translation unit is built with --fmad=false. The fast forms
// (raster_half2.cuh: FP32 and packed half2) share the helpers at the end of this
// file: the packed-record decoding and the exact ellipse-patch test.
#pragma once

#include <cuda_fp16.h>

#include "detmath.h"
#include "pass_common.cuh"

namespace gs {

constexpr float kLog2e = 1.4426950408889634f;

struct ExactMath {
  static constexpr bool kExact = true;
  static __device__ __forceinline__ float exp(float x) { return gsdm::expf_(x); }
  static __device__ __forceinline__ float log(float x) { return gsdm::logf_(x); }
};

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

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

// Frame values the rasterizer reads per sample, held in registers.
struct RasterFrame {
  float vw, vh, t_threshold;
  uint32_t axis;
};

// tileContribution.ts:66-82 gaussian_boundary_delta.
template <bool PERIODIC>
__device__ __forceinline__ void boundary_delta(float pxc, float pyc, float cx, float cy, float ca, float cb,
                                               float cc, const RasterFrame& f, float* dx, float* dy) {
  if (!PERIODIC) {
    *dx = pxc - cx;
    *dy = pyc - cy;
    return;
  }
  float ccx = cx, ccy = cy;
  if (f.axis == 1u) ccx = ccx - floorf(cx / f.vw) * f.vw;
  if (f.axis == 2u) ccy = ccy - floorf(cy / f.vh) * f.vh;
  float ddx = pxc - ccx, ddy = pyc - ccy;
  if (f.axis == 1u) {
    float opt = (-cb * ddy) / ca;
    ddx = ddx - floorf((ddx - opt) / f.vw + 0.5f) * f.vw;
  } else {
    float opt = (-cb * ddx) / cc;
    ddy = ddy - floorf((ddy - opt) / f.vh + 0.5f) * f.vh;
  }
  *dx = ddx;
  *dy = ddy;
}

struct PixelAcc {
  float r, g, b, t, d;
};

// Shared batch of the exact form (NB records: one per thread of the tile's
// block, at most 256): geo = (cx, cy, opacity, threshold), con = (a, b, c,
// depth), colour, and the warp-patch masks (bit w: warp w's 8x4 patch can be
// reached).
template <int NT>
struct Batch {
  static constexpr int NB = NT < 256 ? NT : 256;
  float4 geo[NB];
  float4 con[NB];
  float4 col[NB];
  uint32_t mask[NB];
};

constexpr float kLog2MinAlpha = -7.99435329f;  // log2(1/255)
constexpr float kLog2MaxAlpha = -0.01449957f;  // log2(0.99)

// Which of the tile's NW 8x4 warp patches can hold a pixel centre inside
// the splat's support {q(d) <= 2 threshold}. Warp w's lanes are the Morton
// indices 32 w .. 32 w + 31, so its patch starts at the Morton decode of
// 32 w. Conservative: the support's
// bounding box is widened by 5 % + 0.25 px, far beyond the rounding of the
// per-pixel evaluation for conics whose condition number is below 4e4 (the
// 0.3 px^2 filter bounds it near 3.3e4); worse-conditioned splats, periodic
// boundaries and non-finite values keep every bit set.
template <int NW>
__device__ __forceinline__ uint32_t patch_mask(float cx, float cy, float ca, float cb, float cc, float thr,
                                               float tile_x0, float tile_y0, uint32_t axis) {
  constexpr uint32_t kAll = NW >= 32 ? 0xffffffffu : (1u << NW) - 1u;
  if (axis != 0u) return kAll;
  const float det = ca * cc - cb * cb;
  const float tr = ca + cc;
  if (!(det > 0.0f) || !(tr * tr <= 4e4f * det) || !(thr >= 0.0f)) return kAll;
  const float q = 2.0f * thr;
  const float hx = sqrtf(q * cc / det) * 1.05f + 0.25f;
  const float hy = sqrtf(q * ca / det) * 1.05f + 0.25f;
  if (!(hx < 1e30f) || !(hy < 1e30f)) return kAll;
  uint32_t m = 0;
#pragma unroll
  for (uint32_t w = 0; w < (uint32_t)NW; ++w) {
    const float x0 = tile_x0 + (float)morton_compact(32u * w) + 0.5f;
    const float y0 = tile_y0 + (float)morton_compact(16u * w) + 0.5f;
    const bool hit = cx + hx >= x0 && cx - hx <= x0 + 7.0f && cy + hy >= y0 && cy - hy <= y0 + 3.0f;
    m |= hit ? (1u << w) : 0u;
  }
  return m;
}

// One (pixel, splat) step of the front-to-back blend (TileRasterizer.ts:616-707).
// Returns true when the pixel is done (transmittance below the threshold).
template <class M, bool PERIODIC, int NT>
__device__ __forceinline__ bool blend_one(const Batch<NT>& sb, uint32_t j, float pxc, float pyc, const RasterFrame& f,
                                          PixelAcc& a, uint32_t* blended) {
  const float4 g = sb.geo[j];
  const float4 c = sb.con[j];
  static_assert(M::kExact, "the fast form blends in blend_range_fast");
  float dx, dy;
  boundary_delta<PERIODIC>(pxc, pyc, g.x, g.y, c.x, c.y, c.z, f, &dx, &dy);
  const float power = ((c.x * (dx * dx) + ((c.y * 2.0f) * dx) * dy) + c.z * (dy * dy)) * -0.5f;
  if (power > 0.0f || power < -g.w) return false;
  const float alpha = rclamp(g.z * M::exp(power), 0.0f, 0.99f);
  if (alpha < (float)(1.0 / 255.0)) return false;
  const float4 col = sb.col[j];
  const float contrib = a.t * alpha;
  a.r = a.r + col.x * contrib;
  a.g = a.g + col.y * contrib;
  a.b = a.b + col.z * contrib;
  a.d = a.d + c.w * contrib;
  a.t = a.t * (1.0f - alpha);
  if (blended) ++*blended;
  return a.t < f.t_threshold;
}

struct RasterCounters {
  uint32_t checked, blended;
};

// Blend samples [s0, s1) of the tile into `a` (block-cooperative; every thread
// of the block must call it). `done` marks pixels that take no more samples.
// With STATS, `cnt` receives the reference's per-pixel counters: samples
// examined until done (TileRasterizer.ts:617) and samples blended (:702).
template <class M, bool PERIODIC, bool STATS, int NT>
__device__ __forceinline__ void blend_range(uint32_t begin, uint32_t source_count, uint32_t raster_count,
                                            uint32_t s0, uint32_t s1, bool capped, const uint32_t* __restrict__ ids,
                                            const float4* __restrict__ mean, const float4* __restrict__ conic,
                                            const float4* __restrict__ color, const RasterFrame& f, float tile_x0,
                                            float tile_y0, float pxc, float pyc, bool done, PixelAcc& a,
                                            Batch<NT>& sb, RasterCounters& cnt) {
  const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  const bool counting = STATS && !done;
  uint32_t stop = s1;  // sample index after which this pixel stopped
  constexpr uint32_t NB = (uint32_t)Batch<NT>::NB;
  for (uint32_t b = s0; b < s1; b += NB) {
    if (!__syncthreads_or(!done)) break;
    const uint32_t i = b + t;
    if (t < NB && i < s1) {
      uint32_t src = i;
      if (capped) src = (uint32_t)floorf((((float)i + 0.5f) * (float)source_count) / (float)raster_count);
      const uint32_t g = __ldg(ids + begin + src);
      const float4 m = __ldg(mean + g);
      const float4 c = __ldg(conic + g);
      const float thr = M::log(m.w * 255.0f);
      sb.geo[t] = make_float4(m.x, m.y, m.w, thr);
      sb.con[t] = make_float4(c.x, c.y, c.z, m.z);
      sb.col[t] = __ldg(color + g);
      sb.mask[t] = patch_mask<NT / 32>(m.x, m.y, c.x, c.y, c.z, thr, tile_x0, tile_y0, f.axis);
    }
    __syncthreads();
    const uint32_t n = min(NB, s1 - b);
    for (uint32_t c0 = 0; c0 < n; c0 += 32) {
      if (__all_sync(0xffffffffu, done)) break;
      const uint32_t k = c0 + lane;
      uint32_t bits = __ballot_sync(0xffffffffu, k < n && ((sb.mask[k] >> warp) & 1u));
      while (bits) {
        const uint32_t j = c0 + (uint32_t)(__ffs(bits) - 1);
        bits &= bits - 1u;
        if (!done) {
          done = blend_one<M, PERIODIC, NT>(sb, j, pxc, pyc, f, a, STATS ? &cnt.blended : nullptr);
          if (STATS && done) stop = b + j + 1;
        }
      }
    }
  }
  __syncthreads();  // shared batch buffers are free again
  if (counting) cnt.checked += stop - s0;
}

// The conic (a, b, c) back from a packed raster record's scaled terms.
__device__ __forceinline__ float4 raw_conic(const float4& r0, const float4& r1) {
  constexpr float kNeg2Ln2 = -1.38629436f;  // 1 / (-1/2 log2 e)
  constexpr float kNegLn2 = -0.693147181f;  // 1 / (-log2 e)
  return make_float4(r0.z * kNeg2Ln2, r0.w * kNegLn2, r1.x * kNeg2Ln2, 0.0f);
}

// Can a pixel centre of the rectangle [x0, x0 + wx] x [y0, y0 + wy] pass the
// splat's alpha >= 1/255 test? With F = -(a' dx^2 + b' dx dy + c' dy^2) (the
// packed record's scaled conic, F >= 0) and R = log2(255 opacity), a pixel
// passes when F(d) <= R; the minimum of the convex F over the rectangle is 0
// when the centre is inside, else it lies on an edge, where the one-variable
// minimum is clamped to the edge. The margin (1% of R + 0.01) exceeds the
// rounding of both evaluations for conics whose condition number is below
// about 1e4; worse-conditioned splats always reach the rectangle.
__device__ __forceinline__ bool patch_reach(float cx, float cy, float ap, float bp, float cp, float log2op,
                                            float x0, float y0, float wx, float wy) {
  const float A = -ap, B = -bp, C = -cp;
  const float det4 = 4.0f * A * C - B * B;  // 4 det of [[A, B/2], [B/2, C]]
  const float tr = A + C;
  const float R = log2op + 7.99435329f;
  if (!(A > 0.0f) || !(C > 0.0f) || !(det4 > 0.0f) || !(tr * tr <= 1e4f * det4)) return true;
  const float dxl = x0 - cx, dxh = dxl + wx, dyl = y0 - cy, dyh = dyl + wy;
  if (dxl <= 0.0f && dxh >= 0.0f && dyl <= 0.0f && dyh >= 0.0f) return true;
  const float ic = __fdividef(-0.5f * B, C), ia = __fdividef(-0.5f * B, A);
  float m = __int_as_float(0x7f800000);
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const float X = e ? dxh : dxl;
    const float dy = fminf(fmaxf(ic * X, dyl), dyh);
    m = fminf(m, fmaf(fmaf(C, dy, B * X), dy, A * X * X));
    const float Y = e ? dyh : dyl;
    const float dx = fminf(fmaxf(ia * Y, dxl), dxh);
    m = fminf(m, fmaf(fmaf(A, dx, B * Y), dx, C * Y * Y));
  }
  return !(m > fmaf(R, 1.01f, 0.01f));  // NaN: reach
}

__device__ __forceinline__ bool finite_r(float v) { return v == v && fabsf(v) <= 3.402823e+38f; }

// finalizeGaussianDepth.ts:18-68 with the default nodes (GaussianContextNodes.ts:127-132).
__device__ __forceinline__ float finalize_depth(float wd, float trans, const PassOptions& o, float vnear,
                                                float vfar) {
  float a = 1.0f - trans;
  float out = 0.0f;
  if (a > 0.0f) out = wd / a;
  bool scalar_valid = a > 0.0f && finite_r(wd) && finite_r(out) && out > 0.0f;
  bool valid = scalar_valid && a > o.depth_alpha_threshold;
  float dev = o.invalid_depth;
  if (valid) {
    float enc;
    if (o.depth_encoding == 0u) {
      float vz = -out;
      enc = rclamp(((vnear + vz) * vfar) / ((vfar - vnear) * vz), 0.0f, 1.0f);
    } else {
      enc = out;
    }
    if (finite_r(enc)) dev = enc;
  }
  return dev;
}

// One block of TILE x TILE threads per tile of the batch (in work-list order),
// lanes on pixels in the Morton order (warp w: an 8x4 patch); the tile's view
// supplies its viewport and targets.
template <class M, bool PERIODIC, bool STATS, int TILE>
__global__ void __launch_bounds__(TILE * TILE, TILE == 32 ? 1 : 768 / (TILE * TILE))
    k_raster(const uint32_t* __restrict__ tile_offsets,
                                                   const uint32_t* __restrict__ order,
                                                   const uint32_t* __restrict__ ids,
                                                   const float4* __restrict__ mean,
                                                   const float4* __restrict__ conic,
                                                   const float4* __restrict__ color, BatchView bv, PassOptions o,
                                                   Control* __restrict__ ctl) {
  // Overflow: the reference zeroes the raster dispatch, so nothing is written.
  if (ctl->state[3] != 0u) return;
  constexpr int NT = TILE * TILE;
  __shared__ Batch<NT> sb;
  __shared__ uint32_t s_view;
  __shared__ unsigned long long s_stats[4];
  const uint32_t tile = order ? order[blockIdx.x] : blockIdx.x;
  if (threadIdx.x == 0) s_view = find_view(bv.tile_base, bv.nviews, tile);
  if (STATS && threadIdx.x < 4) s_stats[threadIdx.x] = 0ull;
  __syncthreads();
  const ViewDesc& v = bv.views[s_view];
  const RasterFrame f = {v.vw, v.vh, o.t_threshold, o.axis};
  const uint32_t local = tile - v.tile_base;
  const uint32_t tx = local % v.tiles_x, ty = local / v.tiles_x;
  const uint32_t lx = morton_compact(threadIdx.x), ly = morton_compact(threadIdx.x >> 1);
  const uint32_t px = tx * TILE + lx, py = ty * TILE + ly;
  const uint32_t W = (uint32_t)v.vw, H = (uint32_t)v.vh;
  const bool active = px < W && py < H;
  const uint32_t begin = tile_offsets[tile], end = tile_offsets[tile + 1];
  const uint32_t source_count = end - begin;
  const bool capped = o.max_per_tile != 0u;
  const uint32_t raster_count = capped ? min(source_count, o.max_per_tile) : source_count;
  const uint32_t chunk = o.chunk;
  const bool chunked = chunk != 0u && raster_count > chunk;
  const float pxc = (float)px + 0.5f, pyc = (float)py + 0.5f;
  const float tile_x0 = (float)(tx * TILE), tile_y0 = (float)(ty * TILE);
  PixelAcc a = {0.0f, 0.0f, 0.0f, 1.0f, 0.0f};
  RasterCounters cnt = {0u, 0u};
  if (!chunked) {
    blend_range<M, PERIODIC, STATS, NT>(begin, source_count, raster_count, 0, raster_count, capped, ids, mean,
                                        conic, color, f, tile_x0, tile_y0, pxc, pyc, !active, a, sb, cnt);
  } else {
    const uint32_t nchunk = (raster_count + chunk - 1) / chunk;
    bool finished = !active;
    for (uint32_t ch = 0; ch < nchunk; ++ch) {
      if (!__syncthreads_or(!finished)) break;
      const uint32_t s0 = ch * chunk;
      const uint32_t s1 = min(s0 + chunk, raster_count);
      PixelAcc p = {0.0f, 0.0f, 0.0f, 1.0f, 0.0f};
      blend_range<M, PERIODIC, STATS, NT>(begin, source_count, raster_count, s0, s1, capped, ids, mean, conic,
                                          color, f, tile_x0, tile_y0, pxc, pyc, finished, p, sb, cnt);
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
  if (STATS) {
    // TileRasterizer.ts:749-768: checked, blended, pixels, alpha-stopped.
    if (active) {
      atomicAdd(&s_stats[0], (unsigned long long)cnt.checked);
      atomicAdd(&s_stats[1], (unsigned long long)cnt.blended);
      if (raster_count > 0) {
        atomicAdd(&s_stats[2], 1ull);
        if (a.t < f.t_threshold) atomicAdd(&s_stats[3], 1ull);
      }
    }
    __syncthreads();
    if (threadIdx.x < 4 && s_stats[threadIdx.x]) atomicAdd(&ctl->raster_stats[threadIdx.x], s_stats[threadIdx.x]);
  }
  if (!active) return;
  const float bga = rclamp(o.background[3], 0.0f, 1.0f);
  const float r = a.r + (o.background[0] * a.t) * bga;
  const float g = a.g + (o.background[1] * a.t) * bga;
  const float b = a.b + (o.background[2] * a.t) * bga;
  const float alpha = 1.0f - a.t * (1.0f - bga);
  const size_t off = (size_t)py * W + px;
  if (v.color_half) {
    __half2 lo = __floats2half2_rn(r, g);
    __half2 hi = __floats2half2_rn(b, alpha);
    uint2 w;
    w.x = *reinterpret_cast<uint32_t*>(&lo);
    w.y = *reinterpret_cast<uint32_t*>(&hi);
    reinterpret_cast<uint2*>(v.color)[off] = w;
  } else {
    reinterpret_cast<float4*>(v.color)[off] = make_float4(r, g, b, alpha);
  }
  if (v.depth) v.depth[off] = finalize_depth(a.d, a.t, o, v.vnear, v.vfar);
}

template <class M, int TILE>
void launch_raster_tile(const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* ids,
                        const float4* mean, const float4* conic, const float4* color, const BatchView& b,
                        const PassOptions& o, Control* ctl, bool stats, cudaStream_t st) {
  const bool periodic = o.axis != 0u;
#define GS_RASTER(P, S)                                                                                          \
  k_raster<M, P, S, TILE><<<b.total_tiles, TILE * TILE, 0, st>>>(tile_offsets, order, ids, mean, conic, color, b, \
                                                                  o, ctl)
  if (periodic) {
    if (stats) GS_RASTER(true, true); else GS_RASTER(true, false);
  } else {
    if (stats) GS_RASTER(false, true); else GS_RASTER(false, false);
  }
#undef GS_RASTER
}

template <class M>
void launch_raster_policy(const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* ids,
                          const float4* mean, const float4* conic, const float4* color, const BatchView& b,
                          const PassOptions& o, Control* ctl, bool stats, cudaStream_t st) {
  if (b.total_tiles == 0) return;
  if (o.tile == 8u)
    launch_raster_tile<M, 8>(tile_offsets, order, ids, mean, conic, color, b, o, ctl, stats, st);
  else if (o.tile == 32u)
    launch_raster_tile<M, 32>(tile_offsets, order, ids, mean, conic, color, b, o, ctl, stats, st);
  else
    launch_raster_tile<M, 16>(tile_offsets, order, ids, mean, conic, color, b, o, ctl, stats, st);
}

}  // namespace gs
