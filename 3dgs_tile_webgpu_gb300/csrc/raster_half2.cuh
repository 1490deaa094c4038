// The fast forms of the tile rasterizer (the reference's direct rasterizer,
// src/renderer/pipeline/TileRasterizer.ts:414-805, with the same chunk, cap,
// boundary, background and depth semantics as raster_impl.cuh): FP32 and
// packed half2, one kernel template (HALF) over the same pixel-pair layout.
//
// One warp per 8x8 patch of the tile: 128 threads per 16x16 tile (32 per 8x8,
// 512 per 32x32 tile in batches tuned to those tile sizes); each thread owns
// two pixels of one column, (x, y) and (x, y + 4), so warp w owns the 8x8
// patch at (8 (w mod P), 8 (w div P)), P = tile / 8. The two pixels share dx
// and the x-only terms of the quadratic, the record loads, the culling test
// and the loop.
//
// The warps of a tile work independently (no block barrier while
// blending): each warp walks the tile's sorted records 32 at a time, every
// lane gathers one packed 32-byte record (pass_common.cuh), tests whether the
// splat's support can reach the warp's 8x8 patch (the exact minimum of the
// quadratic over the patch's pixel-centre rectangle, with a margin), and the
// records that can are compacted, in order, into the warp's shared staging
// area. A warp leaves the tile as soon as its 64 pixels are done.
//
// Per record the projection folded the opacity into the exponent:
//   p' = log2(opacity) - (a dx^2 + 2 b dx dy + c dy^2) / 2 * log2(e)
// so alpha = min(opacity e^power, 0.99) = 2^min(p', L), L = min(log2 opacity,
// log2 0.99), and the reference's alpha >= 1/255 test is p' >= log2(1/255).
// Per record and pixel pair:
//   half2 form: p'0 and p'1 in packed half2 from the record's Cholesky
//               factor (cholesky_record below: five HFMA2), the threshold
//               compare, min(p', log2 0.99) and exp2 in packed half2 too
//               (ex2.approx.f16x2), colour from the record's f16 values;
//               the periodic-boundary variant evaluates p' in FP32
//   FP32 form:  dx, dy0, dy1, p'0, p'1, the compares, min(p', L) and exp2
//               per pixel (ex2.approx.f32), FP32 colour
//   both:       FP32 transmittance and colour/depth accumulation
// A pixel's transmittance is tested against the threshold once per group of
// 32 records; a pixel found done stops blending from there on (its threshold
// becomes +inf), so it may blend up to 31 records more than the reference,
// whose contributions sum to less than the threshold.
#pragma once

#include <cuda_fp16.h>

#include "raster_impl.cuh"

namespace gs {


__device__ __forceinline__ __half2 h2ex2_approx(__half2 x) {
  uint32_t in = *reinterpret_cast<uint32_t*>(&x), out;
  asm("ex2.approx.f16x2 %0, %1;" : "=r"(out) : "r"(in));
  return *reinterpret_cast<__half2*>(&out);
}

__device__ __forceinline__ __half2 u2h2(uint32_t u) { return *reinterpret_cast<const __half2*>(&u); }
__device__ __forceinline__ uint32_t h22u(__half2 h) { return *reinterpret_cast<const uint32_t*>(&h); }

// The half2 form's per-pixel evaluation. With M = [[a, b], [b, c]] log2(e)/2
// (the record's conic, positive definite) and its Cholesky factor
// M = L L^T, L = [[l11, 0], [l21, l22]], the exponent of a pixel at offset
// d from the splat centre is
//   p' = log2(opacity) - d^T M d = log2(opacity) - w1^2 - w2^2,
//   w1 = l11 dx + l21 dy,  w2 = l22 dy.
// Per record and warp patch the FP32 staging step evaluates w at the
// patch centre e (offset d_e); a pixel at e + u then has
//   w1 = w1(e) + l11 ux + l21 uy,  w2 = w2(e) + l22 uy
// with |ux|, |uy| <= 3.5 (exact in f16), so the per-pixel work is five
// packed half2 FMAs for two pixels. In this form no intermediate cancels:
// |w| stays near the square root of the exponent, where the expanded
// quadratic (a dx^2 + 2 b dx dy + c dy^2) would round its large, opposite
// terms for a long, tilted splat. And p' <= log2(opacity) after rounding too
// (subtracting squares), so alpha = 2^min(p', log2 0.99) needs no per-record
// limit.
// Words: (l11, l21), (w1(e), w2(e)), (l22, log2 opacity), unused. The factor
// is stored in f16, so approximate reciprocal square roots (2 ulp in FP32)
// suffice. A degenerate record (m00 or the Schur complement not positive,
// which a valid projection does not produce) gets a tiny floor instead; its
// exponent may then overflow to -inf or NaN, and either blends nothing.
__device__ __forceinline__ uint4 cholesky_record(const float4& r0, const float4& r1, float ex, float ey) {
  const float m00 = fmaxf(-r0.z, 1e-30f), m01 = -0.5f * r0.w, m11 = -r1.x;
  const float r = rsqrtf(m00);
  const float l11 = m00 * r, l21 = m01 * r;
  const float s = fmaxf(fmaf(-l21, l21, m11), 1e-30f);
  const float l22 = s * rsqrtf(s);
  const float dx = ex - r0.x, dy = ey - r0.y;
  const float w1 = fmaf(l11, dx, l21 * dy), w2 = l22 * dy;
  return make_uint4(h22u(__floats2half2_rn(l11, l21)), h22u(__floats2half2_rn(w1, w2)),
                    h22u(__floats2half2_rn(l22, r1.y)), 0u);
}

// Alpha of the lane's two pixels from the Cholesky record: 2^min(p', L) where
// p' >= the pixel's threshold (log2(1/255), or +inf once the pixel is done),
// else +0 (a NaN exponent fails the compare and blends +0 too).
__device__ __forceinline__ float2 cholesky_alpha(const uint4& h, __half2 ux, __half2 uy, __half2 th,
                                                 uint32_t* use_mask) {
  const __half2 h0 = u2h2(h.x), h1 = u2h2(h.y), h2 = u2h2(h.z);
  const __half2 t = __hfma2(__low2half2(h0), ux, __low2half2(h1));
  const __half2 w1 = __hfma2(__high2half2(h0), uy, t);
  const __half2 w2 = __hfma2(__low2half2(h2), uy, __high2half2(h1));
  __half2 p = __hfma2(__hneg2(w1), w1, __high2half2(h2));
  p = __hfma2(__hneg2(w2), w2, p);
  const uint32_t m = __hge2_mask(p, th);
  *use_mask = m;
  const uint32_t q = (h22u(p) & m) | (0xFC00FC00u & ~m);  // -inf where unused
  return __half22float2(h2ex2_approx(__hmin2(u2h2(q), __float2half2_rn(kLog2MaxAlpha))));
}

// One warp's staged records (up to 32, compacted in record order).
struct WarpStage {
  float4 geo[32];  // cx, cy, -a/2 log2 e, -b log2 e (the half2 form: its Cholesky record)
  float4 con[32];  // -c/2 log2 e, log2 opacity, L as half2 bits, depth
  float4 col[32];  // r, g, b (the half2 form: and depth)
  float4 raw[32];  // conic (a, b, c) for periodic boundaries
  uint8_t idx[32]; // lane (record offset within the group) of each staged record
};

// DEPTH: some view of the launch has a depth target (otherwise the depth sum
// is never read and is not accumulated).
template <bool DEPTH>
__device__ __forceinline__ void blend_pixel(float alpha, const float4& col, float depth, PixelAcc& a) {
  const float contrib = a.t * alpha;
  a.r = a.r + col.x * contrib;
  a.g = a.g + col.y * contrib;
  a.b = a.b + col.z * contrib;
  if (DEPTH) a.d = a.d + depth * contrib;
  a.t = a.t - contrib;
}

// Blend records [s0, s1) of the tile into this warp's two pixels per lane.
// Warp-level: needs no other warp of the block.
template <bool HALF, bool PERIODIC, bool STATS, bool DEPTH>
__device__ __forceinline__ void blend_range_h2(uint32_t begin, uint32_t source_count, uint32_t raster_count,
                                               uint32_t s0, uint32_t s1, bool capped,
                                               const uint32_t* __restrict__ ids, const float4* __restrict__ mean,
                                               const float4* __restrict__ color,
                                               const float4* __restrict__ rec, bool need_depth,
                                               const RasterFrame& f, float patch_x0, float patch_y0, float pxc,
                                               float pyc0, bool done0, bool done1, PixelAcc& a0, PixelAcc& a1,
                                               WarpStage& ws, RasterCounters& c0n, RasterCounters& c1n) {
  const uint32_t lane = threadIdx.x & 31u;
  const bool count0 = STATS && !done0, count1 = STATS && !done1;
  uint32_t stop0 = s1, stop1 = s1;
  const float pyc1 = pyc0 + 4.0f;
  const uint32_t lt = (1u << lane) - 1u;
  // The half2 form's Cholesky evaluation: the pixels' offsets from the patch
  // centre (multiples of 0.5 within +-3.5, exact in f16).
  constexpr bool kChol = HALF && !PERIODIC;
  const float ecx = patch_x0 + 4.0f, ecy = patch_y0 + 4.0f;
  const __half2 ux2 = __float2half2_rn(pxc - ecx), uy2 = __floats2half2_rn(pyc0 - ecy, pyc1 - ecy);
  auto load_id = [&](uint32_t i) -> uint32_t {
    if (i >= s1) return 0u;
    uint32_t src = i;
    if (capped) src = (uint32_t)floorf((((float)i + 0.5f) * (float)source_count) / (float)raster_count);
    return __ldg(ids + begin + src);
  };
  // The FP32 form loads the next group's record ids one group ahead (the
  // half2 form, at its register limit for 10 blocks per SM, is faster without).
  uint32_t next_id = HALF ? 0u : load_id(s0 + lane);
  for (uint32_t b = s0; b < s1; b += 32) {
    if (__all_sync(0xffffffffu, done0 && done1)) break;
    const uint32_t i = b + lane;
    bool reach = false;
    float4 r0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), r1 = r0, col32 = r0;
    float depth = 0.0f;
    uint32_t cur_id = 0;
    if (!HALF) {
      cur_id = next_id;
      next_id = load_id(b + 32u + lane);
    }
    if (i < s1) {
      const uint32_t g = HALF ? load_id(i) : cur_id;
      r0 = __ldg(rec + 2 * (size_t)g);  // one 32-byte record
      r1 = __ldg(rec + 2 * (size_t)g + 1);
      if (!HALF) col32 = __ldg(color + g);
      if (DEPTH && need_depth) depth = __ldg(&mean[g].z);
      reach = PERIODIC || patch_reach(r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, patch_x0 + 0.5f, patch_y0 + 0.5f,
                                          7.0f, 7.0f);
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, reach);
    if (reach) {
      const uint32_t q = __popc(bal & lt);
      if (kChol) {
        *reinterpret_cast<uint4*>(&ws.geo[q]) = cholesky_record(r0, r1, ecx, ecy);
        const float2 rg = __half22float2(u2h2(__float_as_uint(r1.z)));
        ws.col[q] = make_float4(rg.x, rg.y, __low2float(u2h2(__float_as_uint(r1.w))), depth);
      } else {
        ws.geo[q] = r0;
        if (HALF) {
          const uint32_t rg_bits = __float_as_uint(r1.z), bl_bits = __float_as_uint(r1.w);
          const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&rg_bits));
          const __half2 bl = *reinterpret_cast<const __half2*>(&bl_bits);
          const __half2 lim = __half2half2(__high2half(bl));
          ws.con[q] = make_float4(r1.x, r1.y, __uint_as_float(*reinterpret_cast<const uint32_t*>(&lim)), depth);
          ws.col[q] = make_float4(rg.x, rg.y, __low2float(bl), 0.0f);
        } else {
          ws.con[q] = make_float4(r1.x, r1.y, fminf(r1.y, kLog2MaxAlpha), depth);
          ws.col[q] = col32;
        }
      }
      if (PERIODIC) ws.raw[q] = raw_conic(r0, r1);
      if (STATS) ws.idx[q] = (uint8_t)lane;
    }
    __syncwarp();
    const uint32_t n = __popc(bal);
    const float th0 = done0 ? __int_as_float(0x7f800000) : kLog2MinAlpha;
    const float th1 = done1 ? __int_as_float(0x7f800000) : kLog2MinAlpha;
    if (kChol) {
      const __half2 th2 = __floats2half2_rn(th0, th1);
      for (uint32_t j = 0; j < n; ++j) {
        uint32_t m;
        const float2 al = cholesky_alpha(*reinterpret_cast<const uint4*>(&ws.geo[j]), ux2, uy2, th2, &m);
        const float4 col = ws.col[j];  // r, g, b, depth
        if (!STATS) {
          // Unused pixels blend alpha +0, which changes nothing.
          blend_pixel<DEPTH>(al.x, col, col.w, a0);
          blend_pixel<DEPTH>(al.y, col, col.w, a1);
          continue;
        }
        if (m & 0xFFFFu) {
          blend_pixel<DEPTH>(al.x, col, col.w, a0);
          ++c0n.blended;
          if (a0.t < f.t_threshold && stop0 == s1) stop0 = b + ws.idx[j] + 1;
        }
        if (m >> 16) {
          blend_pixel<DEPTH>(al.y, col, col.w, a1);
          ++c1n.blended;
          if (a1.t < f.t_threshold && stop1 == s1) stop1 = b + ws.idx[j] + 1;
        }
      }
      done0 = done0 || a0.t < f.t_threshold;
      done1 = done1 || a1.t < f.t_threshold;
      __syncwarp();  // the staging area is rewritten by the next group
      continue;
    }
    for (uint32_t j = 0; j < n; ++j) {
      const float4 g = ws.geo[j];
      const float4 c = ws.con[j];
      float p0, p1;
      if (PERIODIC) {
        const float4 r = ws.raw[j];
        float dx0, dy0, dx1, dy1;
        boundary_delta<true>(pxc, pyc0, g.x, g.y, r.x, r.y, r.z, f, &dx0, &dy0);
        boundary_delta<true>(pxc, pyc1, g.x, g.y, r.x, r.y, r.z, f, &dx1, &dy1);
        p0 = fmaf(g.z * dx0, dx0, fmaf(g.w * dx0, dy0, fmaf(c.x * dy0, dy0, c.y)));
        p1 = fmaf(g.z * dx1, dx1, fmaf(g.w * dx1, dy1, fmaf(c.x * dy1, dy1, c.y)));
      } else {
        const float dx = pxc - g.x;
        const float dy0 = pyc0 - g.y, dy1 = pyc1 - g.y;
        const float bdx = g.w * dx, xx = fmaf(g.z * dx, dx, c.y);
        p0 = fmaf(fmaf(c.x, dy0, bdx), dy0, xx);
        p1 = fmaf(fmaf(c.x, dy1, bdx), dy1, xx);
      }
      const bool use0 = p0 >= th0;
      const bool use1 = p1 >= th1;
      if (!STATS) {
        // Branch-free: a pixel below the threshold (or done) blends alpha
        // 2^-inf = +0, which leaves its colour, depth and transmittance
        // exactly unchanged (t * 0 = 0, x + c * 0 = x for finite c).
        const float q0 = use0 ? p0 : -__int_as_float(0x7f800000);
        const float q1 = use1 ? p1 : -__int_as_float(0x7f800000);
        float2 al;
        if (HALF) {
          const uint32_t lim_bits = __float_as_uint(c.z);
          al = __half22float2(
              h2ex2_approx(__hmin2(__floats2half2_rn(q0, q1), *reinterpret_cast<const __half2*>(&lim_bits))));
        } else {
          al.x = ex2_approx(fminf(q0, c.z));
          al.y = ex2_approx(fminf(q1, c.z));
        }
        const float4 col = ws.col[j];
        blend_pixel<DEPTH>(al.x, col, c.w, a0);
        blend_pixel<DEPTH>(al.y, col, c.w, a1);
        continue;
      }
      if (!(use0 || use1)) continue;
      float2 al;
      if (HALF) {
        const uint32_t lim_bits = __float_as_uint(c.z);
        al = __half22float2(
            h2ex2_approx(__hmin2(__floats2half2_rn(p0, p1), *reinterpret_cast<const __half2*>(&lim_bits))));
      } else {
        al.x = ex2_approx(fminf(p0, c.z));
        al.y = ex2_approx(fminf(p1, c.z));
      }
      const float4 col = ws.col[j];
      if (use0) {
        blend_pixel<DEPTH>(al.x, col, c.w, a0);
        if (STATS) {
          ++c0n.blended;
          if (a0.t < f.t_threshold && stop0 == s1) stop0 = b + ws.idx[j] + 1;
        }
      }
      if (use1) {
        blend_pixel<DEPTH>(al.y, col, c.w, a1);
        if (STATS) {
          ++c1n.blended;
          if (a1.t < f.t_threshold && stop1 == s1) stop1 = b + ws.idx[j] + 1;
        }
      }
    }
    done0 = done0 || a0.t < f.t_threshold;
    done1 = done1 || a1.t < f.t_threshold;
    __syncwarp();  // the staging area is rewritten by the next group
  }
  if (count0) c0n.checked += stop0 - s0;
  if (count1) c1n.checked += stop1 - s0;
}

// The same blend for K pixels per lane (pixels (x, y + 4 i), i < K, in pairs):
// the block shape of a warp per 8 x 4K patch. Warp-level: needs no other warp
// of the block.
template <bool HALF, bool PERIODIC, bool STATS, bool DEPTH, int K>
__device__ __forceinline__ void blend_range_hk(uint32_t begin, uint32_t source_count, uint32_t raster_count,
                                               uint32_t s0, uint32_t s1, bool capped,
                                               const uint32_t* __restrict__ ids, const float4* __restrict__ mean,
                                               const float4* __restrict__ color,
                                               const float4* __restrict__ rec, bool need_depth,
                                               const RasterFrame& f, float patch_x0, float patch_y0, float pxc,
                                               float pyc0, bool (&done)[K], PixelAcc (&acc)[K], WarpStage& ws,
                                               RasterCounters (&cnt)[K]) {
  static_assert(K % 2 == 0, "pixels are evaluated in pairs");
  const uint32_t lane = threadIdx.x & 31u;
  bool counting[K];
  uint32_t stop[K];
  float pyc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    counting[k] = STATS && !done[k];
    stop[k] = s1;
    pyc[k] = pyc0 + 4.0f * (float)k;
  }
  const uint32_t lt = (1u << lane) - 1u;
  // The half2 form's Cholesky evaluation about the 8 x 4K patch's centre
  // (offsets within +-3.5 in x and +-(2K - 0.5) in y, exact in f16).
  constexpr bool kChol = HALF && !PERIODIC;
  const float ecx = patch_x0 + 4.0f, ecy = patch_y0 + 2.0f * (float)K;
  const __half2 ux2 = __float2half2_rn(pxc - ecx);
  __half2 uy2[K / 2];
#pragma unroll
  for (int k = 0; k < K; k += 2) uy2[k / 2] = __floats2half2_rn(pyc[k] - ecy, pyc[k + 1] - ecy);
  auto load_id = [&](uint32_t i) -> uint32_t {
    if (i >= s1) return 0u;
    uint32_t src = i;
    if (capped) src = (uint32_t)floorf((((float)i + 0.5f) * (float)source_count) / (float)raster_count);
    return __ldg(ids + begin + src);
  };
  auto all_done = [&]() {
    bool d = true;
#pragma unroll
    for (int k = 0; k < K; ++k) d = d && done[k];
    return d;
  };
  // The FP32 form loads the next group's record ids one group ahead (the
  // half2 form, at its register limit, is faster without).
  uint32_t next_id = HALF ? 0u : load_id(s0 + lane);
  for (uint32_t b = s0; b < s1; b += 32) {
    if (__all_sync(0xffffffffu, all_done())) break;
    const uint32_t i = b + lane;
    bool reach = false;
    float4 r0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), r1 = r0, col32 = r0;
    float depth = 0.0f;
    uint32_t cur_id = 0;
    if (!HALF) {
      cur_id = next_id;
      next_id = load_id(b + 32u + lane);
    }
    if (i < s1) {
      const uint32_t g = HALF ? load_id(i) : cur_id;
      r0 = __ldg(rec + 2 * (size_t)g);  // one 32-byte record
      r1 = __ldg(rec + 2 * (size_t)g + 1);
      if (!HALF) col32 = __ldg(color + g);
      if (DEPTH && need_depth) depth = __ldg(&mean[g].z);
      reach = PERIODIC || patch_reach(r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, patch_x0 + 0.5f, patch_y0 + 0.5f,
                                          7.0f, 4.0f * (float)K - 1.0f);
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, reach);
    if (reach) {
      const uint32_t q = __popc(bal & lt);
      if (kChol) {
        *reinterpret_cast<uint4*>(&ws.geo[q]) = cholesky_record(r0, r1, ecx, ecy);
        const float2 rg = __half22float2(u2h2(__float_as_uint(r1.z)));
        ws.col[q] = make_float4(rg.x, rg.y, __low2float(u2h2(__float_as_uint(r1.w))), depth);
      } else {
        ws.geo[q] = r0;
        if (HALF) {
          const uint32_t rg_bits = __float_as_uint(r1.z), bl_bits = __float_as_uint(r1.w);
          const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&rg_bits));
          const __half2 bl = *reinterpret_cast<const __half2*>(&bl_bits);
          const __half2 lim = __half2half2(__high2half(bl));
          ws.con[q] = make_float4(r1.x, r1.y, __uint_as_float(*reinterpret_cast<const uint32_t*>(&lim)), depth);
          ws.col[q] = make_float4(rg.x, rg.y, __low2float(bl), 0.0f);
        } else {
          ws.con[q] = make_float4(r1.x, r1.y, fminf(r1.y, kLog2MaxAlpha), depth);
          ws.col[q] = col32;
        }
      }
      if (PERIODIC) ws.raw[q] = raw_conic(r0, r1);
      if (STATS) ws.idx[q] = (uint8_t)lane;
    }
    __syncwarp();
    const uint32_t n = __popc(bal);
    float th[K];
#pragma unroll
    for (int k = 0; k < K; ++k) th[k] = done[k] ? __int_as_float(0x7f800000) : kLog2MinAlpha;
    if (kChol) {
      __half2 th2[K / 2];
#pragma unroll
      for (int k = 0; k < K; k += 2) th2[k / 2] = __floats2half2_rn(th[k], th[k + 1]);
      for (uint32_t j = 0; j < n; ++j) {
        const uint4 h = *reinterpret_cast<const uint4*>(&ws.geo[j]);
        const float4 col = ws.col[j];  // r, g, b, depth
#pragma unroll
        for (int k = 0; k < K; k += 2) {
          uint32_t m;
          const float2 al = cholesky_alpha(h, ux2, uy2[k / 2], th2[k / 2], &m);
          if (!STATS) {
            // Unused pixels blend alpha +0, which changes nothing.
            blend_pixel<DEPTH>(al.x, col, col.w, acc[k]);
            blend_pixel<DEPTH>(al.y, col, col.w, acc[k + 1]);
            continue;
          }
          if (m & 0xFFFFu) {
            blend_pixel<DEPTH>(al.x, col, col.w, acc[k]);
            ++cnt[k].blended;
            if (acc[k].t < f.t_threshold && stop[k] == s1) stop[k] = b + ws.idx[j] + 1;
          }
          if (m >> 16) {
            blend_pixel<DEPTH>(al.y, col, col.w, acc[k + 1]);
            ++cnt[k + 1].blended;
            if (acc[k + 1].t < f.t_threshold && stop[k + 1] == s1) stop[k + 1] = b + ws.idx[j] + 1;
          }
        }
      }
#pragma unroll
      for (int k = 0; k < K; ++k) done[k] = done[k] || acc[k].t < f.t_threshold;
      __syncwarp();  // the staging area is rewritten by the next group
      continue;
    }
    for (uint32_t j = 0; j < n; ++j) {
      const float4 g = ws.geo[j];
      const float4 c = ws.con[j];
      float pv[K];
      if (PERIODIC) {
        const float4 r = ws.raw[j];
#pragma unroll
        for (int k = 0; k < K; ++k) {
          float dx, dy;
          boundary_delta<true>(pxc, pyc[k], g.x, g.y, r.x, r.y, r.z, f, &dx, &dy);
          pv[k] = fmaf(g.z * dx, dx, fmaf(g.w * dx, dy, fmaf(c.x * dy, dy, c.y)));
        }
      } else {
        // The lane's pixels share dx and the x-only terms of the quadratic.
        const float dx = pxc - g.x;
        const float bdx = g.w * dx, xx = fmaf(g.z * dx, dx, c.y);
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const float dy = pyc[k] - g.y;
          pv[k] = fmaf(fmaf(c.x, dy, bdx), dy, xx);
        }
      }
      if (!STATS) {
        // Branch-free: a pixel below the threshold (or done) blends alpha
        // 2^-inf = +0, which leaves its colour, depth and transmittance
        // exactly unchanged (t * 0 = 0, x + c * 0 = x for finite c).
        const float4 col = ws.col[j];
#pragma unroll
        for (int k = 0; k < K; k += 2) {
          const float q0 = pv[k] >= th[k] ? pv[k] : -__int_as_float(0x7f800000);
          const float q1 = pv[k + 1] >= th[k + 1] ? pv[k + 1] : -__int_as_float(0x7f800000);
          float2 al;
          if (HALF) {
            const uint32_t lim_bits = __float_as_uint(c.z);
            al = __half22float2(
                h2ex2_approx(__hmin2(__floats2half2_rn(q0, q1), *reinterpret_cast<const __half2*>(&lim_bits))));
          } else {
            al.x = ex2_approx(fminf(q0, c.z));
            al.y = ex2_approx(fminf(q1, c.z));
          }
          blend_pixel<DEPTH>(al.x, col, c.w, acc[k]);
          blend_pixel<DEPTH>(al.y, col, c.w, acc[k + 1]);
        }
        continue;
      }
      const float4 col = ws.col[j];
#pragma unroll
      for (int k = 0; k < K; k += 2) {
        const bool use0 = pv[k] >= th[k];
        const bool use1 = pv[k + 1] >= th[k + 1];
        if (!(use0 || use1)) continue;
        float2 al;
        if (HALF) {
          const uint32_t lim_bits = __float_as_uint(c.z);
          al = __half22float2(h2ex2_approx(
              __hmin2(__floats2half2_rn(pv[k], pv[k + 1]), *reinterpret_cast<const __half2*>(&lim_bits))));
        } else {
          al.x = ex2_approx(fminf(pv[k], c.z));
          al.y = ex2_approx(fminf(pv[k + 1], c.z));
        }
        if (use0) {
          blend_pixel<DEPTH>(al.x, col, c.w, acc[k]);
          ++cnt[k].blended;
          if (acc[k].t < f.t_threshold && stop[k] == s1) stop[k] = b + ws.idx[j] + 1;
        }
        if (use1) {
          blend_pixel<DEPTH>(al.y, col, c.w, acc[k + 1]);
          ++cnt[k + 1].blended;
          if (acc[k + 1].t < f.t_threshold && stop[k + 1] == s1) stop[k + 1] = b + ws.idx[j] + 1;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) done[k] = done[k] || acc[k].t < f.t_threshold;
    __syncwarp();  // the staging area is rewritten by the next group
  }
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (counting[k]) cnt[k].checked += stop[k] - s0;
}

__device__ __forceinline__ void store_pixel(const ViewDesc& v, const PassOptions& o, uint32_t px, uint32_t py,
                                            const PixelAcc& a) {
  const uint32_t W = (uint32_t)v.vw;
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

// Threads of the block for a TILE x TILE tile: one warp per 8x8 patch.
template <int TILE>
constexpr int h2_threads() {
  return 32 * (TILE / 8) * (TILE / 8);
}
// Resident blocks per SM the register budget is set for: 10 blocks of 128
// threads (half2: 48 registers; 9 and 12 blocks measured slower) / 8 (FP32)
// at the reference's 16-pixel tiles, the same threads per SM at other tile
// sizes (at most 32 blocks).
template <bool HALF, int TILE>
constexpr int h2_min_blocks() {
  return (HALF ? 1280 : 1024) / h2_threads<TILE>() > 32 ? 32 : (HALF ? 1280 : 1024) / h2_threads<TILE>();
}

template <bool HALF, bool PERIODIC, bool STATS, bool DEPTH, int TILE>
__global__ void __launch_bounds__(h2_threads<TILE>(), h2_min_blocks<HALF, TILE>())
    k_raster_h2(const uint32_t* __restrict__ tile_offsets,
                                                           const uint32_t* __restrict__ order,
                                                           const uint32_t* __restrict__ ids,
                                                           const float4* __restrict__ mean,
                                                           const float4* __restrict__ color,
                                                           const float4* __restrict__ rec, BatchView bv,
                                                           PassOptions o, Control* __restrict__ ctl) {
  if (ctl->state[3] != 0u) return;  // overflow: nothing is published
  constexpr uint32_t PW = TILE / 8;  // patches per tile row
  __shared__ WarpStage s_stage[PW * PW];
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
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  WarpStage& ws = s_stage[warp];
  const uint32_t patch_x = tx * TILE + 8u * (warp % PW), patch_y = ty * TILE + 8u * (warp / PW);
  const uint32_t px = patch_x + morton_compact(lane);
  const uint32_t py0 = patch_y + morton_compact(lane >> 1);
  const uint32_t py1 = py0 + 4u;
  const uint32_t W = (uint32_t)v.vw, H = (uint32_t)v.vh;
  const bool active0 = px < W && py0 < H, active1 = px < W && py1 < H;
  const uint32_t begin = tile_offsets[tile], end = tile_offsets[tile + 1];
  const uint32_t source_count = end - begin;
  const bool capped = o.max_per_tile != 0u;
  const uint32_t raster_count = capped ? min(source_count, o.max_per_tile) : source_count;
  const uint32_t chunk = o.chunk;
  const bool chunked = chunk != 0u && raster_count > chunk;
  const bool need_depth = v.depth != nullptr;
  const float pxc = (float)px + 0.5f, pyc0 = (float)py0 + 0.5f;
  PixelAcc a0 = {0.0f, 0.0f, 0.0f, 1.0f, 0.0f}, a1 = a0;
  RasterCounters n0 = {0u, 0u}, n1 = {0u, 0u};
  if (!chunked) {
    blend_range_h2<HALF, PERIODIC, STATS, DEPTH>(begin, source_count, raster_count, 0, raster_count, capped, ids, mean,
                                          color, rec, need_depth, f, (float)patch_x, (float)patch_y, pxc, pyc0, !active0, !active1, a0,
                                    a1, ws, n0, n1);
  } else {
    const uint32_t nchunk = (raster_count + chunk - 1) / chunk;
    bool fin0 = !active0, fin1 = !active1;
    for (uint32_t ch = 0; ch < nchunk; ++ch) {
      if (__all_sync(0xffffffffu, fin0 && fin1)) break;
      const uint32_t s0 = ch * chunk, s1 = min(s0 + chunk, raster_count);
      PixelAcc p0 = {0.0f, 0.0f, 0.0f, 1.0f, 0.0f}, p1 = p0;
      blend_range_h2<HALF, PERIODIC, STATS, DEPTH>(begin, source_count, raster_count, s0, s1, capped, ids, mean, color,
                                            rec, need_depth,
                                      f, (float)patch_x, (float)patch_y, pxc, pyc0, fin0, fin1, p0, p1, ws, n0, n1);
      if (!fin0) {
        a0.r = a0.r + p0.r * a0.t; a0.g = a0.g + p0.g * a0.t; a0.b = a0.b + p0.b * a0.t;
        a0.d = a0.d + p0.d * a0.t; a0.t = a0.t * p0.t;
        if (a0.t < f.t_threshold) fin0 = true;
      }
      if (!fin1) {
        a1.r = a1.r + p1.r * a1.t; a1.g = a1.g + p1.g * a1.t; a1.b = a1.b + p1.b * a1.t;
        a1.d = a1.d + p1.d * a1.t; a1.t = a1.t * p1.t;
        if (a1.t < f.t_threshold) fin1 = true;
      }
    }
  }
  if (STATS) {
    for (int q = 0; q < 2; ++q) {
      const bool act = q == 0 ? active0 : active1;
      const RasterCounters& cn = q == 0 ? n0 : n1;
      const PixelAcc& aq = q == 0 ? a0 : a1;
      if (act) {
        atomicAdd(&s_stats[0], (unsigned long long)cn.checked);
        atomicAdd(&s_stats[1], (unsigned long long)cn.blended);
        if (raster_count > 0) {
          atomicAdd(&s_stats[2], 1ull);
          if (aq.t < f.t_threshold) atomicAdd(&s_stats[3], 1ull);
        }
      }
    }
    __syncthreads();
    if (threadIdx.x < 4 && s_stats[threadIdx.x]) atomicAdd(&ctl->raster_stats[threadIdx.x], s_stats[threadIdx.x]);
  }
  if (active0) store_pixel(v, o, px, py0, a0);
  if (active1) store_pixel(v, o, px, py1, a1);
}

// The rasterizer with K pixels per lane (the other block shape of the fast
// forms): threads of the block for a TILE x TILE tile, one warp per 8 x 4K
// patch.
template <int TILE, int K>
constexpr int hk_threads() {
  return 32 * (TILE / 8) * (TILE / (4 * K));
}
// Resident blocks per SM the register budget is set for: 768 threads per SM
// (the K accumulators need more registers than k_raster_h2's pair).
template <bool HALF, int TILE, int K>
constexpr int hk_threads_per_sm() {
  return 768;
}
template <bool HALF, int TILE, int K>
constexpr int hk_min_blocks() {
  return hk_threads_per_sm<HALF, TILE, K>() / hk_threads<TILE, K>() > 32
             ? 32
             : hk_threads_per_sm<HALF, TILE, K>() / hk_threads<TILE, K>();
}

template <bool HALF, bool PERIODIC, bool STATS, bool DEPTH, int TILE, int K>
__global__ void __launch_bounds__(hk_threads<TILE, K>(), hk_min_blocks<HALF, TILE, K>())
    k_raster_hk(const uint32_t* __restrict__ tile_offsets, const uint32_t* __restrict__ order,
                const uint32_t* __restrict__ ids, const float4* __restrict__ mean, const float4* __restrict__ color,
                const float4* __restrict__ rec, BatchView bv, PassOptions o, Control* __restrict__ ctl) {
  if (ctl->state[3] != 0u) return;  // overflow: nothing is published
  constexpr uint32_t PW = TILE / 8;             // patches per tile row
  constexpr uint32_t PH = TILE / (4 * K);       // patch rows per tile
  __shared__ WarpStage s_stage[PW * PH];
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
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  WarpStage& ws = s_stage[warp];
  const uint32_t patch_x = tx * TILE + 8u * (warp % PW), patch_y = ty * TILE + 4u * K * (warp / PW);
  const uint32_t px = patch_x + morton_compact(lane);
  const uint32_t py0 = patch_y + morton_compact(lane >> 1);
  const uint32_t W = (uint32_t)v.vw, H = (uint32_t)v.vh;
  bool active[K];
#pragma unroll
  for (int k = 0; k < K; ++k) active[k] = px < W && py0 + 4u * k < H;
  const uint32_t begin = tile_offsets[tile], end = tile_offsets[tile + 1];
  const uint32_t source_count = end - begin;
  const bool capped = o.max_per_tile != 0u;
  const uint32_t raster_count = capped ? min(source_count, o.max_per_tile) : source_count;
  const uint32_t chunk = o.chunk;
  const bool chunked = chunk != 0u && raster_count > chunk;
  const bool need_depth = v.depth != nullptr;
  const float pxc = (float)px + 0.5f, pyc0 = (float)py0 + 0.5f;
  PixelAcc a[K];
  RasterCounters n[K];
  bool fin[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    a[k] = {0.0f, 0.0f, 0.0f, 1.0f, 0.0f};
    n[k] = {0u, 0u};
    fin[k] = !active[k];
  }
  if (!chunked) {
    blend_range_hk<HALF, PERIODIC, STATS, DEPTH, K>(begin, source_count, raster_count, 0, raster_count, capped, ids,
                                                    mean, color, rec, need_depth, f, (float)patch_x, (float)patch_y,
                                                    pxc, pyc0, fin, a, ws, n);
  } else {
    const uint32_t nchunk = (raster_count + chunk - 1) / chunk;
    for (uint32_t ch = 0; ch < nchunk; ++ch) {
      bool all = true;
#pragma unroll
      for (int k = 0; k < K; ++k) all = all && fin[k];
      if (__all_sync(0xffffffffu, all)) break;
      const uint32_t s0 = ch * chunk, s1 = min(s0 + chunk, raster_count);
      PixelAcc p[K];
      bool pfin[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        p[k] = {0.0f, 0.0f, 0.0f, 1.0f, 0.0f};
        pfin[k] = fin[k];
      }
      blend_range_hk<HALF, PERIODIC, STATS, DEPTH, K>(begin, source_count, raster_count, s0, s1, capped, ids, mean,
                                                      color, rec, need_depth, f, (float)patch_x, (float)patch_y, pxc,
                                                      pyc0, pfin, p, ws, n);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (fin[k]) continue;
        a[k].r = a[k].r + p[k].r * a[k].t; a[k].g = a[k].g + p[k].g * a[k].t; a[k].b = a[k].b + p[k].b * a[k].t;
        a[k].d = a[k].d + p[k].d * a[k].t; a[k].t = a[k].t * p[k].t;
        if (a[k].t < f.t_threshold) fin[k] = true;
      }
    }
  }
  if (STATS) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (active[k]) {
        atomicAdd(&s_stats[0], (unsigned long long)n[k].checked);
        atomicAdd(&s_stats[1], (unsigned long long)n[k].blended);
        if (raster_count > 0) {
          atomicAdd(&s_stats[2], 1ull);
          if (a[k].t < f.t_threshold) atomicAdd(&s_stats[3], 1ull);
        }
      }
    }
    __syncthreads();
    if (threadIdx.x < 4 && s_stats[threadIdx.x]) atomicAdd(&ctl->raster_stats[threadIdx.x], s_stats[threadIdx.x]);
  }
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (active[k]) store_pixel(v, o, px, py0 + 4u * k, a[k]);
}

// half = true: packed half2 form; false: FP32 form. o.any_depth: some view
// of the launch has a depth target.
template <bool HALF, bool PERIODIC, int TILE>
inline void launch_raster_pairs_tile(const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* ids,
                                     const float4* mean, const float4* color, const float4* rec, const BatchView& b,
                                     const PassOptions& o, Control* ctl, bool stats, cudaStream_t st) {
#define GS_RASTER_H2(S, D)                                                                          \
  k_raster_h2<HALF, PERIODIC, S, D, TILE><<<b.total_tiles, h2_threads<TILE>(), 0, st>>>(            \
      tile_offsets, order, ids, mean, color, rec, b, o, ctl)
  const bool depth = o.any_depth != 0u;
  if (stats) {
    if (depth) GS_RASTER_H2(true, true); else GS_RASTER_H2(true, false);
  } else {
    if (depth) GS_RASTER_H2(false, true); else GS_RASTER_H2(false, false);
  }
#undef GS_RASTER_H2
}

template <bool HALF, bool PERIODIC, int TILE, int K>
inline void launch_raster_k_tile(const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* ids,
                                 const float4* mean, const float4* color, const float4* rec, const BatchView& b,
                                 const PassOptions& o, Control* ctl, bool stats, cudaStream_t st) {
#define GS_RASTER_HK(S, D)                                                                          \
  k_raster_hk<HALF, PERIODIC, S, D, TILE, K><<<b.total_tiles, hk_threads<TILE, K>(), 0, st>>>(      \
      tile_offsets, order, ids, mean, color, rec, b, o, ctl)
  const bool depth = o.any_depth != 0u;
  if (stats) {
    if (depth) GS_RASTER_HK(true, true); else GS_RASTER_HK(true, false);
  } else {
    if (depth) GS_RASTER_HK(false, true); else GS_RASTER_HK(false, false);
  }
#undef GS_RASTER_HK
}

template <bool HALF, bool PERIODIC>
inline void launch_raster_pairs_t(const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* ids,
                                  const float4* mean, const float4* color, const float4* rec, const BatchView& b,
                                  const PassOptions& o, Control* ctl, bool stats, cudaStream_t st) {
  // Four pixels per lane (one warp per 8x16 patch) where the tile holds such
  // patches; otherwise two (one warp per 8x8 patch).
  const bool four = o.pixels_per_lane == 4u && o.tile >= 16u;
  if (o.tile == 8u)
    launch_raster_pairs_tile<HALF, PERIODIC, 8>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
  else if (o.tile == 32u && four)
    launch_raster_k_tile<HALF, PERIODIC, 32, 4>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
  else if (o.tile == 32u)
    launch_raster_pairs_tile<HALF, PERIODIC, 32>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
  else if (four)
    launch_raster_k_tile<HALF, PERIODIC, 16, 4>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
  else
    launch_raster_pairs_tile<HALF, PERIODIC, 16>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
}

// The half2 form's Cholesky evaluation needs the screen-space low-pass
// filter: it bounds the conic's eigenvalues by 1 / filterVariance, and with
// that the magnitudes of the f16 factor and of w at the patch centre. Below
// this variance (the filter switched off or nearly: splats may be far thinner
// than a pixel, and w at the patch centre reaches hundreds, past f16's
// resolution) the half2 form renders with the FP32 form's evaluation. A CPU
// model of the f16 arithmetic over random conics (sigma 0.001-300 px,
// anisotropy up to 200) bounds the per-splat alpha error by 0.005 from a
// variance of 0.05 up; with none it reaches 0.25.
constexpr float kHalf2MinFilterVariance = 0.05f;

inline void launch_raster_pairs(bool half, const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* ids,
                                const float4* mean, const float4* color, const float4* rec, const BatchView& b,
                                const PassOptions& o, Control* ctl, bool stats, cudaStream_t st) {
  if (b.total_tiles == 0) return;
  const bool periodic = o.axis != 0u;
  if (half && !periodic && !(o.filter >= kHalf2MinFilterVariance)) half = false;
  if (half) {
    if (periodic) launch_raster_pairs_t<true, true>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
    else launch_raster_pairs_t<true, false>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
  } else {
    if (periodic) launch_raster_pairs_t<false, true>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
    else launch_raster_pairs_t<false, false>(tile_offsets, order, ids, mean, color, rec, b, o, ctl, stats, st);
  }
}

}  // namespace gs
