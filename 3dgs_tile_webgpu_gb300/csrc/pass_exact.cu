// Kernels whose integer outputs must be bit-identical to the CPU restatement:
// projection + tile count, visibility compaction, the saturating intersection
// scan, intersection emission and tile ranges; plus the bit-exact raster form.
// Built with --fmad=false (see build.py): no multiply-add contraction, so each
// float expression rounds exactly like the CPU restatement.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "pass_common.cuh"
#include "raster_impl.cuh"
#include "splat_math.cuh"

namespace gs {

// ---------------------------------------------------------------------------
// K1: decode + project + cull + SH + tile count, one thread per active ordinal
// of every view group (ProjectionStage.ts:385-649): consecutive views of a
// batch that render the same packed scene form a group, and each thread
// decodes its splat once and projects it into every view of the group. Writes
// the projected mean/conic/colour/count like the reference, plus the depth
// sort key (or kInvisibleKey), which the compaction consumes instead of
// re-reading the 16-byte means. Each block belongs to one group; the padding
// items after a view's last ordinal are written as invisible.
__device__ __forceinline__ void load_sh(const uint32_t* __restrict__ p, uint32_t degree, uint32_t* co) {
  if (degree == 3) {
    const uint4* v = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      uint4 w = __ldg(v + i);
      co[4 * i] = w.x; co[4 * i + 1] = w.y; co[4 * i + 2] = w.z; co[4 * i + 3] = w.w;
    }
  } else {
    // Fully unrolled with constant indices so co[] stays in registers.
    const uint32_t C = (degree + 1) * (degree + 1);
#pragma unroll
    for (uint32_t i = 0; i < 16; ++i) co[i] = i < C ? __ldg(p + i) : 0u;
  }
}

// FAST: the colour feeds only a fast raster form (eval_sh_fast); otherwise
// the reference's expression order (eval_sh, bit-exact with the oracle).
template <bool FAST>
__device__ __forceinline__ f3 eval_sh_any(uint32_t degree, const uint32_t* co, f3 d, const float* snorm) {
  if (FAST) {
    switch (degree) {
      case 0: return eval_sh_fast<0>(co, d);
      case 1: return eval_sh_fast<1>(co, d);
      case 2: return eval_sh_fast<2>(co, d);
      default: return eval_sh_fast<3>(co, d);
    }
  }
  switch (degree) {
    case 0: return eval_sh<0>(co, d, snorm);
    case 1: return eval_sh<1>(co, d, snorm);
    case 2: return eval_sh<2>(co, d, snorm);
    default: return eval_sh<3>(co, d, snorm);
  }
}

// Bits [s, e) of a word, 0 <= s < e <= 32.
__device__ __forceinline__ uint32_t bit_range(uint32_t s, uint32_t e) {
  return (e >= 32u ? 0xffffffffu : ((1u << e) - 1u)) & ~((1u << s) - 1u);
}

// Boxes of at least this many tiles are walked by the whole warp, one box at
// a time, instead of in the shared rounds of the tile count and the emission:
// no per-tile owner lookup, the owner's parameters broadcast to every lane.
constexpr uint32_t kWideBox = 64;

// Per-warp tables of the projection's cooperative tile count: the splat
// parameters of the tile test, the box, and the inclusive box-tile counts.
struct CountShared {
  float f[8][kBlock / 32][32];     // cx, cy, conic a, b, c, threshold, rx, ry
  uint32_t u[4][kBlock / 32][32];  // tminx, tminy, box width, box index of the centre tile (or ~0)
  uint32_t incl[kBlock / 32][32];
  uint32_t cnt[kBlock / 32][32];
};

// Counts the tiles of every lane's box that pass the reference's tile test,
// with the warp's lanes spread over the union of the 32 boxes (32 box tiles
// per round) instead of each lane walking its own box. A lane walks nbox
// tiles of its box in row-major order, skipping the box index u[3] (the
// centre's tile, counted by the caller); boxes of kWideBox tiles or more are
// walked afterwards by the whole warp, one at a time. Must be called by all
// 32 lanes; a lane with nbox == 0 contributes nothing. Returns the lane's
// count.
__device__ __forceinline__ uint32_t count_tiles_warp(CountShared& sm, uint32_t nbox, float vw, float vh,
                                                     uint32_t axis, float ts) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  // Wide boxes (kWideBox tiles or more) are left out of the shared rounds and
  // walked by the whole warp afterwards, one box at a time.
  const bool wide = nbox >= kWideBox;
  uint32_t incl = wide ? 0u : nbox;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= (uint32_t)d) incl += y;
  }
  sm.incl[warp][lane] = incl;
  sm.cnt[warp][lane] = 0u;
  __syncwarp();
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  for (uint32_t j0 = 0; j0 < total; j0 += 32) {
    const uint32_t j = j0 + lane;
    const bool valid = j < total;
    uint32_t owner = 0;
#pragma unroll
    for (uint32_t step = 16; step >= 1; step >>= 1)
      if (sm.incl[warp][owner + step - 1] <= j) owner += step;
    bool hit = false;
    if (valid) {
      const uint32_t bw = sm.u[2][warp][owner];
      uint32_t k = j - (owner ? sm.incl[warp][owner - 1] : 0u);
      k += k >= sm.u[3][warp][owner] ? 1u : 0u;
      const uint32_t by = k / bw, bx = k - by * bw;
      hit = boundary_tile_hit(sm.f[0][warp][owner], sm.f[1][warp][owner], sm.f[2][warp][owner],
                              sm.f[3][warp][owner], sm.f[4][warp][owner], sm.f[5][warp][owner],
                              sm.f[6][warp][owner], sm.f[7][warp][owner], (int)(sm.u[0][warp][owner] + bx),
                              (int)(sm.u[1][warp][owner] + by), vw, vh, axis, ts);
    }
    const uint32_t hits = __ballot_sync(0xffffffffu, hit);
    const uint32_t same = __match_any_sync(0xffffffffu, valid ? owner : 32u + lane);
    if (valid && lane == 31u - (uint32_t)__clz(same)) sm.cnt[warp][owner] += __popc(hits & same);
  }
  __syncwarp();
  uint32_t cnt = sm.cnt[warp][lane];
  // Wide boxes: the whole warp walks one box, 32 tiles a step.
  uint32_t wide_lanes = __ballot_sync(0xffffffffu, wide);
  while (wide_lanes) {
    const uint32_t w = (uint32_t)__ffs(wide_lanes) - 1u;
    wide_lanes &= wide_lanes - 1u;
    // The owner's parameters are read from the warp's table at each step
    // (broadcast loads) rather than held in registers across the walk.
    const volatile float(*vf)[kBlock / 32][32] = sm.f;
    const volatile uint32_t(*vu)[kBlock / 32][32] = sm.u;
    const uint32_t n = __shfl_sync(0xffffffffu, nbox, w);
    uint32_t sum = 0;
    for (uint32_t j0 = 0; j0 < n; j0 += 32) {
      uint32_t k = j0 + lane;
      bool hit = false;
      if (k < n) {
        k += k >= vu[3][warp][w] ? 1u : 0u;
        const uint32_t bw = vu[2][warp][w];
        const uint32_t by = k / bw, bx = k - by * bw;
        hit = boundary_tile_hit(vf[0][warp][w], vf[1][warp][w], vf[2][warp][w], vf[3][warp][w], vf[4][warp][w],
                                vf[5][warp][w], vf[6][warp][w], vf[7][warp][w], (int)(vu[0][warp][w] + bx),
                                (int)(vu[1][warp][w] + by), vw, vh, axis, ts);
      }
      sum += __popc(__ballot_sync(0xffffffffu, hit));
    }
    if (lane == w) cnt = sum;
  }
  return cnt;
}

// GROUPED: some group holds several views (decode once, before the view
// loop); otherwise every group is one view and the decode stays inside the
// per-view chain, after the object tests, where it costs fewest registers.
template <bool FP64, bool GROUPED, bool FAST_SH>
__global__ void __launch_bounds__(kBlock, 4) k_project(BatchView b, PassOptions o, float4* __restrict__ mean_out,
                                                    float4* __restrict__ conic_out, float4* __restrict__ color_out,
                                                    uint32_t* __restrict__ count_out, uint32_t* __restrict__ key_out,
                                                    float4* __restrict__ rec_out, float4* __restrict__ erec_out) {
  __shared__ float s_snorm[256];
  __shared__ uint32_t s_group;
  __shared__ CountShared s_count;
  s_snorm[threadIdx.x] = snorm8_value(threadIdx.x);
  if (threadIdx.x == 0) s_group = find_view(b.group_block, b.ngroups, blockIdx.x);
  __syncthreads();
  const uint32_t g = s_group;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t gid = (blockIdx.x - __ldg(b.group_block + g)) * kBlock + threadIdx.x;  // ordinal in each view
  const uint32_t v_first = __ldg(b.group_view + g);
  const uint32_t v_end = GROUPED ? __ldg(b.group_view + g + 1) : v_first + 1u;

  // Decode the splat once for every view of the group (the views share the
  // packed scene, so the active tail, means, shape and rotation are common).
  bool live = false;
  uint32_t slot = 0;
  float4 mo = make_float4(0.0f, 0.0f, 0.0f, 0.0f), so = mo, q = mo;
  m3 local = {};
  {
    const ViewDesc& v = b.views[v_first];
    do {
      if (gid >= v.active) break;  // padding up to the view's next block boundary
      slot = __ldg(v.sh + (size_t)v.count * v.C + gid);
      if (slot >= v.count) break;  // out-of-range tail entries never draw
      mo = __ldg(v.means + slot);
      if (mo.w < 0.0f) break;  // empty slot (ProjectionStage.ts:408-410)
      if (GROUPED) {
        so = decode_scale_opacity(__ldg(v.shape + slot));
        q = decode_rotation(__ldg(v.rot + slot));
        local = local_covariance(so, q);
      }
      live = true;
    } while (false);
  }

  for (uint32_t vi = v_first; vi < v_end; ++vi) {
    const ViewDesc& v = b.views[vi];
    const uint32_t item = v.item_base + gid;
    const float vw = v.vw, vh = v.vh;
    float4 mo4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t cnt = 0, key = kInvisibleKey, nbox = 0;
    bool centre = false;
    Projected pr = {};
    float op = 0.0f, rx = 0.0f, ry = 0.0f, thr = 0.0f;
    float ddx = 0.0f, ddy = 0.0f, ddz = 0.0f;  // positionLocal - cameraLocal
    // Project and cull; a splat that survives gets its tile box.
    do {
      if (!live) break;
      const uint32_t obj = (uint32_t)mo.w;
      if (obj >= v.object_count) break;  // unwritten object rows are zero
      const float* ot = v.objects + 40 * (size_t)obj;
      if (!(__ldg(ot + 36) > 0.0f)) break;  // object visibility (:445-450)
      if (!GROUPED) {
        so = decode_scale_opacity(__ldg(v.shape + slot));
        q = decode_rotation(__ldg(v.rot + slot));
      }
      float mv[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) mv[i] = __ldg(ot + 16 + i);
      const float camx = __ldg(ot + 32), camy = __ldg(ot + 33), camz = __ldg(ot + 34);
      ddx = mo.x - camx; ddy = mo.y - camy; ddz = mo.z - camz;
      // view = modelView * (p, 1) (:479-482); the FP64 form evaluates it in
      // double so far-origin coordinates do not cancel against the translation.
      double vxd = 0.0, vyd = 0.0, vzd = 0.0;
      float vx, vy, vz;
      if (FP64) {
        vxd = (((double)mv[0] * mo.x + (double)mv[4] * mo.y) + (double)mv[8] * mo.z) + (double)mv[12];
        vyd = (((double)mv[1] * mo.x + (double)mv[5] * mo.y) + (double)mv[9] * mo.z) + (double)mv[13];
        vzd = (((double)mv[2] * mo.x + (double)mv[6] * mo.y) + (double)mv[10] * mo.z) + (double)mv[14];
        vx = (float)vxd; vy = (float)vyd; vz = (float)vzd;
      } else {
        vx = ((mv[0] * mo.x + mv[4] * mo.y) + mv[8] * mo.z) + mv[12] * 1.0f;
        vy = ((mv[1] * mo.x + mv[5] * mo.y) + mv[9] * mo.z) + mv[13] * 1.0f;
        vz = ((mv[2] * mo.x + mv[6] * mo.y) + mv[10] * mo.z) + mv[14] * 1.0f;
      }
      m3 l2v;
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) l2v.m[c][r] = mv[4 * c + r];
      const m3 cv = view_covariance(GROUPED ? local : local_covariance(so, q), l2v);
      float P[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) P[i] = v.P[i];
      pr = project({vx, vy, vz}, cv, P, vw, vh, v.vnear, v.vfar, o.filter);
      if (FP64) {
        // Near-singular in FP32 (tiny anti-aliasing factor, high condition
        // number, or rejected past the depth test): redo the chain in double.
        const float cond_num = (pr.cov_x + pr.cov_z) * (pr.cov_x + pr.cov_z);
        const bool redo = !pr.ok ? (-vz > v.vnear && -vz < v.vfar)
                                 : (pr.orig_det < 1e-2f * pr.det || !(cond_num <= 4e3f * pr.det));
        // The redo reads the model-view and projection rows from global memory
        // (the same values as mv and P), so neither array needs a stack copy.
        if (redo) pr = project_fp64(vxd, vyd, vzd, so, q, ot + 16, v.P, vw, vh, v.vnear, v.vfar, o.filter);
      }
      if (!pr.ok) break;
      op = clampf(so.w, 0.0f, 1.0f);
      if (o.antialias == 0u) op = op * sqrtf(clampf(pr.orig_det / pr.det, 0.0f, 1.0f));
      if (op < (float)(1.0 / 255.0) || op != op) break;
      thr = gsdm::logf_(op * 255.0f);
      const float ex = sqrtf((thr * 2.0f) * clampf(pr.cov_x, 1e-12f, 1e4f));
      const float ey = sqrtf((thr * 2.0f) * clampf(pr.cov_z, 1e-12f, 1e4f));
      rx = ceilf(ex);
      ry = ceilf(ey);
      if (rx <= 0.0f || ry <= 0.0f) break;
      const float bminx = pr.cx - rx, bminy = pr.cy - ry, bmaxx = pr.cx + rx, bmaxy = pr.cy + ry;
      if ((o.axis != 1u && (bmaxx < 0.0f || bminx >= vw)) || (o.axis != 2u && (bmaxy < 0.0f || bminy >= vh)))
        break;
      if (o.subpixel != 0u &&
          !subpixel_has_sample(pr.cx, pr.cy, pr.conic_x, pr.conic_y, pr.conic_z, thr, ex, ey, (uint32_t)vw,
                               (uint32_t)vh, o.axis)) {
        mo4 = make_float4(pr.cx, pr.cy, pr.depth, -1.0f);  // subpixel marker (:572-587)
        break;
      }
      const int tiles_x = (int)v.tiles_x, tiles_y = (int)v.tiles_y;
      const float mtx = (float)(tiles_x - 1), mty = (float)(tiles_y - 1);
      // Division by the tile side, a power of two: the product with its
      // reciprocal is the same correctly rounded value.
      const float fx0 = floorf(bminx * o.tile_inv), fy0 = floorf(bminy * o.tile_inv);
      const float fx1 = floorf(bmaxx * o.tile_inv), fy1 = floorf(bmaxy * o.tile_inv);
      int tminx = (int)clampf(fx0, 0.0f, mtx);
      int tminy = (int)clampf(fy0, 0.0f, mty);
      int tmaxx = (int)clampf(fx1, 0.0f, mtx);
      int tmaxy = (int)clampf(fy1, 0.0f, mty);
      if (o.axis == 1u) { tminx = 0; tmaxx = tiles_x - 1; }
      if (o.axis == 2u) { tminy = 0; tmaxy = tiles_y - 1; }
      const uint32_t bw = (uint32_t)(tmaxx - tminx + 1);
      nbox = bw * (uint32_t)(tmaxy - tminy + 1);
      // The tile holding the centre, when it is on screen, lies in the box
      // (the floors are monotone and rx, ry >= 1) and passes the reference's
      // tile test by its centre-inside path (tileContribution.ts:16-59): it
      // counts 1 without a test, and the warp walks the box's other tiles.
      const float fcx = floorf(pr.cx * o.tile_inv), fcy = floorf(pr.cy * o.tile_inv);
      centre = o.axis == 0u && fcx >= 0.0f && fcx <= mtx && fcy >= 0.0f && fcy <= mty;
      s_count.u[3][warp][lane] =
          centre ? ((uint32_t)fcy - (uint32_t)tminy) * bw + ((uint32_t)fcx - (uint32_t)tminx) : 0xffffffffu;
      s_count.f[0][warp][lane] = pr.cx; s_count.f[1][warp][lane] = pr.cy;
      s_count.f[2][warp][lane] = pr.conic_x; s_count.f[3][warp][lane] = pr.conic_y;
      s_count.f[4][warp][lane] = pr.conic_z; s_count.f[5][warp][lane] = thr;
      s_count.f[6][warp][lane] = rx; s_count.f[7][warp][lane] = ry;
      s_count.u[0][warp][lane] = (uint32_t)tminx; s_count.u[1][warp][lane] = (uint32_t)tminy;
      s_count.u[2][warp][lane] = bw;
    } while (false);
    // Tiles passing the tile test (projectionHelpers.ts:223-236), counted by the whole warp.
    cnt = count_tiles_warp(s_count, centre ? nbox - 1u : nbox, vw, vh, o.axis, o.tile_px) + (centre ? 1u : 0u);
    if (cnt > 0) {
      uint32_t co[16];
      load_sh(v.sh + (size_t)slot * v.C, v.degree, co);
      // viewDirection = normalize(positionLocal - cameraLocal) (:469), which
      // feeds only the colour: the reference's quotients for the EXACT form,
      // a reciprocal square root (2 ulp) for the fast forms' colour.
      const float dd2 = (ddx * ddx + ddy * ddy) + ddz * ddz;
      f3 vdir;
      if (FAST_SH) {
        const float r = rsqrtf(dd2);
        vdir = {ddx * r, ddy * r, ddz * r};
      } else {
        const float dlen = sqrtf(dd2);
        vdir = {ddx / dlen, ddy / dlen, ddz / dlen};
      }
      const f3 col = eval_sh_any<FAST_SH>(v.degree, co, vdir, s_snorm);
      mo4 = make_float4(pr.cx, pr.cy, pr.depth, op);
      conic_out[item] = make_float4(pr.conic_x, pr.conic_y, pr.conic_z, rx + ry * 512.0f);
      // Emission record: what the emission reads per depth rank, in one
      // 32-byte gather (layout in pass_common.cuh).
      erec_out[2 * (size_t)item] = make_float4(pr.cx, pr.cy, pr.conic_x, pr.conic_y);
      erec_out[2 * (size_t)item + 1] = make_float4(pr.conic_z, thr, rx + ry * 512.0f, 0.0f);
      color_out[item] = make_float4(col.x, col.y, col.z, __uint_as_float(slot ^ kActiveTag));
      if (rec_out) {
        // Packed raster record of the fast forms (layout in pass_common.cuh).
        const float log2op = __log2f(op);
        const __half2 rg = __floats2half2_rn(col.x, col.y);
        const __half2 bl = __floats2half2_rn(col.z, fminf(log2op, kLog2MaxAlpha));
        rec_out[2 * (size_t)item] = make_float4(pr.cx, pr.cy, -0.5f * kLog2e * pr.conic_x, -kLog2e * pr.conic_y);
        rec_out[2 * (size_t)item + 1] =
            make_float4(-0.5f * kLog2e * pr.conic_z, log2op, __uint_as_float(*reinterpret_cast<const uint32_t*>(&rg)),
                        __uint_as_float(*reinterpret_cast<const uint32_t*>(&bl)));
      }
      if (o.depth_mode == 0u) {
        key = __float_as_uint(pr.depth);  // visibility.ts:139
      } else {
        float t = clampf((pr.depth - v.vnear) / (v.vfar - v.vnear), 0.0f, 1.0f);
        key = (uint32_t)gsdm::round_even_small(t * 65535.0f);  // visibility.ts:140-144
      }
    }
    mean_out[item] = mo4;
    count_out[item] = cnt;
    key_out[item] = key;
  }
}

template <bool FAST_SH>
void launch_project_t(const BatchView& b, const PassOptions& o, float4* mean, float4* conic, float4* color,
                      uint32_t* counts, uint32_t* keys, float4* rec, float4* erec, cudaStream_t st) {
  const bool grouped = b.ngroups < b.nviews;
#define GS_PROJECT(F, G) \
  k_project<F, G, FAST_SH><<<b.total_blocks, kBlock, 0, st>>>(b, o, mean, conic, color, counts, keys, rec, erec)
  if (o.proj_fp64) {
    if (grouped) GS_PROJECT(true, true); else GS_PROJECT(true, false);
  } else {
    if (grouped) GS_PROJECT(false, true); else GS_PROJECT(false, false);
  }
#undef GS_PROJECT
}

// The fast raster forms (rec != null) take the fused-multiply-add SH colour;
// EXACT keeps the reference's order.
void launch_project(const BatchView& b, const PassOptions& o, float4* mean, float4* conic, float4* color,
                    uint32_t* counts, uint32_t* keys, float4* rec, float4* erec, cudaStream_t st) {
  if (b.total_blocks == 0) return;  // projection blocks over the view groups
  if (rec) launch_project_t<true>(b, o, mean, conic, color, counts, keys, rec, erec, st);
  else launch_project_t<false>(b, o, mean, conic, color, counts, keys, rec, erec, st);
}

// ---------------------------------------------------------------------------
// Chunked look-back scans (visibility compaction, ordered-count scan): a
// persistent grid of `chunks` blocks; chunk c (tickets give launch order) is a
// contiguous run of 256-item units, split into one contiguous slice per warp.
// Phase 1 reduces each warp's slice, warp 0 combines the warps and resolves
// the chunk's prefix by decoupled look-back (one chain step per chunk, not per
// 2048 items), and phase 2 walks the slice again writing every output with
// the warp's running offset. A unit is 8 rows of 32 consecutive items, so
// every load and store of a row is one coalesced 128-byte access.
constexpr uint32_t kUnit = 256;
constexpr uint32_t kUnitRows = kUnit / 32;
constexpr uint32_t kScanWarps = kBlock / 32;

__device__ __forceinline__ void chunk_units(uint32_t n, uint32_t chunks, uint32_t c, uint32_t* u0, uint32_t* u1) {
  const uint32_t units = (uint32_t)(((uint64_t)n + kUnit - 1) / kUnit);
  const uint32_t per = (units + chunks - 1) / chunks;
  *u0 = min(c * per, units);
  *u1 = min(*u0 + per, units);
}

__device__ __forceinline__ void warp_units(uint32_t u0, uint32_t u1, uint32_t warp, uint32_t* w0, uint32_t* w1) {
  const uint32_t m = u1 - u0, per = (m + kScanWarps - 1) / kScanWarps;
  *w0 = u0 + min(warp * per, m);
  *w1 = u0 + min((warp + 1) * per, m);
}

// Called by all 32 lanes of warp 0: combines the warps' sums in s_warp
// (replaced by each warp's exclusive base), publishes chunk c and looks back.
// Every lane gets the chunk's exclusive prefix and its total.
template <bool SAT>
__device__ __forceinline__ void chunk_publish(uint32_t* s_warp, unsigned long long* status, uint32_t c,
                                              uint32_t epoch, uint32_t limit, uint32_t* err, uint32_t* prefix_out,
                                              uint32_t* total_out) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wc = lane < kScanWarps ? s_warp[lane] : 0u;
  uint32_t incl = wc;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= (uint32_t)d) incl = SAT ? sat_add(y, incl) : y + incl;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, kScanWarps - 1);
  const uint32_t up = __shfl_up_sync(0xffffffffu, incl, 1);
  const uint32_t excl = lane ? up : 0u;
  unsigned long long* mine = status + c;
  uint32_t prefix = 0;
  if (c == 0) {
    if (lane == 0) st_release(mine, pack_status(epoch, kFlagInclusive, total));
  } else {
    if (lane == 0) st_release(mine, pack_status(epoch, kFlagAggregate, total));
    prefix = warp_lookback<SAT>(status, c, epoch, limit, err);
    if (lane == 0) st_release(mine, pack_status(epoch, kFlagInclusive, SAT ? sat_add(prefix, total) : prefix + total));
  }
  if (lane < kScanWarps) s_warp[lane] = SAT ? sat_add(prefix, excl) : prefix + excl;
  *prefix_out = prefix;
  *total_out = total;
}

// Visibility compaction (scan.ts:9-83 + visibility.ts:9-61). Writes
// visibleOffsets, the (depthKey, ordinal) records in ordinal order and the
// visible state.
__global__ void __launch_bounds__(kBlock) k_compact(const uint32_t* __restrict__ keys, uint32_t n,
                                                    uint32_t* __restrict__ vis_off, uint32_t* __restrict__ keys_out,
                                                    uint32_t* __restrict__ vals_out, Control* __restrict__ ctl,
                                                    unsigned long long* __restrict__ status, Epoch ep,
                                                    uint32_t chunks) {
  __shared__ uint32_t s_chunk;
  __shared__ uint32_t s_warp[kScanWarps];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) s_chunk = atomicAdd(&ctl->tickets[kTicketCompact], 1u);
  __syncthreads();
  const uint32_t c = s_chunk;
  uint32_t u0, u1;
  chunk_units(n, chunks, c, &u0, &u1);
  if (u0 >= u1 && !(n == 0 && c == 0)) return;  // chunks past the last item do nothing
  const bool last = (uint64_t)u1 * kUnit >= n;
  uint32_t w0, w1;
  warp_units(u0, u1, warp, &w0, &w1);
  const uint32_t lt = (1u << lane) - 1u;

  uint32_t cnt = 0;
  for (uint32_t u = w0; u < w1; ++u) {
    uint32_t k[kUnitRows];
#pragma unroll
    for (uint32_t j = 0; j < kUnitRows; ++j) {
      const uint32_t idx = u * kUnit + j * 32u + lane;
      k[j] = idx < n ? keys[idx] : kInvisibleKey;
    }
#pragma unroll
    for (uint32_t j = 0; j < kUnitRows; ++j) cnt += __popc(__ballot_sync(0xffffffffu, k[j] != kInvisibleKey));
  }
  if (lane == 0) s_warp[warp] = cnt;
  __syncthreads();
  if (warp == 0) {
    uint32_t prefix, total;
    chunk_publish<false>(s_warp, status, c, ep.get(), ep.limit(), &ctl->error, &prefix, &total);
    if (lane == 0 && last) {
      const uint32_t v = prefix + total;
      ctl->visible_state[0] = v;
      ctl->visible_state[1] = v;
      ctl->visible_state[2] = (v + 1023u) / 1024u;
      ctl->visible_state[3] = 0u;
    }
  }
  __syncthreads();

  uint32_t run = s_warp[warp];
  for (uint32_t u = w0; u < w1; ++u) {
    uint32_t k[kUnitRows];
#pragma unroll
    for (uint32_t j = 0; j < kUnitRows; ++j) {
      const uint32_t idx = u * kUnit + j * 32u + lane;
      k[j] = idx < n ? keys[idx] : kInvisibleKey;
    }
#pragma unroll
    for (uint32_t j = 0; j < kUnitRows; ++j) {
      const uint32_t idx = u * kUnit + j * 32u + lane;
      const bool vis = k[j] != kInvisibleKey;
      const uint32_t bal = __ballot_sync(0xffffffffu, vis);
      const uint32_t pos = run + __popc(bal & lt);
      if (idx < n) {
        vis_off[idx] = pos;
        if (vis) {
          keys_out[pos] = k[j];
          vals_out[pos] = idx;
        }
      }
      run += __popc(bal);
    }
  }
}

__global__ void k_epoch_begin(uint32_t* base) {
  // Leaves room for kEpochsPerFrame launches; status words are 30-bit epochs.
  const uint32_t next = (*base + kEpochsPerFrame) & ((1u << 30) - 1u);
  *base = next < kEpochsPerFrame ? kEpochsPerFrame : next;
}

void launch_epoch_begin(uint32_t* epoch_base, cudaStream_t st) { k_epoch_begin<<<1, 1, 0, st>>>(epoch_base); }

__global__ void k_skip_ticket(Control* ctl, uint32_t ticket) { ctl->tickets[ticket] += 1u; }

void launch_skip_ticket(Control* ctl, uint32_t ticket, cudaStream_t st) { k_skip_ticket<<<1, 1, 0, st>>>(ctl, ticket); }

uint32_t scan_chunks(uint32_t n_max, int sms) {
  const uint64_t units = ((uint64_t)n_max + kUnit - 1) / kUnit;
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(units, (uint64_t)kScanBlocksPerSm * (uint64_t)sms));
}

void launch_compact(const uint32_t* keys, uint32_t n, uint32_t* vis_off, uint32_t* keys_out, uint32_t* vals_out,
                    Control* ctl, unsigned long long* status, Epoch epoch, uint32_t chunks, cudaStream_t st) {
  k_compact<<<chunks, kBlock, 0, st>>>(keys, n, vis_off, keys_out, vals_out, ctl, status, epoch, chunks);
}

// Depth-ordered tile counts + saturating exclusive scan + prepare_dispatch +
// prepare_intersection_output (visibility.ts:63-76, scan.ts:9-99,
// intersections.ts:10-41,114-133) over the visible ranks. Phase 1 gathers
// each rank's tile count, writes it (the ordered counts) and reduces; phase 2
// re-reads the ordered counts and writes the saturating offsets.
__global__ void __launch_bounds__(kBlock) k_scan_counts(const uint32_t* __restrict__ ids,
                                                        const uint32_t* __restrict__ tile_counts,
                                                        uint32_t* __restrict__ ordered,
                                                        uint32_t* __restrict__ offsets, Control* __restrict__ ctl,
                                                        unsigned long long* __restrict__ status, Epoch ep,
                                                        uint32_t capacity, const uint32_t* __restrict__ frame_params,
                                                        uint32_t* __restrict__ output_state, uint32_t chunks) {
  __shared__ uint32_t s_chunk;
  __shared__ uint32_t s_warp[kScanWarps];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) s_chunk = atomicAdd(&ctl->tickets[kTicketScan], 1u);
  __syncthreads();
  const uint32_t n = ctl->visible_state[0];
  const uint32_t c = s_chunk;
  uint32_t u0, u1;
  chunk_units(n, chunks, c, &u0, &u1);
  if (u0 >= u1 && !(n == 0 && c == 0)) return;
  const bool last = (uint64_t)u1 * kUnit >= n;
  uint32_t w0, w1;
  warp_units(u0, u1, warp, &w0, &w1);

  uint32_t sum = 0;
  for (uint32_t u = w0; u < w1; ++u) {
    uint32_t id[kUnitRows];
#pragma unroll
    for (uint32_t j = 0; j < kUnitRows; ++j) {
      const uint32_t r = u * kUnit + j * 32u + lane;
      id[j] = r < n ? ids[r] : 0u;
    }
#pragma unroll
    for (uint32_t j = 0; j < kUnitRows; ++j) {
      const uint32_t r = u * kUnit + j * 32u + lane;
      if (r < n) {
        const uint32_t cnt = __ldg(tile_counts + id[j]);
        ordered[r] = cnt;
        sum = sat_add(sum, cnt);
      }
    }
  }
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) sum = sat_add(sum, __shfl_xor_sync(0xffffffffu, sum, d));
  if (lane == 0) s_warp[warp] = sum;
  __syncthreads();
  if (warp == 0) {
    uint32_t prefix, total;
    chunk_publish<true>(s_warp, status, c, ep.get(), ep.limit(), &ctl->error, &prefix, &total);
    if (lane == 0 && last) {
      const uint32_t all = sat_add(prefix, total);
      const bool overflow = all > capacity;
      const uint32_t count = overflow ? 0u : all;
      ctl->state[0] = count;
      ctl->state[1] = all;
      ctl->state[2] = (uint32_t)(((uint64_t)count + 1023u) / 1024u);
      ctl->state[3] = overflow ? 1u : 0u;
      const uint32_t attempt = frame_params[0];
      const uint32_t last_version = frame_params[1] ? 0u : output_state[1];
      output_state[0] = attempt;
      output_state[1] = overflow ? last_version : attempt;
      output_state[2] = all;
      output_state[3] = overflow ? 1u : 0u;
    }
  }
  __syncthreads();

  uint32_t run = s_warp[warp];
  for (uint32_t u = w0; u < w1; ++u) {
    uint32_t cnt[kUnitRows];
#pragma unroll
    for (uint32_t j = 0; j < kUnitRows; ++j) {
      const uint32_t r = u * kUnit + j * 32u + lane;
      cnt[j] = r < n ? ordered[r] : 0u;  // written by this thread in phase 1
    }
#pragma unroll
    for (uint32_t j = 0; j < kUnitRows; ++j) {
      const uint32_t r = u * kUnit + j * 32u + lane;
      uint32_t incl = cnt[j];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (uint32_t)d) incl = sat_add(y, incl);
      }
      const uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
      if (r < n) offsets[r] = sat_add(run, lane ? excl : 0u);
      run = sat_add(run, __shfl_sync(0xffffffffu, incl, 31));
    }
  }
}

void launch_scan_counts(const uint32_t* ids, const uint32_t* tile_counts, uint32_t* ordered, uint32_t* offsets,
                        Control* ctl, unsigned long long* status, Epoch epoch, uint32_t capacity,
                        const uint32_t* frame_params, uint32_t* output_state, uint32_t chunks, cudaStream_t st) {
  k_scan_counts<<<chunks, kBlock, 0, st>>>(ids, tile_counts, ordered, offsets, ctl, status, epoch, capacity,
                                           frame_params, output_state, chunks);
}

// ---------------------------------------------------------------------------
// Intersection emission (intersections.ts:43-111): per depth rank, one
// (tile, item) record for every tile the splat contributes to, written at the
// rank's scanned offset; sentinel padding if fewer hits than reserved. Tile
// ids are global over the batch (the view's tile_base + local id; the
// sentinel is the batch's tile total).
//
// Warp-cooperative: a warp owns 32 consecutive depth ranks and spreads the
// union of their bounding-box tiles over its lanes, 32 box tiles per round,
// so one wide splat no longer idles the other 31 lanes. Each lane finds the
// rank owning its box tile by a binary search over the warp's inclusive box
// counts, runs the reference's tile test, and places a hit after the owner's
// earlier hits (owner's running count + hits of lower lanes with the same
// owner this round). A splat's records thus fill its reserved range in
// row-major box order, the order of the per-splat loop; the record set per
// splat is what the stable tile sort sees, so the sorted result is the same.
constexpr int kEmitWarps = kBlock / 32;

struct EmitShared {
  float f[10][kEmitWarps][32];     // cx, cy, conic a, b, c, threshold, rx, ry, view width, height
  uint32_t u[9][kEmitWarps][32];   // tminx, tminy, box width, tiles_x, tile_base, base, reserved, item,
                                   // first box tile of the warp's walk
  uint32_t own[kEmitWarps][32];    // lane owning the k-th segment of the round
  uint32_t filled[kEmitWarps][32]; // records placed so far per rank
};

// One group of kBlock depth ranks (32 per warp): stage each lane's box and
// tile-test inputs for its warp, walk the union of the warp's boxes 32 box
// tiles per round, place hits after the owner's earlier hits, pad with
// sentinels. The lane's rank data were loaded by the caller.
__device__ __forceinline__ void emit_group(EmitShared& sm, bool live, uint32_t g, float4 e0, float4 e1,
                                           uint32_t reserved, uint32_t base_off, const BatchView& bv,
                                           const PassOptions& o, uint32_t capacity, uint32_t* __restrict__ tile_keys,
                                           uint32_t* __restrict__ tile_vals) {
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t sentinel = bv.total_tiles;
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t nbox = 0;
  if (live) {
    const ViewDesc& v = bv.views[find_view(bv.item_base, bv.nviews, g)];
    // Emission record: (cx, cy, conic a, b), (conic c, threshold, rx + 512 ry, 0).
    const float4 m = make_float4(e0.x, e0.y, 0.0f, 0.0f), c = make_float4(e0.z, e0.w, e1.x, 0.0f);
    const uint32_t packed = (uint32_t)e1.z;
    const float rx = (float)(packed % 512u), ry = (float)(packed / 512u);
    const float thr = e1.y;  // log(opacity * 255), computed by the projection
    const int tiles_x = (int)v.tiles_x, tiles_y = (int)v.tiles_y;
    const float mtx = (float)(tiles_x - 1), mty = (float)(tiles_y - 1);
    int tminx = (int)clampf(floorf((m.x - rx) * o.tile_inv), 0.0f, mtx);
    int tminy = (int)clampf(floorf((m.y - ry) * o.tile_inv), 0.0f, mty);
    int tmaxx = (int)clampf(floorf((m.x + rx) * o.tile_inv), 0.0f, mtx);
    int tmaxy = (int)clampf(floorf((m.y + ry) * o.tile_inv), 0.0f, mty);
    if (o.axis == 1u) { tminx = 0; tmaxx = tiles_x - 1; }
    if (o.axis == 2u) { tminy = 0; tmaxy = tiles_y - 1; }
    const uint32_t bw = (uint32_t)(tmaxx - tminx + 1);
    // A rank with nothing reserved emits nothing; its box takes no rounds.
    nbox = reserved ? bw * (uint32_t)(tmaxy - tminy + 1) : 0u;
    sm.f[0][warp][lane] = m.x; sm.f[1][warp][lane] = m.y;
    sm.f[2][warp][lane] = c.x; sm.f[3][warp][lane] = c.y; sm.f[4][warp][lane] = c.z;
    sm.f[5][warp][lane] = thr; sm.f[6][warp][lane] = rx; sm.f[7][warp][lane] = ry;
    sm.f[8][warp][lane] = v.vw; sm.f[9][warp][lane] = v.vh;
    sm.u[0][warp][lane] = (uint32_t)tminx; sm.u[1][warp][lane] = (uint32_t)tminy; sm.u[2][warp][lane] = bw;
    sm.u[3][warp][lane] = (uint32_t)tiles_x; sm.u[4][warp][lane] = v.tile_base;
    sm.u[5][warp][lane] = base_off; sm.u[6][warp][lane] = reserved; sm.u[7][warp][lane] = g;
  }
  const uint32_t le = lt | (1u << lane);
  sm.filled[warp][lane] = 0u;
  uint32_t filled = 0;
  // A splat whose every box tile passed the projection's count (reserved ==
  // nbox) emits its whole box: those boxes are walked first without the tile
  // test, the others after it with the test. Each splat is walked once, so
  // its records keep row-major box order. Wide boxes (kWideBox tiles or more)
  // are walked afterwards by the whole warp, one box at a time.
  const bool full = reserved == nbox;
  const bool wide = nbox >= kWideBox;
#pragma unroll 1
  for (int pass = 0; pass < 2; ++pass) {
    const uint32_t nb = !wide && (pass == 0) == full ? nbox : 0u;
    uint32_t incl = nb;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= (uint32_t)d) incl += y;
    }
    const uint32_t excl = incl - nb;
    sm.u[8][warp][lane] = excl;
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);

    // Rounds of 32 box tiles. The boxes lie end to end in lane order, so a
    // round is a run of segments, one per owning lane: a lane finds its
    // segment from the OR of the segment starts and the segment's owner from
    // a table the owners wrote; each owner adds its hits under its own mask.
    for (uint32_t j0 = 0; j0 < total; j0 += 32) {
      const uint32_t lo = max(excl, j0), hi = min(incl, j0 + 32u);
      const bool seg = lo < hi;
      const uint32_t starts = __reduce_or_sync(0xffffffffu, seg ? 1u << (lo - j0) : 0u);
      const uint32_t owners = __ballot_sync(0xffffffffu, seg);
      if (seg) sm.own[warp][__popc(owners & lt)] = lane;
      __syncwarp();
      const uint32_t j = j0 + lane;
      const bool valid = j < total;
      uint32_t owner = 0, seg_start = 0;
      bool hit = false;
      uint32_t t = 0;
      if (valid) {
        const uint32_t mine = starts & le;
        owner = sm.own[warp][__popc(mine) - 1u];
        seg_start = 31u - (uint32_t)__clz(mine);
        const uint32_t bw = sm.u[2][warp][owner];
        const uint32_t kk = j - sm.u[8][warp][owner];
        const uint32_t by = kk / bw, bx = kk - by * bw;
        const int tx = (int)(sm.u[0][warp][owner] + bx), ty = (int)(sm.u[1][warp][owner] + by);
        hit = pass == 0 ||
              boundary_tile_hit(sm.f[0][warp][owner], sm.f[1][warp][owner], sm.f[2][warp][owner],
                                sm.f[3][warp][owner], sm.f[4][warp][owner], sm.f[5][warp][owner],
                                sm.f[6][warp][owner], sm.f[7][warp][owner], tx, ty, sm.f[8][warp][owner],
                                sm.f[9][warp][owner], o.axis, o.tile_px);
        t = sm.u[4][warp][owner] + (uint32_t)ty * sm.u[3][warp][owner] + (uint32_t)tx;
      }
      const uint32_t hits = __ballot_sync(0xffffffffu, hit);
      if (hit) {
        // After the owner's earlier hits: those of past rounds, then those of
        // this round below this lane within the owner's segment.
        const uint32_t local = sm.filled[warp][owner] + __popc(hits & lt & ~((1u << seg_start) - 1u));
        const uint32_t base = sm.u[5][warp][owner];
        if (local < sm.u[6][warp][owner] && base + local < capacity) {
          tile_keys[base + local] = t;
          tile_vals[base + local] = sm.u[7][warp][owner];
        }
      }
      __syncwarp();  // every read of filled, the owner table and the walk bases is done
      if (seg) {
        filled += __popc(hits & bit_range(lo - j0, hi - j0));
        sm.filled[warp][lane] = filled;
      }
    }
    __syncwarp();
  }

  // Wide boxes: the warp walks one box 32 tiles at a time, in row-major box
  // order, each hit after the box's earlier hits (no per-tile owner lookup).
  uint32_t wide_lanes = __ballot_sync(0xffffffffu, wide);
  while (wide_lanes) {
    const uint32_t w = (uint32_t)__ffs(wide_lanes) - 1u;
    wide_lanes &= wide_lanes - 1u;
    // The owner's parameters are read from the warp's table at each step
    // (broadcast loads) rather than held in registers across the walk.
    const volatile float(*vf)[kEmitWarps][32] = sm.f;
    const volatile uint32_t(*vu)[kEmitWarps][32] = sm.u;
    const uint32_t wn = __shfl_sync(0xffffffffu, nbox, w);
    const uint32_t wres = vu[6][warp][w];
    const bool wfull = wres == wn;
    uint32_t wfilled = 0;
    for (uint32_t k0 = 0; k0 < wn; k0 += 32) {
      const uint32_t k = k0 + lane;
      bool hit = false;
      uint32_t t = 0;
      if (k < wn) {
        const uint32_t wbw = vu[2][warp][w];
        const uint32_t by = k / wbw, bx = k - by * wbw;
        const int tx = (int)(vu[0][warp][w] + bx), ty = (int)(vu[1][warp][w] + by);
        hit = wfull || boundary_tile_hit(vf[0][warp][w], vf[1][warp][w], vf[2][warp][w], vf[3][warp][w],
                                         vf[4][warp][w], vf[5][warp][w], vf[6][warp][w], vf[7][warp][w], tx, ty,
                                         vf[8][warp][w], vf[9][warp][w], o.axis, o.tile_px);
        t = vu[4][warp][w] + (uint32_t)ty * vu[3][warp][w] + (uint32_t)tx;
      }
      const uint32_t hits = __ballot_sync(0xffffffffu, hit);
      if (hit) {
        const uint32_t local = wfilled + __popc(hits & lt);
        const uint32_t wbase = vu[5][warp][w];
        if (local < wres && wbase + local < capacity) {
          tile_keys[wbase + local] = t;
          tile_vals[wbase + local] = vu[7][warp][w];
        }
      }
      wfilled += __popc(hits);
    }
    if (lane == w) filled = wfilled;
  }

  // Sentinel padding for reserved slots without a hit.
  if (live) {
    for (uint32_t pad = filled; pad < reserved; ++pad)
      if (base_off + pad < capacity) {
        tile_keys[base_off + pad] = sentinel;
        tile_vals[base_off + pad] = g;
      }
  }
  __syncwarp();  // the warp's tables are rewritten by the next group
}

// A block takes G groups of kBlock consecutive depth ranks and issues every
// group's loads (ids, reserved counts, offsets, then the gathered mean and
// conic) before working through the groups, so the gather latency of later
// groups overlaps the earlier groups' work. Two groups pay off on large
// launches (many blocks in flight anyway); one keeps small launches wide.
constexpr uint32_t kEmitTwoGroupsFrom = 1u << 23;  // ranks per launch

template <int G>
__global__ void __launch_bounds__(kBlock) k_emit(const uint32_t* __restrict__ ids, const float4* __restrict__ erec,
                                                 const uint32_t* __restrict__ ordered,
                                                 const uint32_t* __restrict__ offsets, BatchView bv, PassOptions o,
                                                 Control* __restrict__ ctl, uint32_t capacity,
                                                 uint32_t* __restrict__ tile_keys, uint32_t* __restrict__ tile_vals) {
  if (ctl->state[3] != 0u) return;  // overflow: emission dispatch is zero
  __shared__ EmitShared sm;
  const uint32_t tid = threadIdx.x;
  const uint32_t n = ctl->visible_state[0];
  const uint32_t first = blockIdx.x * kBlock * G;
  if (first >= n) return;  // whole block past the visible count
  uint32_t g[G], res[G], off[G];
  float4 e0[G], e1[G];
#pragma unroll
  for (int h = 0; h < G; ++h) {
    const uint32_t r = first + (uint32_t)h * kBlock + tid;
    g[h] = 0u; res[h] = 0u; off[h] = 0u;
    if (r < n) {
      g[h] = ids[r];
      res[h] = ordered[r];
      off[h] = offsets[r];
    }
  }
#pragma unroll
  for (int h = 0; h < G; ++h) {
    const uint32_t r = first + (uint32_t)h * kBlock + tid;
    e0[h] = e1[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (r < n) {
      e0[h] = __ldg(erec + 2 * (size_t)g[h]);
      e1[h] = __ldg(erec + 2 * (size_t)g[h] + 1);
    }
  }
#pragma unroll
  for (int h = 0; h < G; ++h) {
    const uint32_t r = first + (uint32_t)h * kBlock + tid;
    emit_group(sm, r < n, g[h], e0[h], e1[h], res[h], off[h], bv, o, capacity, tile_keys, tile_vals);
  }
}

void launch_emit(const uint32_t* ids, uint32_t n_max, const float4* erec, const uint32_t* ordered,
                 const uint32_t* offsets, const BatchView& b, const PassOptions& o, Control* ctl, uint32_t capacity,
                 uint32_t* tile_keys, uint32_t* tile_vals, cudaStream_t st) {
  if (n_max == 0) return;
  if (n_max >= kEmitTwoGroupsFrom) {
    const uint32_t grid = (n_max + 2 * kBlock - 1) / (2 * kBlock);
    k_emit<2><<<grid, kBlock, 0, st>>>(ids, erec, ordered, offsets, b, o, ctl, capacity, tile_keys,
                                       tile_vals);
  } else {
    const uint32_t grid = (n_max + kBlock - 1) / kBlock;
    k_emit<1><<<grid, kBlock, 0, st>>>(ids, erec, ordered, offsets, b, o, ctl, capacity, tile_keys,
                                       tile_vals);
  }
}

// ---------------------------------------------------------------------------
// Tile ranges (tileOffsets.ts:4-128): offsets[t] = first sorted index with
// tile >= t, i.e. the reference's boundary detection followed by its
// suffix-min fill, written directly (offsets[T] = first sentinel or count).
__global__ void __launch_bounds__(kBlock) k_tile_ranges(const uint32_t* __restrict__ keys,
                                                        const Control* __restrict__ ctl, uint32_t ntile,
                                                        uint32_t* __restrict__ off) {
  // Each thread owns 8 consecutive boundaries i in [i0, i0 + 8), reading the
  // keys with two 16-byte loads (i0 is a multiple of 8).
  const uint32_t n = ctl->state[0];
  const uint32_t i0 = (blockIdx.x * kBlock + threadIdx.x) * 8u;
  if (i0 > n) return;
  uint32_t k[9];  // k[0] = keys[i0 - 1], k[1 + j] = keys[i0 + j]
  k[0] = i0 ? keys[i0 - 1] : 0u;
  if (i0 + 8u <= n) {
    const uint4 a = *reinterpret_cast<const uint4*>(keys + i0);
    const uint4 b = *reinterpret_cast<const uint4*>(keys + i0 + 4);
    k[1] = a.x; k[2] = a.y; k[3] = a.z; k[4] = a.w; k[5] = b.x; k[6] = b.y; k[7] = b.z; k[8] = b.w;
  } else {
#pragma unroll
    for (uint32_t j = 0; j < 8u; ++j) k[1 + j] = i0 + j < n ? keys[i0 + j] : 0u;
  }
#pragma unroll
  for (uint32_t j = 0; j < 8u; ++j) {
    const uint32_t i = i0 + j;
    if (i > n) break;
    const uint32_t lo = i == 0 ? 0u : k[j] + 1u;
    const uint32_t hi = i == n ? ntile : min(k[1 + j], ntile);
    for (uint32_t t = lo; t <= hi; ++t) off[t] = i;
  }
}

void launch_tile_ranges(const uint32_t* keys, Control* ctl, uint32_t ntile, uint32_t n_max, uint32_t* offsets,
                        cudaStream_t st) {
  const uint32_t grid = (uint32_t)(((uint64_t)n_max + 1 + 8ull * kBlock - 1) / (8ull * kBlock));
  k_tile_ranges<<<grid, kBlock, 0, st>>>(keys, ctl, ntile, offsets);
}

// ---------------------------------------------------------------------------
// Profiling diagnostics (ProfileDiagnosticsStage.ts:22-116).
//
// profileSubpixelCoverageWGSL (kernels/profileDiagnostics.ts:8-64): a
// projected splat counts when the projection marked it subpixel (mean.w < 0),
// or when its alpha-support box is at most one pixel in both dimensions and
// holds no pixel centre inside the support. Counted on the device instead of
// a per-splat flag buffer read back.
__global__ void __launch_bounds__(kBlock) k_zero_pixel(const float4* __restrict__ mean,
                                                       const float4* __restrict__ conic, BatchView bv,
                                                       uint32_t n, uint32_t* __restrict__ count) {
  const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
  uint32_t flag = 0;
  if (i < n) {
    const float4 m = mean[i];
    if (m.w < 0.0f) {
      flag = 1u;
    } else if (m.w > 0.0f) {
      const float4 c = conic[i];
      const float det = c.x * c.z - c.y * c.y;
      const float thr = gsdm::logf_(m.w * 255.0f);
      if (det > 1e-12f && thr > 0.0f) {
        const float s00 = c.z / det, s11 = c.x / det;
        const float ex = sqrtf(maxf((2.0f * thr) * s00, 0.0f)), ey = sqrtf(maxf((2.0f * thr) * s11, 0.0f));
        if (!(ex * 2.0f > 1.0f || ey * 2.0f > 1.0f)) {
          const ViewDesc& v = bv.views[find_view(bv.item_base, bv.nviews, i)];
          const int W = (int)v.vw, H = (int)v.vh;
          const int x0 = max((int)ceilf((m.x - ex) - 0.5f), 0), y0 = max((int)ceilf((m.y - ey) - 0.5f), 0);
          const int x1 = min((int)floorf((m.x + ex) - 0.5f), W - 1), y1 = min((int)floorf((m.y + ey) - 0.5f), H - 1);
          bool has = false;
          for (int py = y0; py <= y1; ++py)
            for (int px = x0; px <= x1; ++px) {
              const float dx = ((float)px + 0.5f) - m.x, dy = ((float)py + 0.5f) - m.y;
              const float sigma = 0.5f * ((c.x * dx * dx + 2.0f * c.y * dx * dy) + c.z * dy * dy);
              if (sigma <= thr) has = true;
            }
          flag = has ? 0u : 1u;
        }
      }
    }
  }
  const uint32_t warp_sum = __popc(__ballot_sync(0xffffffffu, flag != 0u));
  if ((threadIdx.x & 31u) == 0u && warp_sum) atomicAdd(count, warp_sum);
}

// Tile loads (utils/profileStats.ts:9-114): sums, maxima and threshold counts
// over offsets[t + 1] - offsets[t], the same for the loads capped at each of
// up to four caps, and a histogram of the loads (bin 65535 collects larger
// ones) from which the host reads the median and percentiles.
__global__ void __launch_bounds__(kBlock) k_tile_loads(const uint32_t* __restrict__ off, uint32_t ntile,
                                                       uint4 caps, TileLoadSums* __restrict__ out,
                                                       uint32_t* __restrict__ hist) {
  const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
  if (t >= ntile) return;
  const uint32_t load = off[t + 1] > off[t] ? off[t + 1] - off[t] : 0u;
  atomicAdd(&out->total, (unsigned long long)load);
  atomicMax(&out->max, load);
  if (load > 256u) atomicAdd(&out->over[0], 1u);
  if (load > 512u) atomicAdd(&out->over[1], 1u);
  if (load > 1024u) atomicAdd(&out->over[2], 1u);
  if (load > 2048u) atomicAdd(&out->over[3], 1u);
  const uint32_t batches = (load + 255u) / 256u;
  atomicAdd(&out->batches, (unsigned long long)batches);
  atomicMax(&out->max_batches, batches);
  atomicAdd(&hist[min(load, 65535u)], 1u);
  const uint32_t cap[4] = {caps.x, caps.y, caps.z, caps.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (cap[k] == 0u) continue;
    const uint32_t r = min(load, cap[k]), d = load - r;
    atomicAdd(&out->cap_rasterized[k], (unsigned long long)r);
    if (d) {
      atomicAdd(&out->cap_dropped[k], (unsigned long long)d);
      atomicAdd(&out->cap_affected[k], 1u);
    }
    const uint32_t b = (r + 255u) / 256u;
    atomicAdd(&out->cap_batches[k], (unsigned long long)b);
    atomicMax(&out->cap_max_batches[k], b);
  }
}

void launch_profile(const float4* mean, const float4* conic, const BatchView& b, uint32_t n,
                    const uint32_t* tile_offsets, uint32_t ntile, const uint32_t caps[4], TileLoadSums* sums,
                    uint32_t* hist, uint32_t* zero_count, cudaStream_t st) {
  if (n) k_zero_pixel<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(mean, conic, b, n, zero_count);
  if (ntile)
    k_tile_loads<<<(ntile + kBlock - 1) / kBlock, kBlock, 0, st>>>(tile_offsets, ntile,
                                                                  make_uint4(caps[0], caps[1], caps[2], caps[3]),
                                                                  sums, hist);
}

// ---------------------------------------------------------------------------
void launch_raster_exact(const uint32_t* tile_offsets, const uint32_t* order, const uint32_t* ids,
                         const float4* mean, const float4* conic, const float4* color, const BatchView& b,
                         const PassOptions& o, Control* ctl, bool stats, cudaStream_t st) {
  launch_raster_policy<ExactMath>(tile_offsets, order, ids, mean, conic, color, b, o, ctl, stats, st);
}

}  // namespace gs
