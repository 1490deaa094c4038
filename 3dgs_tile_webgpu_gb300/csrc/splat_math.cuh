// Per-splat projection and tile-test arithmetic for the CUDA pass.
//
// Restates, in registers, the reference's WGSL/TSL formulas:
//   decode            src/renderer/kernels/compactGaussians.ts:2-19
//   view covariance   src/renderer/kernels/projectionHelpers.ts:4-35
//   projection result projectionHelpers.ts:38-83
//   perspective       projectionHelpers.ts:86-96
//   validity          projectionHelpers.ts:99-116
//   SH rgb8e8         projectionHelpers.ts:118-179
//   subpixel test     projectionHelpers.ts:185-221
//   tile/ellipse test src/renderer/kernels/tileContribution.ts:16-59,84-114
//
// Integer outputs (tile counts, tile ids, depth keys) must be bit-identical to
// the CPU restatement, so every expression keeps the reference's evaluation
// order (left-to-right, no reassociation) and this header is only compiled in
// translation units built with --fmad=false. Transcendentals come from
// detmath.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "detmath.h"

namespace gs {

constexpr uint32_t kActiveTag = 0x3f800000u;  // src/renderer/pipeline/activeSlots.ts:4
constexpr uint32_t kInvisibleKey = 0xffffffffu;

struct f2 { float x, y; };
struct f3 { float x, y, z; };

__device__ __forceinline__ float clampf(float x, float lo, float hi) {
  float y = x < lo ? lo : x;
  return y > hi ? hi : y;
}
__device__ __forceinline__ float maxf(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float absf(float a) { return a < 0.0f ? -a : a; }
__device__ __forceinline__ bool finitef(float v) { return v == v && absf(v) <= 3.402823e+38f; }

// Column-major 3x3 held as nine registers: m[c][r].
struct m3 { float m[3][3]; };

__device__ __forceinline__ m3 mul33(const m3& a, const m3& b) {
  m3 o;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      float s = a.m[0][r] * b.m[c][0];
      s = s + a.m[1][r] * b.m[c][1];
      s = s + a.m[2][r] * b.m[c][2];
      o.m[c][r] = s;
    }
  return o;
}
__device__ __forceinline__ m3 transpose33(const m3& a) {
  m3 o;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) o.m[c][r] = a.m[r][c];
  return o;
}
__device__ __forceinline__ f3 mul3v(const m3& a, f3 v) {
  f3 o;
  float* op = &o.x;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    float s = a.m[0][r] * v.x;
    s = s + a.m[1][r] * v.y;
    s = s + a.m[2][r] * v.z;
    op[r] = s;
  }
  return o;
}
__device__ __forceinline__ float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

// compactGaussians.ts:2-7
__device__ __forceinline__ float4 decode_scale_opacity(uint2 p) {
  float sx = gsdm::half_bits_to_float(p.x & 0xffffu);
  float sy = gsdm::half_bits_to_float(p.x >> 16);
  float sz = gsdm::half_bits_to_float(p.y & 0xffffu);
  float a = gsdm::half_bits_to_float(p.y >> 16);
  return make_float4(gsdm::expf_(sx), gsdm::expf_(sy), gsdm::expf_(sz), a);
}

// compactGaussians.ts:10-19
__device__ __forceinline__ float4 decode_rotation(uint32_t packed) {
  float px = (((float)(packed & 1023u) / 1023.0f) * 2.0f) - 1.0f;
  float py = (((float)((packed >> 10) & 1023u) / 1023.0f) * 2.0f) - 1.0f;
  float z = (1.0f - absf(px)) - absf(py);
  float t = maxf(-z, 0.0f);
  float x = px >= 0.0f ? px - t : px + t;
  float y = py >= 0.0f ? py - t : py + t;
  float len = sqrtf((x * x + y * y) + z * z);
  float ax = x / len, ay = y / len, az = z / len;
  float half = ((float)(packed >> 20) / 4095.0f) * 1.5707963267948966f;
  float s = gsdm::sinf_(half);
  return make_float4(ax * s, ay * s, az * s, gsdm::cosf_(half));
}

// projectionHelpers.ts:4-35, first half: the object-space 3D covariance
// R S^2 R^T, which depends on the splat alone (shared by every view of it).
__device__ __forceinline__ m3 local_covariance(float4 so, float4 q_in) {
  float sx = maxf(so.x, 1e-7f), sy = maxf(so.y, 1e-7f), sz = maxf(so.z, 1e-7f);
  float d = ((q_in.x * q_in.x + q_in.y * q_in.y) + q_in.z * q_in.z) + q_in.w * q_in.w;
  float len = sqrtf(d);
  float qx = q_in.x / len, qy = q_in.y / len, qz = q_in.z / len, qw = q_in.w / len;
  float xx = qx * qx, yy = qy * qy, zz = qz * qz;
  float xy = qx * qy, xz = qx * qz, yz = qy * qz;
  float xw = qx * qw, yw = qy * qw, zw = qz * qw;
  m3 rot;
  rot.m[0][0] = 1.0f - 2.0f * (yy + zz); rot.m[0][1] = 2.0f * (xy + zw); rot.m[0][2] = 2.0f * (xz - yw);
  rot.m[1][0] = 2.0f * (xy - zw); rot.m[1][1] = 1.0f - 2.0f * (xx + zz); rot.m[1][2] = 2.0f * (yz + xw);
  rot.m[2][0] = 2.0f * (xz + yw); rot.m[2][1] = 2.0f * (yz - xw); rot.m[2][2] = 1.0f - 2.0f * (xx + yy);
  m3 sc;
  sc.m[0][0] = sx * sx; sc.m[0][1] = 0.0f; sc.m[0][2] = 0.0f;
  sc.m[1][0] = 0.0f; sc.m[1][1] = sy * sy; sc.m[1][2] = 0.0f;
  sc.m[2][0] = 0.0f; sc.m[2][1] = 0.0f; sc.m[2][2] = sz * sz;
  return mul33(mul33(rot, sc), transpose33(rot));
}

// projectionHelpers.ts:4-35, second half: L (R S^2 R^T) L^T with L the
// model-view's upper 3x3.
__device__ __forceinline__ m3 view_covariance(const m3& local, const m3& l2v) {
  return mul33(mul33(l2v, local), transpose33(l2v));
}

struct Projected {
  bool ok;
  float cx, cy, depth;
  float conic_x, conic_y, conic_z;
  float cov_x, cov_z;
  float det, orig_det;
};

// projectionHelpers.ts:38-96 and the validity test :99-116.
__device__ __forceinline__ Projected project(f3 view, const m3& cv, const float* P, float vw, float vh,
                                             float vnear, float vfar, float filter) {
  Projected o;
  o.ok = false;
  float depth = -view.z;
  if (!(depth > vnear && depth < vfar)) return o;
  // clip = P * (view, 1): rows 0, 1, 3 are needed.
  float clip_x = ((P[0] * view.x + P[4] * view.y) + P[8] * view.z) + P[12] * 1.0f;
  float clip_y = ((P[1] * view.x + P[5] * view.y) + P[9] * view.z) + P[13] * 1.0f;
  float clip_w = ((P[3] * view.x + P[7] * view.y) + P[11] * view.z) + P[15] * 1.0f;
  if (clip_w <= 0.0f) return o;
  float ndcx = clip_x / clip_w, ndcy = clip_y / clip_w;
  float cx = (ndcx * 0.5f + 0.5f) * vw;
  float cy = (0.5f - ndcy * 0.5f) * vh;
  float fx = (0.5f * vw) * P[0];
  float fy = (0.5f * vh) * P[5];
  float inv = 1.0f / depth;
  f3 j0 = {fx * inv, 0.0f, ((fx * view.x) * inv) * inv};
  float nfy = -fy;
  f3 j1 = {0.0f, nfy * inv, ((nfy * view.y) * inv) * inv};
  float c_x = dot3(j0, mul3v(cv, j0));
  float c_y = dot3(j0, mul3v(cv, j1));
  float c_z = dot3(j1, mul3v(cv, j1));
  // gaussian_projection_result
  float orig_det = maxf(c_x * c_z - c_y * c_y, 0.0f);
  float s00 = c_x + filter, s01 = c_y, s11 = c_z + filter;
  if (!(finitef(s00) && finitef(s01) && finitef(s11))) return o;
  float mid = 0.5f * (s00 + s11);
  float rad = sqrtf((0.25f * (s00 - s11)) * (s00 - s11) + s01 * s01);
  float lmin = clampf(mid - rad, 1e-6f, 1e4f);
  float lmax = clampf(mid + rad, 1e-6f, 1e4f);
  float theta = 0.5f * gsdm::atan2f_(2.0f * s01, s00 - s11);
  float cs = gsdm::cosf_(theta), sn = gsdm::sinf_(theta);
  s00 = (lmin * sn) * sn + (lmax * cs) * cs;
  s01 = ((lmax - lmin) * cs) * sn;
  s11 = (lmin * cs) * cs + (lmax * sn) * sn;
  float det = s00 * s11 - s01 * s01;
  if (det <= 1e-8f) return o;
  float invd = 1.0f / det;
  float k0 = s11 * invd, k1 = -s01 * invd, k2 = s00 * invd;
  // gaussian_projection_is_valid on (center, depth, 1), (conic, det), (cov, orig_det)
  if (!(finitef(cx) && finitef(cy) && finitef(depth) && finitef(k0) && finitef(k1) && finitef(k2) &&
        finitef(det) && finitef(s00) && finitef(s01) && finitef(s11) && finitef(orig_det)))
    return o;
  // The validity test recomputes the determinant (vdet) from the same s00,
  // s01, s11 with the same expression, so vdet == det bit for bit here (no
  // multiply-add contraction): `vdet > 1e-8` repeats the test above, and its
  // consistency checks always pass. |det - vdet| = 0; and with d = det in
  // (1e-8, 1e8], invd = RN(1/d) is normal, so k = RN(s * invd) and
  // e = RN(s / d) differ by a few units in the last place of s/d, far below
  // max(1e-6, |e| 1e-3) (for s00, s11 in (0, 1e4] and |s01| <= sqrt(s00 s11)).
  // Those checks are therefore left out; every outcome is unchanged.
  if (!(depth > 0.0f && s00 > 0.0f && s11 > 0.0f && s00 <= 1e4f && s11 <= 1e4f && k0 > 0.0f && k2 > 0.0f &&
        orig_det >= 0.0f))
    return o;
  o.ok = true;
  o.cx = cx; o.cy = cy; o.depth = depth;
  o.conic_x = k0; o.conic_y = k1; o.conic_z = k2;
  o.cov_x = s00; o.cov_z = s11;
  o.det = det; o.orig_det = orig_det;
  return o;
}

// FP64 form of view_covariance + project (projectionHelpers.ts:4-116), for the
// FP64 projection form: the same steps, constants and tests in double
// precision, from the view-space centre the caller computed in double. Used
// for far-origin scenes (the caller's double mean transform avoids the
// cancellation between large world coordinates and the model-view
// translation) and for near-singular splats (the 2D covariance, its
// determinant and the conic lose most of their bits in FP32 when the
// projected covariance is nearly rank one).
__device__ __noinline__ Projected project_fp64(double vx, double vy, double vz, float4 so, float4 q_in,
                                               const float* mv, const float* P, float vw, float vh, float vnear,
                                               float vfar, float filter) {
  Projected o;
  o.ok = false;
  const double depth = -vz;
  if (!(depth > (double)vnear && depth < (double)vfar)) return o;
  const double clip_x = (P[0] * vx + P[4] * vy) + P[8] * vz + P[12];
  const double clip_y = (P[1] * vx + P[5] * vy) + P[9] * vz + P[13];
  const double clip_w = (P[3] * vx + P[7] * vy) + P[11] * vz + P[15];
  if (clip_w <= 0.0) return o;
  // 3D covariance R S^2 R^T in view space (L R S^2 R^T L^T, L = model-view 3x3).
  const double sx = fmax((double)so.x, 1e-7), sy = fmax((double)so.y, 1e-7), sz = fmax((double)so.z, 1e-7);
  const double qn = sqrt(((double)q_in.x * q_in.x + (double)q_in.y * q_in.y) + (double)q_in.z * q_in.z +
                         (double)q_in.w * q_in.w);
  const double qx = q_in.x / qn, qy = q_in.y / qn, qz = q_in.z / qn, qw = q_in.w / qn;
  double R[3][3];  // R[c][r], column-major like m3
  R[0][0] = 1.0 - 2.0 * (qy * qy + qz * qz); R[0][1] = 2.0 * (qx * qy + qz * qw); R[0][2] = 2.0 * (qx * qz - qy * qw);
  R[1][0] = 2.0 * (qx * qy - qz * qw); R[1][1] = 1.0 - 2.0 * (qx * qx + qz * qz); R[1][2] = 2.0 * (qy * qz + qx * qw);
  R[2][0] = 2.0 * (qx * qz + qy * qw); R[2][1] = 2.0 * (qy * qz - qx * qw); R[2][2] = 1.0 - 2.0 * (qx * qx + qy * qy);
  const double s2[3] = {sx * sx, sy * sy, sz * sz};
  double M[3][3];  // M = L R (columns), so the covariance is M diag(s2) M^T
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r)
      M[c][r] = ((double)mv[r] * R[c][0] + (double)mv[4 + r] * R[c][1]) + (double)mv[8 + r] * R[c][2];
  double cv[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) cv[c][r] = (M[0][r] * s2[0] * M[0][c] + M[1][r] * s2[1] * M[1][c]) + M[2][r] * s2[2] * M[2][c];
  const double cx = ((clip_x / clip_w) * 0.5 + 0.5) * vw;
  const double cy = (0.5 - (clip_y / clip_w) * 0.5) * vh;
  const double fx = (0.5 * vw) * P[0], fy = (0.5 * vh) * P[5];
  const double inv = 1.0 / depth;
  const double j0[3] = {fx * inv, 0.0, fx * vx * inv * inv};
  const double j1[3] = {0.0, -fy * inv, -fy * vy * inv * inv};
  double t0[3], t1[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    t0[r] = (cv[0][r] * j0[0] + cv[1][r] * j0[1]) + cv[2][r] * j0[2];
    t1[r] = (cv[0][r] * j1[0] + cv[1][r] * j1[1]) + cv[2][r] * j1[2];
  }
  const double c_x = (j0[0] * t0[0] + j0[1] * t0[1]) + j0[2] * t0[2];
  const double c_y = (j0[0] * t1[0] + j0[1] * t1[1]) + j0[2] * t1[2];
  const double c_z = (j1[0] * t1[0] + j1[1] * t1[1]) + j1[2] * t1[2];
  const double orig_det = fmax(c_x * c_z - c_y * c_y, 0.0);
  double s00 = c_x + filter, s01 = c_y, s11 = c_z + filter;
  if (!(isfinite(s00) && isfinite(s01) && isfinite(s11))) return o;
  const double mid = 0.5 * (s00 + s11);
  const double rad = sqrt((0.25 * (s00 - s11)) * (s00 - s11) + s01 * s01);
  const double lmin = fmin(fmax(mid - rad, 1e-6), 1e4), lmax = fmin(fmax(mid + rad, 1e-6), 1e4);
  const double theta = 0.5 * atan2(2.0 * s01, s00 - s11);
  const double cs = cos(theta), sn = sin(theta);
  s00 = (lmin * sn) * sn + (lmax * cs) * cs;
  s01 = ((lmax - lmin) * cs) * sn;
  s11 = (lmin * cs) * cs + (lmax * sn) * sn;
  // Exact arithmetic keeps both diagonal terms in [lmin, lmax]; hold that so
  // the 1e4 bound below does not flip on rounding for splats whose
  // eigenvalues are both clamped (the FP32 form drops some of those).
  s00 = fmin(fmax(s00, lmin), lmax);
  s11 = fmin(fmax(s11, lmin), lmax);
  const double det = s00 * s11 - s01 * s01;
  if (det <= 1e-8) return o;
  const double k0 = s11 / det, k1 = -s01 / det, k2 = s00 / det;
  if (!(isfinite(cx) && isfinite(cy) && isfinite(depth) && isfinite(k0) && isfinite(k1) && isfinite(k2)))
    return o;
  if (!(depth > 0.0 && s00 > 0.0 && s11 > 0.0 && s00 <= 1e4 && s11 <= 1e4 && k0 > 0.0 && k2 > 0.0)) return o;
  o.ok = true;
  o.cx = (float)cx; o.cy = (float)cy; o.depth = (float)depth;
  o.conic_x = (float)k0; o.conic_y = (float)k1; o.conic_z = (float)k2;
  o.cov_x = (float)s00; o.cov_z = (float)s11;
  o.det = (float)det; o.orig_det = (float)orig_det;
  return o;
}

// projectionHelpers.ts:150-155: unpack4x8snorm(.xyz) * exp2(e). `snorm`
// holds max(b / 127, -1) for every signed byte b (index b & 255), the exact
// quotients, so the lookup is bit-identical to dividing.
__device__ __forceinline__ f3 decode_sh(uint32_t packed, const float* snorm) {
  int e = (int)((packed >> 24) & 255u) - 127;
  float scale = gsdm::pow2i(e);
  float m0 = snorm[packed & 255u];
  float m1 = snorm[(packed >> 8) & 255u];
  float m2 = snorm[(packed >> 16) & 255u];
  return {m0 * scale, m1 * scale, m2 * scale};
}

__device__ __forceinline__ float snorm8_value(uint32_t byte) {
  return maxf((float)(int)(int8_t)(uint8_t)byte / 127.0f, -1.0f);
}

__device__ __forceinline__ void sh_acc(f3& col, float w, uint32_t packed, const float* snorm) {
  f3 c = decode_sh(packed, snorm);
  col.x = col.x + w * c.x;
  col.y = col.y + w * c.y;
  col.z = col.z + w * c.z;
}

// projectionHelpers.ts:118-179 for rgb8e8; co[] holds the C coefficients.
template <int DEG>
__device__ __forceinline__ f3 eval_sh(const uint32_t* co, f3 d, const float* snorm) {
  float x = d.x, y = d.y, z = d.z;
  f3 c0 = decode_sh(co[0], snorm);
  const float k0 = 0.28209479177387814f;
  f3 col = {k0 * c0.x, k0 * c0.y, k0 * c0.z};
  if (DEG >= 1) {
    sh_acc(col, -0.4886025119029199f * y, co[1], snorm);
    sh_acc(col, 0.4886025119029199f * z, co[2], snorm);
    sh_acc(col, -0.4886025119029199f * x, co[3], snorm);
  }
  if (DEG >= 2) {
    float xx = x * x, yy = y * y, zz = z * z;
    sh_acc(col, (1.0925484305920792f * x) * y, co[4], snorm);
    sh_acc(col, (-1.0925484305920792f * y) * z, co[5], snorm);
    sh_acc(col, 0.31539156525252005f * ((2.0f * zz - xx) - yy), co[6], snorm);
    sh_acc(col, (-1.0925484305920792f * x) * z, co[7], snorm);
    sh_acc(col, 0.5462742152960396f * (xx - yy), co[8], snorm);
  }
  if (DEG >= 3) {
    float xx = x * x, yy = y * y, zz = z * z;
    sh_acc(col, (-0.5900435899266435f * y) * (3.0f * xx - yy), co[9], snorm);
    sh_acc(col, ((2.890611442640554f * x) * y) * z, co[10], snorm);
    sh_acc(col, (-0.4570457994644658f * y) * ((4.0f * zz - xx) - yy), co[11], snorm);
    sh_acc(col, (0.3731763325901154f * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy), co[12], snorm);
    sh_acc(col, (-0.4570457994644658f * x) * ((4.0f * zz - xx) - yy), co[13], snorm);
    sh_acc(col, (1.445305721320277f * z) * (xx - yy), co[14], snorm);
    sh_acc(col, (-0.5900435899266435f * x) * (xx - 3.0f * yy), co[15], snorm);
  }
  return {clampf(col.x + 0.5f, 0.0f, 1.0f), clampf(col.y + 0.5f, 0.0f, 1.0f), clampf(col.z + 0.5f, 0.0f, 1.0f)};
}

// The same SH colour for the fast raster forms, whose colour feeds only the
// image (the EXACT form and the integer stages keep eval_sh): each
// coefficient's rgb8e8 scale 2^(e - 127) is the float whose exponent field is
// e (e = 0, a scale of 2^-127, becomes 0: far below a colour's resolution;
// e = 255 is +inf either way), each signed byte converts directly, and the
// 1/127 of snorm(b) = max(b, -127) / 127 is folded into the basis weights, so
// the decode needs no table. The sum runs as fused multiply-adds from the
// +0.5 offset. The result differs from eval_sh by the rounding of the
// reordered products and sum (a few ulps of the colour), and is clamped to
// [0, 1] the same way.
template <int DEG>
__device__ __forceinline__ f3 eval_sh_fast(const uint32_t* co, f3 d) {
  const float x = d.x, y = d.y, z = d.z;
  constexpr float S = 1.0f / 127.0f;
  float w[16];
  w[0] = 0.28209479177387814f * S;
  if (DEG >= 1) {
    w[1] = (-0.4886025119029199f * S) * y;
    w[2] = (0.4886025119029199f * S) * z;
    w[3] = (-0.4886025119029199f * S) * x;
  }
  if (DEG >= 2) {
    const float xx = x * x, yy = y * y, zz = z * z;
    w[4] = ((1.0925484305920792f * S) * x) * y;
    w[5] = ((-1.0925484305920792f * S) * y) * z;
    w[6] = (0.31539156525252005f * S) * ((2.0f * zz - xx) - yy);
    w[7] = ((-1.0925484305920792f * S) * x) * z;
    w[8] = (0.5462742152960396f * S) * (xx - yy);
  }
  if (DEG >= 3) {
    const float xx = x * x, yy = y * y, zz = z * z;
    w[9] = ((-0.5900435899266435f * S) * y) * (3.0f * xx - yy);
    w[10] = (((2.890611442640554f * S) * x) * y) * z;
    w[11] = ((-0.4570457994644658f * S) * y) * ((4.0f * zz - xx) - yy);
    w[12] = ((0.3731763325901154f * S) * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
    w[13] = ((-0.4570457994644658f * S) * x) * ((4.0f * zz - xx) - yy);
    w[14] = ((1.445305721320277f * S) * z) * (xx - yy);
    w[15] = ((-0.5900435899266435f * S) * x) * (xx - 3.0f * yy);
  }
  f3 col = {0.5f, 0.5f, 0.5f};
#pragma unroll
  for (int k = 0; k < (DEG + 1) * (DEG + 1); ++k) {
    const uint32_t p = co[k];
    const float ws = w[k] * __uint_as_float((p >> 1) & 0x7f800000u);
    col.x = __fmaf_rn(ws, fmaxf((float)(int8_t)(uint8_t)p, -127.0f), col.x);
    col.y = __fmaf_rn(ws, fmaxf((float)(int8_t)(uint8_t)(p >> 8), -127.0f), col.y);
    col.z = __fmaf_rn(ws, fmaxf((float)(int8_t)(uint8_t)(p >> 16), -127.0f), col.z);
  }
  return {clampf(col.x, 0.0f, 1.0f), clampf(col.y, 0.0f, 1.0f), clampf(col.z, 0.0f, 1.0f)};
}

// projectionHelpers.ts:185-221
__device__ __forceinline__ bool subpixel_has_sample(float cx, float cy, float k0, float k1, float k2, float thr,
                                                    float ex, float ey, uint32_t vw, uint32_t vh, uint32_t axis) {
  if (ex * 2.0f > 1.0f || ey * 2.0f > 1.0f) return true;
  float ccx = cx, ccy = cy;
  if (axis == 1u) ccx = ccx - floorf(cx / (float)vw) * (float)vw;
  if (axis == 2u) ccy = ccy - floorf(cy / (float)vh) * (float)vh;
  int minx = (int)ceilf((ccx - ex) - 0.5f);
  int miny = (int)ceilf((ccy - ey) - 0.5f);
  int maxx = (int)floorf((ccx + ex) - 0.5f);
  int maxy = (int)floorf((ccy + ey) - 0.5f);
  int pminx = axis == 1u ? minx : max(minx, 0);
  int pminy = axis == 2u ? miny : max(miny, 0);
  int pmaxx = axis == 1u ? maxx : min(maxx, (int)vw - 1);
  int pmaxy = axis == 2u ? maxy : min(maxy, (int)vh - 1);
  for (int py = pminy; py <= pmaxy; ++py)
    for (int px = pminx; px <= pmaxx; ++px) {
      float dx = ((float)px + 0.5f) - ccx;
      float dy = ((float)py + 0.5f) - ccy;
      float sigma = 0.5f * (((k0 * dx) * dx + ((2.0f * k1) * dx) * dy) + (k2 * dy) * dy);
      if (sigma <= thr) return true;
    }
  return false;
}

// tileContribution.ts:16-59 for one image centre; ts = pixels per tile side
// (the reference's TILE_SIZE, 16, constants.ts:1; 8 and 32 in batched renders
// tuned to them).
__device__ __forceinline__ bool tile_rect_test(float cx, float cy, float k0, float k1, float k2, float thr, int tx,
                                               int ty, float ts) {
  float rminx = (float)tx * ts, rminy = (float)ty * ts;
  float rmaxx = rminx + ts, rmaxy = rminy + ts;
  bool x_left = cx < rminx, x_right = cx > rmaxx;
  bool in_x = !(x_left || x_right);
  bool y_above = cy < rminy, y_below = cy > rmaxy;
  bool in_y = !(y_above || y_below);
  if (in_x && in_y) return true;
  float cornerx = x_left ? rminx : rmaxx;
  float cornery = y_above ? rminy : rmaxy;
  float ex = x_left ? ts : -ts;
  float ey = y_above ? ts : -ts;
  float dfx = cx - cornerx, dfy = cy - cornery;
  float txr = ((ex * k0) * dfx + (ex * k1) * dfy) / ((ex * k0) * ex);
  float tyr = ((ey * k1) * dfx + (ey * k2) * dfy) / ((ey * k2) * ey);
  float t_x = in_y ? 0.0f : clampf(txr, 0.0f, 1.0f);
  float t_y = in_x ? 0.0f : clampf(tyr, 0.0f, 1.0f);
  float clx = cornerx + t_x * ex, cly = cornery + t_y * ey;
  float dx = clx - cx, dy = cly - cy;
  float sigma = 0.5f * ((k0 * dx) * dx + (k2 * dy) * dy) + (k1 * dx) * dy;
  return sigma <= thr;
}

// tileContribution.ts:84-114
__device__ __forceinline__ bool boundary_tile_hit(float cx, float cy, float k0, float k1, float k2, float thr,
                                                  float rx, float ry, int tx, int ty, float vw, float vh,
                                                  uint32_t axis, float ts) {
  if (axis == 0u) return tile_rect_test(cx, cy, k0, k1, k2, thr, tx, ty, ts);
  bool ax = axis == 1u;
  float period = ax ? vw : vh;
  float cen = ax ? cx : cy;
  float canon = cen - floorf(cen / period) * period;
  float ccx = ax ? canon : cx, ccy = ax ? cy : canon;
  float tstart = (float)(ax ? tx : ty) * ts;
  float r = ax ? rx : ry;
  int first = (int)ceilf(((tstart - r) - canon) / period);
  int last = (int)floorf((((tstart + ts) + r) - canon) / period);
  for (int img = first; img <= last; ++img) {
    float icx = ccx, icy = ccy;
    if (ax) icx = icx + (float)img * vw; else icy = icy + (float)img * vh;
    if (tile_rect_test(icx, icy, k0, k1, k2, thr, tx, ty, ts)) return true;
  }
  return false;
}

}  // namespace gs
