// On-device compact packer: linear splat attributes -> the packed storage
// buffers the pass consumes (GaussianData.ts:10-33), one thread per splat.
// Restates, on the GPU, the reference's CPU packer for the compact layout:
//   rust/gaussian-backend/src/engine.rs:1801-1891 encode_attributes (compact):
//     means          (x, y, z, objectId)
//     scalesOpacity  [f16 ln sx | f16 ln sy << 16, f16 ln sz | f16 opacity << 16]
//                    (rust/vendor/spark-lib/src/splat_encode.rs:127-136 encode_ext_splat)
//     rotations      oct101012 of the normalised quaternion (splat_encode.rs:234-252)
//     shCoefficients rgb8e8 words: DC = (rgb - 0.5) / SH_C0, then the higher bands
//                    (engine.rs:1857-1872, pack_sh :1940-1949)
// Built with --fmad=false so products and sums round like the Rust code.
// f16 conversion rounds to nearest even (half::f16::from_f32), round() is half
// away from zero (f32::round), the rgb8e8 exponent is ceil(log2 max|c|)
// computed exactly from the binary exponent. ln, acos and sin are CUDA's; where
// a result sits within an ulp of a quantisation boundary the packed field can
// differ by one step from the CPU packer's.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gs3d.h"

namespace {

constexpr float kShC0 = 0.28209479177387814f;  // engine.rs:1858
constexpr float kPi = 3.14159265358979323846f;

__device__ __forceinline__ uint32_t f16_bits(float x) { return (uint32_t)__half_as_ushort(__float2half_rn(x)); }

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

// splat_encode.rs:234-252 encode_quat_oct101012.
__device__ uint32_t encode_oct101012(float qx, float qy, float qz, float qw) {
  if (qw < 0.0f) {
    qx = -qx; qy = -qy; qz = -qz; qw = -qw;
  }
  const float theta = 2.0f * acosf(clampf(qw, 0.0f, 1.0f));
  const float s = sinf(theta * 0.5f);
  float ax = 1.0f, ay = 0.0f, az = 0.0f;
  if (!(fabsf(s) < 1e-6f)) {
    ax = qx / s; ay = qy / s; az = qz / s;
  }
  const float sum = (fabsf(ax) + fabsf(ay)) + fabsf(az);
  float p0 = ax / sum, p1 = ay / sum;
  if (az < 0.0f) {
    const float f0 = (1.0f - fabsf(p1)) * (p0 >= 0.0f ? 1.0f : -1.0f);
    const float f1 = (1.0f - fabsf(p0)) * (p1 >= 0.0f ? 1.0f : -1.0f);
    p0 = f0; p1 = f1;
  }
  const uint32_t u = (uint32_t)roundf(clampf((p0 * 0.5f + 0.5f) * 1023.0f, 0.0f, 1023.0f));
  const uint32_t v = (uint32_t)roundf(clampf((p1 * 0.5f + 0.5f) * 1023.0f, 0.0f, 1023.0f));
  const uint32_t r = (uint32_t)roundf(clampf(theta / kPi * 4095.0f, 0.0f, 4095.0f));
  return (r << 20) | (v << 10) | u;
}

// The shared exponent of engine.rs:1945, `max.log2().ceil()` on an f32: the
// ceiling of log2 rounded to f32. It equals the exact ceiling except just
// above a power of two 2^e (e != 0), where log2 rounds down to e itself and
// the exponent stays e instead of e + 1. Decided exactly: the f32 neighbour
// of e towards e + 1 lies ulp(e) above a positive e, and below |e| by
// ulp(|e|) (half that when |e| is a power of two) for a negative e; log2
// rounds to e when log2(m) is under half that gap. log2(m) is evaluated in
// double, far more precisely than the decision needs.
__device__ int rounded_log2_ceil(float mx) {
  if (isnan(mx)) return 0;       // Rust's saturating cast of NaN
  if (isinf(mx)) return 127;     // clamped below
  int ex = 0;
  const float f = frexpf(mx, &ex);  // mx = f 2^ex, f in [0.5, 1)
  if (f == 0.5f) return ex - 1;      // a power of two
  const int e = ex - 1;              // floor(log2 mx); mantissa m = 2 f in (1, 2)
  if (e == 0) return 1;              // log2 m itself is representable: above 0
  const int a = e > 0 ? e : -e;
  int gap_exp = (31 - __clz(a)) - 23;
  if (e < 0 && (a & (a - 1)) == 0) gap_exp -= 1;
  const double log2_m = log1p((double)(2.0f * f) - 1.0) * 1.4426950408889634074;
  return log2_m < ldexp(1.0, gap_exp - 1) ? e : e + 1;
}

// engine.rs:1940-1949 pack_sh.
__device__ uint32_t pack_sh(float r, float g, float b) {
  const float mx = fmaxf(fmaxf(fabsf(r), fabsf(g)), fabsf(b));
  if (mx == 0.0f) return 0u;
  int e = rounded_log2_ceil(mx);
  e = e < -126 ? -126 : (e > 127 ? 127 : e);
  const float mult = 127.0f / ldexpf(1.0f, e);
  const float c[3] = {r, g, b};
  uint32_t w = (uint32_t)(e + 127) << 24;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float q = clampf(floorf(c[i] * mult + 0.5f), -127.0f, 127.0f);
    w |= ((uint32_t)(int32_t)q & 255u) << (8 * i);
  }
  return w;
}

__global__ void k_pack(gs3d_splat_source src, uint32_t first, float4* __restrict__ means,
                       uint2* __restrict__ shape, uint32_t* __restrict__ rot, uint32_t* __restrict__ sh, uint32_t C) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= src.count) return;
  const size_t slot = (size_t)first + i;
  const float cx = src.centers[3 * (size_t)i], cy = src.centers[3 * (size_t)i + 1], cz = src.centers[3 * (size_t)i + 2];
  means[slot] = make_float4(cx, cy, cz, (float)src.object_id);
  const float sx = src.scales[3 * (size_t)i], sy = src.scales[3 * (size_t)i + 1], sz = src.scales[3 * (size_t)i + 2];
  shape[slot] = make_uint2(f16_bits(logf(sx)) | (f16_bits(logf(sy)) << 16),
                           f16_bits(logf(sz)) | (f16_bits(src.opacity[i]) << 16));
  // glam Quat::normalize: multiply by the reciprocal of the length.
  const float* q = src.quaternions + 4 * (size_t)i;
  const float inv = 1.0f / sqrtf(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
  rot[slot] = encode_oct101012(q[0] * inv, q[1] * inv, q[2] * inv, q[3] * inv);
  uint32_t* out = sh + slot * C;
  const float* rgb = src.rgb + 3 * (size_t)i;
  out[0] = pack_sh((rgb[0] - 0.5f) / kShC0, (rgb[1] - 0.5f) / kShC0, (rgb[2] - 0.5f) / kShC0);
  for (uint32_t k = 1; k < C; ++k) {
    const float* c = src.sh_rest + (size_t)i * (C - 1) * 3 + (size_t)(k - 1) * 3;
    out[k] = pack_sh(c[0], c[1], c[2]);
  }
}

}  // namespace

extern "C" gs3d_status gs3d_pack_splats(const gs3d_splat_source* src, uint32_t first_slot, float* means,
                                        uint32_t* scales_opacity, uint32_t* rotations, uint32_t* sh_coefficients,
                                        uint32_t capacity, void* stream) {
  if (!src || !means || !scales_opacity || !rotations || !sh_coefficients) return GS3D_ERROR_INVALID_ARGUMENT;
  if (src->sh_degree > 3) return GS3D_ERROR_RANGE;
  if ((uint64_t)first_slot + src->count > capacity) return GS3D_ERROR_RANGE;
  if (src->count == 0) return GS3D_OK;
  if (!src->centers || !src->scales || !src->opacity || !src->quaternions || !src->rgb ||
      (src->sh_degree > 0 && !src->sh_rest))
    return GS3D_ERROR_INVALID_ARGUMENT;
  if (((uintptr_t)means & 15u) || ((uintptr_t)scales_opacity & 7u)) return GS3D_ERROR_INVALID_ARGUMENT;
  const uint32_t C = (src->sh_degree + 1) * (src->sh_degree + 1);
  const uint32_t grid = (src->count + 255u) / 256u;
  k_pack<<<grid, 256, 0, (cudaStream_t)stream>>>(*src, first_slot, reinterpret_cast<float4*>(means),
                                                 reinterpret_cast<uint2*>(scales_opacity), rotations,
                                                 sh_coefficients, C);
  return cudaGetLastError() == cudaSuccess ? GS3D_OK : GS3D_ERROR_CUDA;
}
