// CPU oracle for the tiled Gaussian-splatting pass — TEST INFRASTRUCTURE ONLY.
//
// Only tests, the smoke check and bench.py's CPU-baseline leg load this
// library. It is the checker, never the product: the CUDA library under
// 3dgs_tile_webgpu_gb300/ does not link or call it.
//
// It restates the reference's WGSL/TSL kernels on the CPU in the reference's
// own operation order, templated on the scalar type:
//   * Real = float  : the FP32 restatement. Integer outputs (tile counts, scan
//                     offsets, depth keys, sorted records, tile ranges) are the
//                     bit-exact parity target of the CUDA path.
//   * Real = double : the FP64 twin, the image oracle for max-abs error / PSNR.
// Transcendentals in FP32 come from csrc/detmath.h (the same deterministic
// functions the CUDA path uses); FP64 uses the C library.
//
// Parity pins: the reference's executed-WGSL known-answer tests
// (test/ProjectionBoundary.test.ts, test/ScalarOutput.test.ts,
// test/rasterizationWGSL.test.ts, test/GaussianSh.test.ts) and the Rust
// compact-geometry test (rust/gaussian-backend/tests/backend.rs:1086-1174) are
// ported in tests/test_oracle_known_answers.py. The reference has no image
// golden, so image-level parity is pinned only through these function-level
// tests.
//
// Build: oracle/__init__.py build() (g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math -fopenmp).

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../3dgs_tile_webgpu_gb300/csrc/detmath.h"

#if defined(_OPENMP)
#include <omp.h>
#endif

namespace {

constexpr int TILE = 16;               // src/renderer/pipeline/constants.ts:1
constexpr uint32_t ACTIVE_TAG = 0x3f800000u;  // activeSlots.ts:4

// ---------------------------------------------------------------------------
// Math dispatch: FP32 uses the deterministic functions, FP64 the C library.
template <typename T> struct Mth;
template <> struct Mth<float> {
  static float exp(float x) { return gsdm::expf_(x); }
  static float log(float x) { return gsdm::logf_(x); }
  static float sin(float x) { return gsdm::sinf_(x); }
  static float cos(float x) { return gsdm::cosf_(x); }
  static float atan2(float y, float x) { return gsdm::atan2f_(y, x); }
  static float sqrt(float x) { return sqrtf(x); }
  static float floor(float x) { return floorf(x); }
  static float ceil(float x) { return ceilf(x); }
  static float maxfin() { return 3.402823e+38f; }
};
template <> struct Mth<double> {
  static double exp(double x) { return ::exp(x); }
  static double log(double x) { return ::log(x); }
  static double sin(double x) { return ::sin(x); }
  static double cos(double x) { return ::cos(x); }
  static double atan2(double y, double x) { return ::atan2(y, x); }
  static double sqrt(double x) { return ::sqrt(x); }
  static double floor(double x) { return ::floor(x); }
  static double ceil(double x) { return ::ceil(x); }
  static double maxfin() { return (double)3.402823e+38f; }
};

// WGSL literal constants are f32; the FP64 twin widens the same f32 values.
template <typename T> static inline T K(float v) { return (T)v; }

template <typename T> static inline T clampT(T x, T lo, T hi) {
  T y = x < lo ? lo : x;
  return y > hi ? hi : y;
}
template <typename T> static inline T maxT(T a, T b) { return a < b ? b : a; }
template <typename T> static inline T minT(T a, T b) { return b < a ? b : a; }
template <typename T> static inline T absT(T a) { return a < 0 ? -a : a; }
template <typename T> static inline bool finiteT(T v) {
  return v == v && absT(v) <= Mth<T>::maxfin();
}

template <typename T> struct V2 { T x, y; };
template <typename T> struct V3 { T x, y, z; };
template <typename T> struct V4 { T x, y, z, w; };
// Column-major like WGSL: c[k] is column k.
template <typename T> struct M3 { V3<T> c[3]; };
template <typename T> struct M4 { V4<T> c[4]; };

template <typename T> static inline T row3(const M3<T>& m, int r, int k) {
  const V3<T>& col = m.c[k];
  return r == 0 ? col.x : (r == 1 ? col.y : col.z);
}
template <typename T> static inline T row4(const M4<T>& m, int r, int k) {
  const V4<T>& col = m.c[k];
  return r == 0 ? col.x : (r == 1 ? col.y : (r == 2 ? col.z : col.w));
}

// (A * B)[r][c] = sum_k A[r][k] B[k][c], accumulated in increasing k.
template <typename T> static M3<T> mul33(const M3<T>& a, const M3<T>& b) {
  M3<T> o;
  for (int c = 0; c < 3; ++c) {
    T v[3];
    for (int r = 0; r < 3; ++r) {
      T s = row3(a, r, 0) * row3(b, 0, c);
      s = s + row3(a, r, 1) * row3(b, 1, c);
      s = s + row3(a, r, 2) * row3(b, 2, c);
      v[r] = s;
    }
    o.c[c] = {v[0], v[1], v[2]};
  }
  return o;
}
template <typename T> static M3<T> transpose3(const M3<T>& m) {
  M3<T> o;
  for (int c = 0; c < 3; ++c) o.c[c] = {row3(m, c, 0), row3(m, c, 1), row3(m, c, 2)};
  return o;
}
template <typename T> static V3<T> mul3v(const M3<T>& m, V3<T> v) {
  T o[3];
  for (int r = 0; r < 3; ++r) {
    T s = row3(m, r, 0) * v.x;
    s = s + row3(m, r, 1) * v.y;
    s = s + row3(m, r, 2) * v.z;
    o[r] = s;
  }
  return {o[0], o[1], o[2]};
}
template <typename T> static V4<T> mul4v(const M4<T>& m, V4<T> v) {
  T o[4];
  for (int r = 0; r < 4; ++r) {
    T s = row4(m, r, 0) * v.x;
    s = s + row4(m, r, 1) * v.y;
    s = s + row4(m, r, 2) * v.z;
    s = s + row4(m, r, 3) * v.w;
    o[r] = s;
  }
  return {o[0], o[1], o[2], o[3]};
}
template <typename T> static inline T dot3(V3<T> a, V3<T> b) {
  return (a.x * b.x + a.y * b.y) + a.z * b.z;
}
template <typename T> static V3<T> normalize3(V3<T> v) {
  T len = Mth<T>::sqrt(dot3(v, v));
  return {v.x / len, v.y / len, v.z / len};
}
template <typename T> static V4<T> normalize4(V4<T> v) {
  T d = ((v.x * v.x + v.y * v.y) + v.z * v.z) + v.w * v.w;
  T len = Mth<T>::sqrt(d);
  return {v.x / len, v.y / len, v.z / len, v.w / len};
}

template <typename T> static M4<T> load_m4(const float* e) {
  M4<T> m;
  for (int c = 0; c < 4; ++c)
    m.c[c] = {(T)e[4 * c + 0], (T)e[4 * c + 1], (T)e[4 * c + 2], (T)e[4 * c + 3]};
  return m;
}

template <typename T> static M4<T> zero_m4() {
  M4<T> m;
  memset(&m, 0, sizeof(m));
  return m;
}

// ---------------------------------------------------------------------------
// Input codecs.

// compactGaussians.ts:2-7 decodeCompactScaleOpacity.
template <typename T> static V4<T> decode_compact_scale_opacity(uint32_t px, uint32_t py) {
  T sx = (T)gsdm::half_bits_to_float(px & 0xffffu);
  T sy = (T)gsdm::half_bits_to_float(px >> 16);
  T sz = (T)gsdm::half_bits_to_float(py & 0xffffu);
  T a = (T)gsdm::half_bits_to_float(py >> 16);
  return {Mth<T>::exp(sx), Mth<T>::exp(sy), Mth<T>::exp(sz), a};
}

// compactGaussians.ts:10-19 decodeCompactRotation (Spark oct101012).
template <typename T> static V4<T> decode_compact_rotation(uint32_t packed) {
  T px = (((T)(float)(packed & 1023u) / K<T>(1023.0f)) * K<T>(2.0f)) - K<T>(1.0f);
  T py = (((T)(float)((packed >> 10) & 1023u) / K<T>(1023.0f)) * K<T>(2.0f)) - K<T>(1.0f);
  T z = (K<T>(1.0f) - absT(px)) - absT(py);
  T t = maxT(-z, K<T>(0.0f));
  T x = px >= 0 ? px - t : px + t;
  T y = py >= 0 ? py - t : py + t;
  V3<T> axis = normalize3<T>({x, y, z});
  T half = ((T)(float)(packed >> 20) / K<T>(4095.0f)) * K<T>(1.5707963267948966f);
  T s = Mth<T>::sin(half);
  return {axis.x * s, axis.y * s, axis.z * s, Mth<T>::cos(half)};
}

// projectionHelpers.ts:150-155 decode_sh_rgb8e8: unpack4x8snorm(.xyz) * exp2(e).
template <typename T> static V3<T> decode_sh_rgb8e8(uint32_t packed) {
  int exponent = (int)((packed >> 24) & 255u) - 127;
  // exp2 of an integer: exact in f32 (inf at 2^128), exact in double.
  T scale = sizeof(T) == 4 ? (T)gsdm::pow2i(exponent) : (T)ldexp(1.0, exponent);
  T m[3];
  for (int i = 0; i < 3; ++i) {
    int b = (int)(int8_t)(uint8_t)(packed >> (8 * i));
    T v = (T)(float)b / K<T>(127.0f);
    m[i] = maxT(v, K<T>(-1.0f));
  }
  return {m[0] * scale, m[1] * scale, m[2] * scale};
}

// ---------------------------------------------------------------------------
// Projection helpers (projectionHelpers.ts).

// projectionHelpers.ts:4-35 gaussian_view_covariance.
template <typename T> static M3<T> view_covariance(V3<T> s_in, V4<T> r_in, const M4<T>& mv) {
  V3<T> s = {maxT(s_in.x, K<T>(1e-7f)), maxT(s_in.y, K<T>(1e-7f)), maxT(s_in.z, K<T>(1e-7f))};
  V4<T> q = normalize4(r_in);
  T xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
  T xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
  T xw = q.x * q.w, yw = q.y * q.w, zw = q.z * q.w;
  const T one = K<T>(1.0f), two = K<T>(2.0f);
  M3<T> rot;
  rot.c[0] = {one - two * (yy + zz), two * (xy + zw), two * (xz - yw)};
  rot.c[1] = {two * (xy - zw), one - two * (xx + zz), two * (yz + xw)};
  rot.c[2] = {two * (xz + yw), two * (yz - xw), one - two * (xx + yy)};
  M3<T> sc;
  sc.c[0] = {s.x * s.x, K<T>(0.0f), K<T>(0.0f)};
  sc.c[1] = {K<T>(0.0f), s.y * s.y, K<T>(0.0f)};
  sc.c[2] = {K<T>(0.0f), K<T>(0.0f), s.z * s.z};
  M3<T> local = mul33(mul33(rot, sc), transpose3(rot));
  M3<T> l2v;
  l2v.c[0] = {mv.c[0].x, mv.c[0].y, mv.c[0].z};
  l2v.c[1] = {mv.c[1].x, mv.c[1].y, mv.c[1].z};
  l2v.c[2] = {mv.c[2].x, mv.c[2].y, mv.c[2].z};
  return mul33(mul33(l2v, local), transpose3(l2v));
}

// projectionHelpers.ts:38-83 gaussian_projection_result.
template <typename T> static M4<T> projection_result(V2<T> center, T depth, V3<T> cov, T filter) {
  T orig_det = maxT(cov.x * cov.z - cov.y * cov.y, K<T>(0.0f));
  T s00 = cov.x + filter;
  T s01 = cov.y;
  T s11 = cov.z + filter;
  if (!(finiteT(s00) && finiteT(s01) && finiteT(s11))) return zero_m4<T>();
  T mid = K<T>(0.5f) * (s00 + s11);
  T rad = Mth<T>::sqrt((K<T>(0.25f) * (s00 - s11)) * (s00 - s11) + s01 * s01);
  T lmin = clampT(mid - rad, K<T>(1e-6f), K<T>(1e4f));
  T lmax = clampT(mid + rad, K<T>(1e-6f), K<T>(1e4f));
  T theta = K<T>(0.5f) * Mth<T>::atan2(K<T>(2.0f) * s01, s00 - s11);
  T cs = Mth<T>::cos(theta);
  T sn = Mth<T>::sin(theta);
  s00 = (lmin * sn) * sn + (lmax * cs) * cs;
  s01 = ((lmax - lmin) * cs) * sn;
  s11 = (lmin * cs) * cs + (lmax * sn) * sn;
  if (sizeof(T) == sizeof(double)) {
    // FP64 twin: in exact arithmetic both diagonal terms lie in [lmin, lmax]
    // (cos^2 + sin^2 = 1); keep that so the validity test's 1e4 bound does not
    // flip on the last bit for splats whose eigenvalues are both clamped. The
    // FP32 restatement keeps the reference's rounding, cliff included.
    s00 = clampT(s00, lmin, lmax);
    s11 = clampT(s11, lmin, lmax);
  }
  T det = s00 * s11 - s01 * s01;
  if (det <= K<T>(1e-8f)) return zero_m4<T>();
  T inv = K<T>(1.0f) / det;
  M4<T> o;
  o.c[0] = {center.x, center.y, depth, K<T>(1.0f)};
  o.c[1] = {s11 * inv, -s01 * inv, s00 * inv, det};
  o.c[2] = {s00, s01, s11, orig_det};
  o.c[3] = {0, 0, 0, 0};
  return o;
}

// projectionHelpers.ts:86-96 perspective_gaussian_projection.
template <typename T>
static M4<T> perspective_projection(V3<T> view, const M3<T>& cv, const M4<T>& proj, V4<T> vp, T filter) {
  T depth = -view.z;
  if (!(depth > vp.z && depth < vp.w)) return zero_m4<T>();
  V4<T> clip = mul4v(proj, V4<T>{view.x, view.y, view.z, K<T>(1.0f)});
  if (clip.w <= 0) return zero_m4<T>();
  T ndcx = clip.x / clip.w, ndcy = clip.y / clip.w;
  V2<T> center = {(ndcx * K<T>(0.5f) + K<T>(0.5f)) * vp.x, (K<T>(0.5f) - ndcy * K<T>(0.5f)) * vp.y};
  T fx = (K<T>(0.5f) * vp.x) * proj.c[0].x;
  T fy = (K<T>(0.5f) * vp.y) * proj.c[1].y;
  T inv = K<T>(1.0f) / depth;
  V3<T> j0 = {fx * inv, K<T>(0.0f), ((fx * view.x) * inv) * inv};
  T nfy = -fy;
  V3<T> j1 = {K<T>(0.0f), nfy * inv, ((nfy * view.y) * inv) * inv};
  V3<T> cov = {dot3(j0, mul3v(cv, j0)), dot3(j0, mul3v(cv, j1)), dot3(j1, mul3v(cv, j1))};
  return projection_result(center, depth, cov, filter);
}

// projectionHelpers.ts:99-116 gaussian_projection_is_valid.
template <typename T> static bool projection_is_valid(const M4<T>& p) {
  for (int i = 0; i < 3; ++i) {
    const V4<T>& c = p.c[i];
    if (!(finiteT(c.x) && finiteT(c.y) && finiteT(c.z) && finiteT(c.w))) return false;
  }
  V3<T> cov = {p.c[2].x, p.c[2].y, p.c[2].z};
  T det = cov.x * cov.z - cov.y * cov.y;
  V3<T> conic = {p.c[1].x, p.c[1].y, p.c[1].z};
  if (!(p.c[0].w > 0 && p.c[0].z > 0 && det > K<T>(1e-8f) && cov.x > 0 && cov.z > 0 &&
        cov.x <= K<T>(1e4f) && cov.z <= K<T>(1e4f) && conic.x > 0 && conic.z > 0 && p.c[2].w >= 0))
    return false;
  V3<T> e = {cov.z / det, -cov.y / det, cov.x / det};
  bool ok = absT(p.c[1].w - det) <= maxT(K<T>(1e-6f), det * K<T>(1e-3f));
  ok = ok && absT(conic.x - e.x) <= maxT(K<T>(1e-6f), absT(e.x) * K<T>(1e-3f));
  ok = ok && absT(conic.y - e.y) <= maxT(K<T>(1e-6f), absT(e.y) * K<T>(1e-3f));
  ok = ok && absT(conic.z - e.z) <= maxT(K<T>(1e-6f), absT(e.z) * K<T>(1e-3f));
  return ok;
}

// projectionHelpers.ts:118-179 evaluate_gaussian_sh_rgb8e8.
template <typename T> static V3<T> eval_sh_rgb8e8(const uint32_t* co, uint32_t degree, V3<T> d) {
  T x = d.x, y = d.y, z = d.z;
  auto acc = [&](V3<T>& col, T w, uint32_t i) {
    V3<T> c = decode_sh_rgb8e8<T>(co[i]);
    col.x = col.x + w * c.x;
    col.y = col.y + w * c.y;
    col.z = col.z + w * c.z;
  };
  V3<T> c0 = decode_sh_rgb8e8<T>(co[0]);
  const T k0 = K<T>(0.28209479177387814f);
  V3<T> col = {k0 * c0.x, k0 * c0.y, k0 * c0.z};
  if (degree >= 1) {
    acc(col, K<T>(-0.4886025119029199f) * y, 1);
    acc(col, K<T>(0.4886025119029199f) * z, 2);
    acc(col, K<T>(-0.4886025119029199f) * x, 3);
  }
  if (degree >= 2) {
    T xx = x * x, yy = y * y, zz = z * z;
    acc(col, (K<T>(1.0925484305920792f) * x) * y, 4);
    acc(col, (K<T>(-1.0925484305920792f) * y) * z, 5);
    acc(col, K<T>(0.31539156525252005f) * ((K<T>(2.0f) * zz - xx) - yy), 6);
    acc(col, (K<T>(-1.0925484305920792f) * x) * z, 7);
    acc(col, K<T>(0.5462742152960396f) * (xx - yy), 8);
  }
  if (degree >= 3) {
    T xx = x * x, yy = y * y, zz = z * z;
    acc(col, (K<T>(-0.5900435899266435f) * y) * (K<T>(3.0f) * xx - yy), 9);
    acc(col, ((K<T>(2.890611442640554f) * x) * y) * z, 10);
    acc(col, (K<T>(-0.4570457994644658f) * y) * ((K<T>(4.0f) * zz - xx) - yy), 11);
    acc(col, (K<T>(0.3731763325901154f) * z) * ((K<T>(2.0f) * zz - K<T>(3.0f) * xx) - K<T>(3.0f) * yy), 12);
    acc(col, (K<T>(-0.4570457994644658f) * x) * ((K<T>(4.0f) * zz - xx) - yy), 13);
    acc(col, (K<T>(1.445305721320277f) * z) * (xx - yy), 14);
    acc(col, (K<T>(-0.5900435899266435f) * x) * (xx - K<T>(3.0f) * yy), 15);
  }
  const T h = K<T>(0.5f), z0 = K<T>(0.0f), o = K<T>(1.0f);
  return {clampT(col.x + h, z0, o), clampT(col.y + h, z0, o), clampT(col.z + h, z0, o)};
}

// projectionHelpers.ts:185-221 subpixel_has_sample.
template <typename T>
static bool subpixel_has_sample(V2<T> center, V3<T> conic, T thr, V2<T> extent, uint32_t vw, uint32_t vh,
                                uint32_t axis) {
  if (extent.x * K<T>(2.0f) > K<T>(1.0f) || extent.y * K<T>(2.0f) > K<T>(1.0f)) return true;
  V2<T> cc = center;
  if (axis == 1u) cc.x = cc.x - Mth<T>::floor(center.x / (T)(float)vw) * (T)(float)vw;
  if (axis == 2u) cc.y = cc.y - Mth<T>::floor(center.y / (T)(float)vh) * (T)(float)vh;
  int minx = (int)Mth<T>::ceil((cc.x - extent.x) - K<T>(0.5f));
  int miny = (int)Mth<T>::ceil((cc.y - extent.y) - K<T>(0.5f));
  int maxx = (int)Mth<T>::floor((cc.x + extent.x) - K<T>(0.5f));
  int maxy = (int)Mth<T>::floor((cc.y + extent.y) - K<T>(0.5f));
  int pminx = axis == 1u ? minx : std::max(minx, 0);
  int pminy = axis == 2u ? miny : std::max(miny, 0);
  int pmaxx = axis == 1u ? maxx : std::min(maxx, (int)vw - 1);
  int pmaxy = axis == 2u ? maxy : std::min(maxy, (int)vh - 1);
  for (int py = pminy; py <= pmaxy; ++py) {
    for (int px = pminx; px <= pmaxx; ++px) {
      T dx = ((T)(float)px + K<T>(0.5f)) - cc.x;
      T dy = ((T)(float)py + K<T>(0.5f)) - cc.y;
      T sigma = K<T>(0.5f) * (((conic.x * dx) * dx + ((K<T>(2.0f) * conic.y) * dx) * dy) + (conic.z * dy) * dy);
      if (sigma <= thr) return true;
    }
  }
  return false;
}

// tileContribution.ts:16-59, inlined by tileContribution.ts:84-114 for one image.
template <typename T> static bool tile_rect_test(V2<T> c, V3<T> conic, T thr, int tx, int ty) {
  const T ts = K<T>((float)TILE);
  T rminx = (T)(float)tx * ts, rminy = (T)(float)ty * ts;
  T rmaxx = rminx + ts, rmaxy = rminy + ts;
  bool x_left = c.x < rminx, x_right = c.x > rmaxx;
  bool in_x = !(x_left || x_right);
  bool y_above = c.y < rminy, y_below = c.y > rmaxy;
  bool in_y = !(y_above || y_below);
  if (in_x && in_y) return true;
  T cornerx = x_left ? rminx : rmaxx;
  T cornery = y_above ? rminy : rmaxy;
  T ex = x_left ? ts : -ts;
  T ey = y_above ? ts : -ts;
  T dfx = c.x - cornerx, dfy = c.y - cornery;
  T txr = ((ex * conic.x) * dfx + (ex * conic.y) * dfy) / ((ex * conic.x) * ex);
  T tyr = ((ey * conic.y) * dfx + (ey * conic.z) * dfy) / ((ey * conic.z) * ey);
  T tx_ = in_y ? K<T>(0.0f) : clampT(txr, K<T>(0.0f), K<T>(1.0f));
  T ty_ = in_x ? K<T>(0.0f) : clampT(tyr, K<T>(0.0f), K<T>(1.0f));
  T clx = cornerx + tx_ * ex, cly = cornery + ty_ * ey;
  T dx = clx - c.x, dy = cly - c.y;
  T sigma = K<T>(0.5f) * ((conic.x * dx) * dx + (conic.z * dy) * dy) + (conic.y * dx) * dy;
  return sigma <= thr;
}

// tileContribution.ts:84-114 gaussian_boundary_tile_hit.
template <typename T>
static bool boundary_tile_hit(V2<T> center, V3<T> conic, T thr, V2<T> radius, int tx, int ty, V2<T> vp,
                              uint32_t axis) {
  V2<T> cc = center;
  int first = 0, last = 0;
  if (axis != 0u) {
    bool ax = axis == 1u;
    T period = ax ? vp.x : vp.y;
    T cen = ax ? center.x : center.y;
    T canon = cen - Mth<T>::floor(cen / period) * period;
    if (ax) cc.x = canon; else cc.y = canon;
    T tstart = (T)(float)(ax ? tx : ty) * K<T>((float)TILE);
    T r = ax ? radius.x : radius.y;
    first = (int)Mth<T>::ceil(((tstart - r) - canon) / period);
    last = (int)Mth<T>::floor((((tstart + K<T>((float)TILE)) + r) - canon) / period);
  }
  for (int img = first; img <= last; ++img) {
    V2<T> ic = cc;
    if (axis == 1u) ic.x = ic.x + (T)(float)img * vp.x;
    if (axis == 2u) ic.y = ic.y + (T)(float)img * vp.y;
    if (tile_rect_test(ic, conic, thr, tx, ty)) return true;
  }
  return false;
}

// projectionHelpers.ts:223-236 count_contributing_tiles.
template <typename T>
static uint32_t count_tiles(V2<T> center, V3<T> conic, T thr, V2<T> radius, int tminx, int tminy, int tmaxx,
                            int tmaxy, V2<T> vp, uint32_t axis) {
  uint32_t n = 0;
  for (int ty = tminy; ty <= tmaxy; ++ty)
    for (int tx = tminx; tx <= tmaxx; ++tx)
      if (boundary_tile_hit(center, conic, thr, radius, tx, ty, vp, axis)) ++n;
  return n;
}

// tileContribution.ts:66-82 gaussian_boundary_delta.
template <typename T> static V2<T> boundary_delta(V2<T> pixel, V2<T> center, V3<T> conic, V2<T> vp, uint32_t axis) {
  V2<T> cc = center;
  if (axis == 1u) cc.x = cc.x - Mth<T>::floor(center.x / vp.x) * vp.x;
  if (axis == 2u) cc.y = cc.y - Mth<T>::floor(center.y / vp.y) * vp.y;
  V2<T> d = {pixel.x - cc.x, pixel.y - cc.y};
  if (axis == 1u) {
    T opt = (-conic.y * d.y) / conic.x;
    d.x = d.x - Mth<T>::floor((d.x - opt) / vp.x + K<T>(0.5f)) * vp.x;
  }
  if (axis == 2u) {
    T opt = (-conic.y * d.x) / conic.z;
    d.y = d.y - Mth<T>::floor((d.y - opt) / vp.y + K<T>(0.5f)) * vp.y;
  }
  return d;
}

// finalizeGaussianDepth.ts:18-68 with the default nodes of
// GaussianContextNodes.ts:127-132 (encoding 0: device depth) or the raw
// alpha-weighted scalar (encoding 1: rasterOutputDepth itself).
template <typename T>
static float finalize_depth(T wdepth, T trans, T near_, T far_, T alpha_thr, float invalid, int encoding) {
  T a = K<T>(1.0f) - trans;
  T out = K<T>(0.0f);
  if (a > 0) out = wdepth / a;
  bool scalar_valid = a > 0 && finiteT(wdepth) && finiteT(out) && out > 0;
  bool default_valid = scalar_valid && a > alpha_thr;
  float dev = invalid;
  if (scalar_valid && default_valid) {
    T enc;
    if (encoding == 0) {
      T vz = -out;
      enc = clampT(((near_ + vz) * far_) / ((far_ - near_) * vz), K<T>(0.0f), K<T>(1.0f));
    } else {
      enc = out;
    }
    if (finiteT(enc)) dev = (float)enc;
  }
  return dev;
}

}  // namespace

// ===========================================================================
// Exported C interface (ctypes).
extern "C" {

// Frame/scene descriptors shared with tests through ctypes.
struct GsoScene {
  uint32_t count;         // slot capacity
  uint32_t active_count;  // ordinals to project
  uint32_t sh_degree;     // 0..3
  uint32_t _pad;
  const float* means;          // count * 4 (xyz, objectId or -1)
  const uint32_t* shape;       // count * 2 compact f16 log-scales + opacity
  const uint32_t* rotations;   // count, oct101012
  const uint32_t* sh;          // count * C rgb8e8 + active tail (count)
};

struct GsoFrame {
  float projection[16];  // column-major
  float viewport[4];     // width, height, near, far
  float filter_variance;
  uint32_t boundary_axis;    // 0 clip, 1 repeat-x, 2 repeat-y
  uint32_t object_count;
  uint32_t depth_sort_mode;  // 0 float32, 1 packed16
  const float* objects;      // object_count * 40 floats
  float background[4];
  float transmittance_threshold;
  float depth_alpha_threshold;
  float invalid_depth_value;
  uint32_t antialias;          // 0 compensated, 1 classic
  uint32_t subpixel_culling;   // 1 on
  uint32_t raster_chunk_size;  // 0 = single workgroup path
  uint32_t max_splats_per_tile;  // 0 = uncapped
  uint32_t capacity;             // intersection record capacity
  uint32_t depth_encoding;       // 0 device depth, 1 raw scalar
  uint32_t attempt;
  uint32_t last_version;
  uint32_t reset_valid;
  uint32_t _pad;
};

struct GsoOutputs {
  // Per active ordinal (length active_count).
  float* proj_mean;      // *4
  float* proj_conic;     // *4
  float* proj_color;     // *4
  uint32_t* tile_counts;
  uint32_t* visible_offsets;
  // Per visible rank (length >= visible count).
  uint32_t* depth_sorted;    // *2 (key, ordinal)
  uint32_t* ordered_counts;
  uint32_t* intersection_offsets;
  uint32_t visible_state[4];
  uint32_t state[4];          // count, total, radix blocks, overflow
  uint32_t output_state[4];   // attempt, version, demand, overflow
  uint32_t* sorted_records;   // capacity * 2 (tile, ordinal)
  uint32_t* tile_offsets;     // tiles + 1
  float* rgba;                // width * height * 4 (left untouched on overflow)
  float* depth;               // width * height or null
  uint64_t checked;           // raster work counters (TileRasterizer.ts:545-546)
  uint64_t blended;
};

// --- codec and helper entry points used by the known-answer tests ---------
float gso_expf(float x) { return gsdm::expf_(x); }
float gso_logf(float x) { return gsdm::logf_(x); }
float gso_sinf(float x) { return gsdm::sinf_(x); }
float gso_cosf(float x) { return gsdm::cosf_(x); }
float gso_atan2f(float y, float x) { return gsdm::atan2f_(y, x); }
float gso_half_to_float(uint32_t h) { return gsdm::half_bits_to_float(h); }

void gso_decode_scale_opacity(uint32_t px, uint32_t py, float* out4) {
  V4<float> v = decode_compact_scale_opacity<float>(px, py);
  out4[0] = v.x; out4[1] = v.y; out4[2] = v.z; out4[3] = v.w;
}
void gso_decode_rotation(uint32_t packed, float* out4) {
  V4<float> v = decode_compact_rotation<float>(packed);
  out4[0] = v.x; out4[1] = v.y; out4[2] = v.z; out4[3] = v.w;
}
void gso_decode_sh(uint32_t packed, float* out3) {
  V3<float> v = decode_sh_rgb8e8<float>(packed);
  out3[0] = v.x; out3[1] = v.y; out3[2] = v.z;
}

uint32_t gso_f16_bits(float x);
uint32_t gso_zero_pixel_flag(const float* mean4, const float* conic4, uint32_t vw, uint32_t vh);

// engine.rs:1801-1891 encode_attributes (compact layout) for one splat: the
// packed means, scalesOpacity, rotation and C rgb8e8 SH words, on the CPU with
// libm like the Rust backend (checks the on-device packer).
void gso_pack_splat(const float* center, const float* scale, float opacity, const float* quat, const float* rgb,
                    const float* sh_rest, uint32_t C, uint32_t object_id, float* means4, uint32_t* shape2,
                    uint32_t* rot, uint32_t* sh);

// rust/gaussian-backend/src/engine.rs:1940-1949 pack_sh.
uint32_t gso_pack_sh(const float* rgb) {
  float mx = 0.0f;
  for (int i = 0; i < 3; ++i) mx = std::max(mx, fabsf(rgb[i]));
  if (mx == 0.0f) return 0u;
  float e = ceilf(log2f(mx));
  e = e < -126.0f ? -126.0f : (e > 127.0f ? 127.0f : e);
  int exponent = isnan(e) ? 0 : (int)e;  // Rust's `as i32` maps NaN to 0
  float mult = 127.0f / ldexpf(1.0f, exponent);
  uint32_t b[3];
  for (int i = 0; i < 3; ++i) {
    float q = floorf(rgb[i] * mult + 0.5f);
    q = q < -127.0f ? -127.0f : (q > 127.0f ? 127.0f : q);
    b[i] = (uint32_t)(int32_t)q & 255u;
  }
  return b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)(exponent + 127) << 24);
}

// IEEE binary16 bits of a float, round to nearest even (half::f16::from_f32).
static uint32_t f16_bits_rne(float x) {
  uint32_t b;
  memcpy(&b, &x, 4);
  const uint32_t sign = (b >> 16) & 0x8000u;
  const uint32_t ab = b & 0x7fffffffu;
  if (ab >= 0x7f800000u) return sign | (ab > 0x7f800000u ? 0x7e00u : 0x7c00u);  // NaN / inf
  if (ab >= 0x477ff000u) return sign | 0x7c00u;                                   // rounds past 65504
  if (ab < 0x33000001u) return sign;                                              // below half the smallest subnormal
  const int e = (int)(ab >> 23) - 127;
  uint32_t mant = (ab & 0x7fffffu) | 0x800000u;
  if (e < -14) {  // subnormal half
    const int shift = -e - 14 + 13;
    const uint32_t q = mant >> shift, rem = mant & ((1u << shift) - 1u), halfway = 1u << (shift - 1);
    return sign | (q + (rem > halfway || (rem == halfway && (q & 1u))));
  }
  const uint32_t q = mant >> 13, rem = mant & 0x1fffu;
  uint32_t h = ((uint32_t)(e + 15) << 10) | (q & 0x3ffu);
  if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) ++h;  // carries into the exponent correctly
  return sign | h;
}

// rust/vendor/spark-lib/src/splat_encode.rs:234-252 encode_quat_oct101012.
uint32_t gso_encode_oct101012(const float* q_in) {
  float q[4] = {q_in[0], q_in[1], q_in[2], q_in[3]};
  if (q[3] < 0.0f)
    for (int i = 0; i < 4; ++i) q[i] = -q[i];
  float theta = 2.0f * acosf(std::min(std::max(q[3], 0.0f), 1.0f));
  float s = sinf(theta * 0.5f);
  float axis[3];
  if (fabsf(s) < 1e-6f) {
    axis[0] = 1.0f; axis[1] = 0.0f; axis[2] = 0.0f;
  } else {
    for (int i = 0; i < 3; ++i) axis[i] = q[i] / s;
  }
  float sum = fabsf(axis[0]) + fabsf(axis[1]) + fabsf(axis[2]);
  float p[2] = {axis[0] / sum, axis[1] / sum};
  if (axis[2] < 0.0f) {
    float p0 = (1.0f - fabsf(p[1])) * (p[0] >= 0.0f ? 1.0f : -1.0f);
    float p1 = (1.0f - fabsf(p[0])) * (p[1] >= 0.0f ? 1.0f : -1.0f);
    p[0] = p0; p[1] = p1;
  }
  uint32_t uv[2];
  for (int i = 0; i < 2; ++i) {
    float v = (p[i] * 0.5f + 0.5f) * 1023.0f;
    v = v < 0.0f ? 0.0f : (v > 1023.0f ? 1023.0f : v);
    uv[i] = (uint32_t)roundf(v);
  }
  float r = theta / 3.14159265358979323846f * 4095.0f;
  r = r < 0.0f ? 0.0f : (r > 4095.0f ? 4095.0f : r);
  return ((uint32_t)roundf(r) << 20) | (uv[1] << 10) | uv[0];
}

uint32_t gso_f16_bits(float x) { return f16_bits_rne(x); }

// kernels/profileDiagnostics.ts:8-64 profileSubpixelCoverageWGSL for one
// projected splat (mean4, conic4 as the projection wrote them).
uint32_t gso_zero_pixel_flag(const float* m, const float* c, uint32_t vw, uint32_t vh) {
  if (m[3] < 0.0f) return 1u;
  if (m[3] <= 0.0f) return 0u;
  const float det = c[0] * c[2] - c[1] * c[1];
  if (det <= 1e-12f) return 0u;
  const float thr = gsdm::logf_(m[3] * 255.0f);
  if (thr <= 0.0f) return 0u;
  const float s00 = c[2] / det, s11 = c[0] / det;
  const float ex = sqrtf(std::max((2.0f * thr) * s00, 0.0f)), ey = sqrtf(std::max((2.0f * thr) * s11, 0.0f));
  if (ex * 2.0f > 1.0f || ey * 2.0f > 1.0f) return 0u;
  const int x0 = std::max((int)ceilf((m[0] - ex) - 0.5f), 0), y0 = std::max((int)ceilf((m[1] - ey) - 0.5f), 0);
  const int x1 = std::min((int)floorf((m[0] + ex) - 0.5f), (int)vw - 1);
  const int y1 = std::min((int)floorf((m[1] + ey) - 0.5f), (int)vh - 1);
  bool has = false;
  for (int py = y0; py <= y1; ++py)
    for (int px = x0; px <= x1; ++px) {
      const float dx = ((float)px + 0.5f) - m[0], dy = ((float)py + 0.5f) - m[1];
      const float sigma = 0.5f * ((c[0] * dx * dx + 2.0f * c[1] * dx * dy) + c[2] * dy * dy);
      if (sigma <= thr) has = true;
    }
  return has ? 0u : 1u;
}

void gso_pack_splat(const float* center, const float* scale, float opacity, const float* quat, const float* rgb,
                    const float* sh_rest, uint32_t C, uint32_t object_id, float* means4, uint32_t* shape2,
                    uint32_t* rot, uint32_t* sh) {
  means4[0] = center[0]; means4[1] = center[1]; means4[2] = center[2]; means4[3] = (float)object_id;
  shape2[0] = f16_bits_rne(logf(scale[0])) | (f16_bits_rne(logf(scale[1])) << 16);
  shape2[1] = f16_bits_rne(logf(scale[2])) | (f16_bits_rne(opacity) << 16);
  const float inv = 1.0f / sqrtf(((quat[0] * quat[0] + quat[1] * quat[1]) + quat[2] * quat[2]) + quat[3] * quat[3]);
  const float q[4] = {quat[0] * inv, quat[1] * inv, quat[2] * inv, quat[3] * inv};
  *rot = gso_encode_oct101012(q);
  const float k = 0.28209479177387814f;
  const float dc[3] = {(rgb[0] - 0.5f) / k, (rgb[1] - 0.5f) / k, (rgb[2] - 0.5f) / k};
  sh[0] = gso_pack_sh(dc);
  for (uint32_t c = 1; c < C; ++c) sh[c] = gso_pack_sh(sh_rest + 3 * (size_t)(c - 1));
}

void gso_view_covariance(const float* scale, const float* rot, const float* mv16, float* out9) {
  M4<float> mv = load_m4<float>(mv16);
  M3<float> c = view_covariance<float>({scale[0], scale[1], scale[2]}, {rot[0], rot[1], rot[2], rot[3]}, mv);
  for (int k = 0; k < 3; ++k) {
    out9[3 * k + 0] = c.c[k].x; out9[3 * k + 1] = c.c[k].y; out9[3 * k + 2] = c.c[k].z;
  }
}

static void store_m4(const M4<float>& m, float* out16) {
  for (int c = 0; c < 4; ++c) {
    out16[4 * c + 0] = m.c[c].x; out16[4 * c + 1] = m.c[c].y;
    out16[4 * c + 2] = m.c[c].z; out16[4 * c + 3] = m.c[c].w;
  }
}

void gso_projection_result(const float* center, float depth, const float* cov3, float filter, float* out16) {
  store_m4(projection_result<float>({center[0], center[1]}, depth, {cov3[0], cov3[1], cov3[2]}, filter), out16);
}

void gso_perspective_projection(const float* view3, const float* cov9, const float* proj16, const float* vp4,
                                float filter, float* out16) {
  M3<float> cv;
  for (int k = 0; k < 3; ++k) cv.c[k] = {cov9[3 * k], cov9[3 * k + 1], cov9[3 * k + 2]};
  store_m4(perspective_projection<float>({view3[0], view3[1], view3[2]}, cv, load_m4<float>(proj16),
                                         {vp4[0], vp4[1], vp4[2], vp4[3]}, filter),
           out16);
}

int gso_projection_is_valid(const float* p16) { return projection_is_valid<float>(load_m4<float>(p16)) ? 1 : 0; }

void gso_boundary_delta(const float* pixel, const float* center, const float* conic, const float* vp, uint32_t axis,
                        float* out2) {
  V2<float> d = boundary_delta<float>({pixel[0], pixel[1]}, {center[0], center[1]}, {conic[0], conic[1], conic[2]},
                                      {vp[0], vp[1]}, axis);
  out2[0] = d.x; out2[1] = d.y;
}

int gso_boundary_tile_hit(const float* center, const float* conic, float thr, const float* radius, int tx, int ty,
                          const float* vp, uint32_t axis) {
  return boundary_tile_hit<float>({center[0], center[1]}, {conic[0], conic[1], conic[2]}, thr,
                                  {radius[0], radius[1]}, tx, ty, {vp[0], vp[1]}, axis) ? 1 : 0;
}

uint32_t gso_count_tiles(const float* center, const float* conic, float thr, const float* radius, int tminx,
                         int tminy, int tmaxx, int tmaxy, const float* vp, uint32_t axis) {
  return count_tiles<float>({center[0], center[1]}, {conic[0], conic[1], conic[2]}, thr, {radius[0], radius[1]},
                            tminx, tminy, tmaxx, tmaxy, {vp[0], vp[1]}, axis);
}

int gso_subpixel_has_sample(const float* center, const float* conic, float thr, const float* extent, uint32_t vw,
                            uint32_t vh, uint32_t axis) {
  return subpixel_has_sample<float>({center[0], center[1]}, {conic[0], conic[1], conic[2]}, thr,
                                    {extent[0], extent[1]}, vw, vh, axis) ? 1 : 0;
}

float gso_finalize_depth(float wdepth, float trans, float near_, float far_, float alpha_thr, float invalid,
                         int encoding) {
  return finalize_depth<float>(wdepth, trans, near_, far_, alpha_thr, invalid, encoding);
}

uint32_t gso_tile_sort_bits(uint32_t tiles) {
  // TiledGaussianPipeline.ts:431,442-445: capacity = 2^ceil(log2 tiles),
  // bits = max(1, ceil(log2(max(2, capacity + 1)))).
  uint32_t cap = 1;
  while (cap < tiles) cap <<= 1;
  uint32_t v = std::max<uint32_t>(2, cap + 1);
  uint32_t bits = 0;
  while ((1ull << bits) < v) ++bits;
  return std::max<uint32_t>(1, bits);
}

int gso_num_threads(void) {
#if defined(_OPENMP)
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"

namespace {

// ProjectionStage.ts:385-649: the projection thread body for one ordinal.
template <typename T>
static void project_one(const GsoScene& sc, const GsoFrame& fr, uint32_t gid, float* mean4, float* conic4,
                        float* color4, uint32_t* count_out, T* dmean, T* dconic) {
  uint32_t C = (sc.sh_degree + 1) * (sc.sh_degree + 1);
  *count_out = 0;
  mean4[0] = mean4[1] = mean4[2] = mean4[3] = 0.0f;
  if (dmean) dmean[0] = dmean[1] = dmean[2] = dmean[3] = 0;
  uint32_t slot = sc.sh[(size_t)sc.count * C + gid];
  if (slot >= sc.count) return;  // out-of-range tail entries never draw
  const float* mo = sc.means + 4 * (size_t)slot;
  if (mo[3] < 0.0f) return;  // ProjectionStage.ts:408-410
  uint32_t obj = (uint32_t)mo[3];
  V4<T> so = decode_compact_scale_opacity<T>(sc.shape[2 * (size_t)slot], sc.shape[2 * (size_t)slot + 1]);
  V4<T> rot = decode_compact_rotation<T>(sc.rotations[slot]);
  if (obj >= fr.object_count) return;  // unwritten object rows are zero (invisible)
  const float* ot = fr.objects + 40 * (size_t)obj;
  M4<T> mv = load_m4<T>(ot + 16);
  V3<T> cam = {(T)ot[32], (T)ot[33], (T)ot[34]};
  if (!(ot[36] > 0.0f)) return;  // ProjectionStage.ts:445-450
  V3<T> p = {(T)mo[0], (T)mo[1], (T)mo[2]};
  V3<T> vdir = normalize3<T>({p.x - cam.x, p.y - cam.y, p.z - cam.z});
  V4<T> vpos = mul4v(mv, V4<T>{p.x, p.y, p.z, K<T>(1.0f)});
  M3<T> cv = view_covariance<T>({so.x, so.y, so.z}, rot, mv);
  M4<T> proj = load_m4<T>(fr.projection);
  V4<T> vp = {(T)fr.viewport[0], (T)fr.viewport[1], (T)fr.viewport[2], (T)fr.viewport[3]};
  M4<T> pr = perspective_projection<T>({vpos.x, vpos.y, vpos.z}, cv, proj, vp, (T)fr.filter_variance);
  if (!projection_is_valid(pr)) return;
  V2<T> center = {pr.c[0].x, pr.c[0].y};
  T depth = pr.c[0].z;
  V3<T> conic = {pr.c[1].x, pr.c[1].y, pr.c[1].z};
  T det = pr.c[1].w;
  V3<T> cov = {pr.c[2].x, pr.c[2].y, pr.c[2].z};
  T odet = pr.c[2].w;
  T op = clampT(so.w, K<T>(0.0f), K<T>(1.0f));
  if (fr.antialias == 0) op = op * Mth<T>::sqrt(clampT(odet / det, K<T>(0.0f), K<T>(1.0f)));
  if (op < K<T>((float)(1.0 / 255.0)) || op != op) return;
  T thr = Mth<T>::log(op * K<T>(255.0f));
  T ex = Mth<T>::sqrt((thr * K<T>(2.0f)) * clampT(cov.x, K<T>(1e-12f), K<T>(1e4f)));
  T ey = Mth<T>::sqrt((thr * K<T>(2.0f)) * clampT(cov.z, K<T>(1e-12f), K<T>(1e4f)));
  T rx = Mth<T>::ceil(ex), ry = Mth<T>::ceil(ey);
  if (rx <= 0 || ry <= 0) return;
  V2<T> bmin = {center.x - rx, center.y - ry};
  V2<T> bmax = {center.x + rx, center.y + ry};
  if ((fr.boundary_axis != 1u && (bmax.x < 0 || bmin.x >= vp.x)) ||
      (fr.boundary_axis != 2u && (bmax.y < 0 || bmin.y >= vp.y)))
    return;
  if (fr.subpixel_culling) {
    if (!subpixel_has_sample<T>(center, conic, thr, {ex, ey}, (uint32_t)fr.viewport[0], (uint32_t)fr.viewport[1],
                                fr.boundary_axis)) {
      mean4[0] = (float)center.x; mean4[1] = (float)center.y; mean4[2] = (float)depth; mean4[3] = -1.0f;
      if (dmean) { dmean[0] = center.x; dmean[1] = center.y; dmean[2] = depth; dmean[3] = -1; }
      return;
    }
  }
  int tiles_x = (int)ceilf(fr.viewport[0] / (float)TILE);
  int tiles_y = (int)ceilf(fr.viewport[1] / (float)TILE);
  T mtx = (T)(float)(tiles_x - 1), mty = (T)(float)(tiles_y - 1);
  int tminx = (int)clampT(Mth<T>::floor(bmin.x / K<T>((float)TILE)), K<T>(0.0f), mtx);
  int tminy = (int)clampT(Mth<T>::floor(bmin.y / K<T>((float)TILE)), K<T>(0.0f), mty);
  int tmaxx = (int)clampT(Mth<T>::floor(bmax.x / K<T>((float)TILE)), K<T>(0.0f), mtx);
  int tmaxy = (int)clampT(Mth<T>::floor(bmax.y / K<T>((float)TILE)), K<T>(0.0f), mty);
  if (fr.boundary_axis == 1u) { tminx = 0; tmaxx = tiles_x - 1; }
  if (fr.boundary_axis == 2u) { tminy = 0; tmaxy = tiles_y - 1; }
  V3<T> color = eval_sh_rgb8e8<T>(sc.sh + (size_t)slot * C, sc.sh_degree, vdir);
  uint32_t cnt = count_tiles<T>(center, conic, thr, {rx, ry}, tminx, tminy, tmaxx, tmaxy, {vp.x, vp.y},
                                fr.boundary_axis);
  if (cnt == 0) return;
  mean4[0] = (float)center.x; mean4[1] = (float)center.y; mean4[2] = (float)depth; mean4[3] = (float)op;
  conic4[0] = (float)conic.x; conic4[1] = (float)conic.y; conic4[2] = (float)conic.z;
  conic4[3] = (float)(rx + ry * K<T>(512.0f));
  color4[0] = (float)color.x; color4[1] = (float)color.y; color4[2] = (float)color.z;
  color4[3] = gsdm::u2f(slot ^ ACTIVE_TAG);
  if (dmean) { dmean[0] = center.x; dmean[1] = center.y; dmean[2] = depth; dmean[3] = op; }
  if (dconic) { dconic[0] = conic.x; dconic[1] = conic.y; dconic[2] = conic.z; dconic[3] = rx + ry * K<T>(512.0f); }
  *count_out = cnt;
}

static inline uint32_t sat_add(uint32_t a, uint32_t b) { return a + std::min(b, 0xffffffffu - a); }

// visibility.ts:37-61 depth key.
static inline uint32_t depth_key(float depth, const GsoFrame& fr) {
  if (fr.depth_sort_mode == 0) return gsdm::f2u(depth);
  float t = gsdm::clampf_((depth - fr.viewport[2]) / (fr.viewport[3] - fr.viewport[2]), 0.0f, 1.0f);
  return (uint32_t)gsdm::round_even_small(t * 65535.0f);
}

// TileRasterizer.ts:547-746: blend one pixel over samples [s0, s1) of a tile.
template <typename T>
static void blend_span(const uint32_t* recs, uint32_t begin, uint32_t source_count, uint32_t raster_count,
                       uint32_t s0, uint32_t s1, bool capped, const T* mean, const T* conic, const float* color,
                       T pxc, T pyc, const GsoFrame& fr, T* acc, T* trans, T* wdepth, uint64_t* checked,
                       uint64_t* blended) {
  const T tthr = (T)fr.transmittance_threshold;
  V2<T> vp = {(T)fr.viewport[0], (T)fr.viewport[1]};
  for (uint32_t s = s0; s < s1; ++s) {
    uint32_t src = s;
    if (capped) src = (uint32_t)floorf((((float)s + 0.5f) * (float)source_count) / (float)raster_count);
    uint32_t g = recs[2 * (size_t)(begin + src) + 1];
    const T* m = mean + 4 * (size_t)g;
    const T* c = conic + 4 * (size_t)g;
    ++*checked;
    T thr = Mth<T>::log(m[3] * K<T>(255.0f));
    V2<T> d = boundary_delta<T>({pxc, pyc}, {m[0], m[1]}, {c[0], c[1], c[2]}, vp, fr.boundary_axis);
    T power = ((c[0] * (d.x * d.x) + ((c[1] * K<T>(2.0f)) * d.x) * d.y) + c[2] * (d.y * d.y)) * K<T>(-0.5f);
    if (power > 0 || power < -thr) continue;
    T alpha = clampT(m[3] * Mth<T>::exp(power), K<T>(0.0f), K<T>(0.99f));
    if (alpha < K<T>((float)(1.0 / 255.0))) continue;
    const float* col = color + 4 * (size_t)g;
    T contrib = *trans * alpha;
    acc[0] = acc[0] + (T)col[0] * contrib;
    acc[1] = acc[1] + (T)col[1] * contrib;
    acc[2] = acc[2] + (T)col[2] * contrib;
    *wdepth = *wdepth + m[2] * contrib;
    ++*blended;
    *trans = *trans * (K<T>(1.0f) - alpha);
    if (*trans < tthr) break;
  }
}

template <typename T>
static void raster_all(const GsoFrame& fr, uint32_t tiles_x, uint32_t tiles_y, const uint32_t* recs,
                       const uint32_t* offsets, const T* mean, const T* conic, const float* color, float* rgba,
                       float* depth_out, uint64_t* checked_out, uint64_t* blended_out) {
  const uint32_t W = (uint32_t)fr.viewport[0], H = (uint32_t)fr.viewport[1];
  const uint32_t ntile = tiles_x * tiles_y;
  const T tthr = (T)fr.transmittance_threshold;
  const T bga = clampT((T)fr.background[3], K<T>(0.0f), K<T>(1.0f));
  uint64_t checked = 0, blended = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : checked, blended)
  for (int64_t t = 0; t < (int64_t)ntile; ++t) {
    uint32_t begin = offsets[t], end = offsets[t + 1];
    uint32_t source_count = end - begin;
    bool capped = fr.max_splats_per_tile != 0;
    uint32_t raster_count = capped ? std::min(source_count, fr.max_splats_per_tile) : source_count;
    bool chunked = fr.raster_chunk_size != 0 && raster_count > fr.raster_chunk_size;
    uint32_t tx = (uint32_t)t % tiles_x, ty = (uint32_t)t / tiles_x;
    for (uint32_t ly = 0; ly < (uint32_t)TILE; ++ly) {
      for (uint32_t lx = 0; lx < (uint32_t)TILE; ++lx) {
        uint32_t px = tx * TILE + lx, py = ty * TILE + ly;
        if (px >= W || py >= H) continue;
        T pxc = (T)(float)px + K<T>(0.5f), pyc = (T)(float)py + K<T>(0.5f);
        T acc[3] = {0, 0, 0}, trans = K<T>(1.0f), wd = 0;
        uint64_t ck = 0, bl = 0;
        if (!chunked) {
          blend_span<T>(recs, begin, source_count, raster_count, 0, raster_count, capped, mean, conic, color, pxc,
                        pyc, fr, acc, &trans, &wd, &ck, &bl);
        } else {
          // TileRasterizer.ts:828-873: independent chunk partials, ordered composite.
          uint32_t nchunk = (raster_count + fr.raster_chunk_size - 1) / fr.raster_chunk_size;
          for (uint32_t ch = 0; ch < nchunk; ++ch) {
            uint32_t s0 = ch * fr.raster_chunk_size;
            uint32_t s1 = std::min(s0 + fr.raster_chunk_size, raster_count);
            T pa[3] = {0, 0, 0}, pt = K<T>(1.0f), pd = 0;
            blend_span<T>(recs, begin, source_count, raster_count, s0, s1, capped, mean, conic, color, pxc, pyc,
                          fr, pa, &pt, &pd, &ck, &bl);
            acc[0] = acc[0] + pa[0] * trans;
            acc[1] = acc[1] + pa[1] * trans;
            acc[2] = acc[2] + pa[2] * trans;
            wd = wd + pd * trans;
            trans = trans * pt;
            if (trans < tthr) break;
          }
        }
        checked += ck;
        blended += bl;
        // TileRasterizer.ts:930-948 storeFinalPixel.
        size_t o = (size_t)py * W + px;
        for (int k = 0; k < 3; ++k) acc[k] = acc[k] + ((T)fr.background[k] * trans) * bga;
        rgba[4 * o + 0] = (float)acc[0];
        rgba[4 * o + 1] = (float)acc[1];
        rgba[4 * o + 2] = (float)acc[2];
        rgba[4 * o + 3] = (float)(K<T>(1.0f) - trans * (K<T>(1.0f) - bga));
        if (depth_out)
          depth_out[o] = finalize_depth<T>(wd, trans, (T)fr.viewport[2], (T)fr.viewport[3],
                                           (T)fr.depth_alpha_threshold, fr.invalid_depth_value,
                                           (int)fr.depth_encoding);
      }
    }
  }
  *checked_out = checked;
  *blended_out = blended;
}

// The whole pass (TiledGaussianPipeline.ts:324-341) for one frame.
template <typename T> static int render(const GsoScene& sc, const GsoFrame& fr, GsoOutputs* out) {
  const uint32_t N = sc.active_count;
  const uint32_t tiles_x = (uint32_t)ceilf(fr.viewport[0] / (float)TILE);
  const uint32_t tiles_y = (uint32_t)ceilf(fr.viewport[1] / (float)TILE);
  const uint32_t ntile = tiles_x * tiles_y;
  std::vector<T> dmean(4 * (size_t)N, 0), dconic(4 * (size_t)N, 0);
  const bool twin = sizeof(T) == 8;

  // Projection (K1).
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < (int64_t)N; ++g) {
    project_one<T>(sc, fr, (uint32_t)g, out->proj_mean + 4 * g, out->proj_conic + 4 * g, out->proj_color + 4 * g,
                   out->tile_counts + g, twin ? dmean.data() + 4 * g : nullptr,
                   twin ? dconic.data() + 4 * g : nullptr);
  }
  if (!twin) {
    for (size_t i = 0; i < 4 * (size_t)N; ++i) {
      dmean[i] = (T)out->proj_mean[i];
      dconic[i] = (T)out->proj_conic[i];
    }
  }

  // Visibility scan + compaction (scan.ts:78-83, visibility.ts:9-61).
  uint32_t V = 0;
  for (uint32_t g = 0; g < N; ++g) {
    out->visible_offsets[g] = V;
    if (out->proj_mean[4 * (size_t)g + 3] > 0.0f) V = sat_add(V, 1u);
  }
  std::vector<uint32_t> rec_key(V), rec_id(V);
  for (uint32_t g = 0; g < N; ++g) {
    if (!(out->proj_mean[4 * (size_t)g + 3] > 0.0f)) continue;
    uint32_t o = out->visible_offsets[g];
    rec_key[o] = depth_key(out->proj_mean[4 * (size_t)g + 2], fr);
    rec_id[o] = g;
  }
  out->visible_state[0] = V;
  out->visible_state[1] = V;
  out->visible_state[2] = (V + 1023u) / 1024u;
  out->visible_state[3] = 0;

  // Depth sort: stable by key (RadixSorter.ts:50-223 is a stable LSD sort).
  std::vector<uint32_t> order(V);
  for (uint32_t i = 0; i < V; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return rec_key[a] < rec_key[b]; });
  for (uint32_t r = 0; r < V; ++r) {
    out->depth_sorted[2 * (size_t)r] = rec_key[order[r]];
    out->depth_sorted[2 * (size_t)r + 1] = rec_id[order[r]];
  }

  // Depth-ordered counts + intersection scan + prepare_dispatch
  // (visibility.ts:63-76, scan.ts, intersections.ts:10-41).
  uint32_t run = 0;
  for (uint32_t r = 0; r < V; ++r) {
    uint32_t c = out->tile_counts[out->depth_sorted[2 * (size_t)r + 1]];
    out->ordered_counts[r] = c;
    out->intersection_offsets[r] = run;
    run = sat_add(run, c);
  }
  uint32_t total = run;
  bool overflow = total > fr.capacity;
  uint32_t count = overflow ? 0u : total;
  out->state[0] = count;
  out->state[1] = total;
  out->state[2] = (count + 1023u) / 1024u;
  out->state[3] = overflow ? 1u : 0u;
  // intersections.ts:114-133 prepare_intersection_output.
  uint32_t last_version = fr.reset_valid ? 0u : fr.last_version;
  out->output_state[0] = fr.attempt;
  out->output_state[1] = overflow ? last_version : fr.attempt;
  out->output_state[2] = total;
  out->output_state[3] = overflow ? 1u : 0u;

  // Emission (intersections.ts:43-111), only for a complete set.
  const uint32_t sentinel = ntile;
  std::vector<uint32_t> erec(2 * (size_t)count);
  if (!overflow) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t r = 0; r < (int64_t)V; ++r) {
      uint32_t g = out->depth_sorted[2 * (size_t)r + 1];
      // Emission re-derives the tile test from the projected buffers, like the
      // WGSL kernel; the FP64 twin reads its own double projection.
      const T* m = dmean.data() + 4 * (size_t)g;
      const T* c = dconic.data() + 4 * (size_t)g;
      uint32_t packed = (uint32_t)c[3];
      T rx = (T)(float)(packed % 512u), ry = (T)(float)(packed / 512u);
      T thr = Mth<T>::log(m[3] * K<T>(255.0f));
      const T ts = K<T>((float)TILE);
      T mtx = (T)(float)((int)tiles_x - 1), mty = (T)(float)((int)tiles_y - 1);
      int tminx = (int)clampT(Mth<T>::floor((m[0] - rx) / ts), K<T>(0.0f), mtx);
      int tminy = (int)clampT(Mth<T>::floor((m[1] - ry) / ts), K<T>(0.0f), mty);
      int tmaxx = (int)clampT(Mth<T>::floor((m[0] + rx) / ts), K<T>(0.0f), mtx);
      int tmaxy = (int)clampT(Mth<T>::floor((m[1] + ry) / ts), K<T>(0.0f), mty);
      if (fr.boundary_axis == 1u) { tminx = 0; tmaxx = (int)tiles_x - 1; }
      if (fr.boundary_axis == 2u) { tminy = 0; tmaxy = (int)tiles_y - 1; }
      uint32_t reserved = out->ordered_counts[r];
      uint32_t base = out->intersection_offsets[r];
      uint32_t local = 0;
      for (int ty = tminy; ty <= tmaxy; ++ty)
        for (int tx = tminx; tx <= tmaxx; ++tx)
          if (boundary_tile_hit<T>({m[0], m[1]}, {c[0], c[1], c[2]}, thr, {rx, ry}, tx, ty,
                                   {(T)fr.viewport[0], (T)fr.viewport[1]}, fr.boundary_axis)) {
            if (local < reserved && base + local < fr.capacity) {
              erec[2 * (size_t)(base + local)] = (uint32_t)ty * tiles_x + (uint32_t)tx;
              erec[2 * (size_t)(base + local) + 1] = g;
            }
            ++local;
          }
      for (uint32_t pad = local; pad < reserved; ++pad)
        if (base + pad < fr.capacity) {
          erec[2 * (size_t)(base + pad)] = sentinel;
          erec[2 * (size_t)(base + pad) + 1] = g;
        }
    }
  }

  // Tile sort: stable by tile id (counting sort; tile ids <= sentinel).
  std::vector<uint32_t> hist((size_t)ntile + 2, 0);
  for (uint32_t i = 0; i < count; ++i) hist[erec[2 * (size_t)i] + 1]++;
  for (size_t t = 1; t < hist.size(); ++t) hist[t] += hist[t - 1];
  for (uint32_t i = 0; i < count; ++i) {
    uint32_t d = hist[erec[2 * (size_t)i]]++;
    out->sorted_records[2 * (size_t)d] = erec[2 * (size_t)i];
    out->sorted_records[2 * (size_t)d + 1] = erec[2 * (size_t)i + 1];
  }

  // Tile ranges (tileOffsets.ts:4-128): first index per tile, suffix-min.
  uint32_t* off = out->tile_offsets;
  for (uint32_t t = 0; t <= ntile; ++t) off[t] = t == ntile ? count : 0xffffffffu;
  for (uint32_t i = 0; i < count; ++i) {
    uint32_t tile = out->sorted_records[2 * (size_t)i];
    if (tile <= ntile && (i == 0 || out->sorted_records[2 * (size_t)(i - 1)] != tile)) off[tile] = i;
  }
  for (int64_t t = (int64_t)ntile - 1; t >= 0; --t) off[t] = std::min(off[t], off[t + 1]);

  // Raster (skipped on overflow: the raster dispatch is zeroed).
  out->checked = out->blended = 0;
  if (!overflow)
    raster_all<T>(fr, tiles_x, tiles_y, out->sorted_records, off, dmean.data(), dconic.data(), out->proj_color,
                  out->rgba, out->depth, &out->checked, &out->blended);
  return 0;
}

}  // namespace

extern "C" {

// precision: 0 = FP32 restatement, 1 = FP64 twin.
int gso_render(const GsoScene* scene, const GsoFrame* frame, GsoOutputs* out, int precision) {
  if (precision == 1) return render<double>(*scene, *frame, out);
  return render<float>(*scene, *frame, out);
}

}  // extern "C"
