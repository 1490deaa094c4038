/*
 * Node-API addon: the GaussianPass data path of the reference
 * (src/renderer/GaussianPass.ts:710-805 driving TiledGaussianPipeline,
 * src/renderer/pipeline/TiledGaussianPipeline.ts:65-425) over the gs3d C ABI
 * (include/gs3d.h). The TypeScript shim in index.ts gives it the reference's
 * class surface; the Store, LOD selection and streaming protocol stay in
 * TypeScript and hand their packed buffers to createScene / updateScene.
 *
 * Threading follows the reference: every call returns without waiting for
 * the GPU. render() only enqueues work on the pipeline's own CUDA stream.
 * readStats() and readImage() return Promises; their copies are enqueued on
 * that stream and a libuv worker waits for them, so the JS thread never
 * blocks (GaussianPass.ts:1019-1079 keeps one output-state read-back in
 * flight the same way). Each pipeline owns its colour and depth targets.
 *
 * Errors: RangeError for GS3D_ERROR_RANGE, TypeError for
 * GS3D_ERROR_INVALID_ARGUMENT, Error otherwise, with the pipeline's message.
 */
#include <node_api.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "gs3d.h"

#define CHECK_NAPI(env, call)                                   \
  do {                                                          \
    if ((call) != napi_ok) {                                    \
      napi_throw_error((env), NULL, "Node-API call failed: " #call); \
      return NULL;                                              \
    }                                                           \
  } while (0)

/* ------------------------------------------------------------------------ */
/* Helpers */

static napi_value throw_status(napi_env env, gs3d_status s, gs3d_pipeline* p) {
  const char* msg = p ? gs3d_pipeline_last_error(p) : "";
  if (!msg || !msg[0]) msg = gs3d_status_string(s);
  if (s == GS3D_ERROR_RANGE) napi_throw_range_error(env, NULL, msg);
  else if (s == GS3D_ERROR_INVALID_ARGUMENT) napi_throw_type_error(env, NULL, msg);
  else napi_throw_error(env, NULL, msg);
  return NULL;
}

static napi_value throw_cuda(napi_env env, cudaError_t e, const char* what) {
  char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  napi_throw_error(env, NULL, buf);
  return NULL;
}

static int get_u32(napi_env env, napi_value obj, const char* name, uint32_t* out) {
  napi_value v;
  if (napi_get_named_property(env, obj, name, &v) != napi_ok) return 0;
  return napi_get_value_uint32(env, v, out) == napi_ok;
}

static int get_f64(napi_env env, napi_value obj, const char* name, double* out) {
  napi_value v;
  if (napi_get_named_property(env, obj, name, &v) != napi_ok) return 0;
  return napi_get_value_double(env, v, out) == napi_ok;
}

/* The bytes of a typed array argument. */
static int typed_bytes(napi_env env, napi_value v, void** data, size_t* bytes) {
  bool is_typed = false;
  if (napi_is_typedarray(env, v, &is_typed) != napi_ok || !is_typed) return 0;
  napi_typedarray_type type;
  size_t length = 0, offset = 0;
  napi_value buffer;
  if (napi_get_typedarray_info(env, v, &type, &length, data, &buffer, &offset) != napi_ok) return 0;
  size_t elem = 1;
  switch (type) {
    case napi_int16_array: case napi_uint16_array: elem = 2; break;
    case napi_int32_array: case napi_uint32_array: case napi_float32_array: elem = 4; break;
    case napi_float64_array: case napi_bigint64_array: case napi_biguint64_array: elem = 8; break;
    default: elem = 1; break;
  }
  *bytes = length * elem;
  return 1;
}

static int typed_field(napi_env env, napi_value obj, const char* name, void** data, size_t* bytes) {
  napi_value v;
  if (napi_get_named_property(env, obj, name, &v) != napi_ok) return 0;
  return typed_bytes(env, v, data, bytes);
}

static napi_value make_u32(napi_env env, uint32_t v) {
  napi_value r;
  napi_create_uint32(env, v, &r);
  return r;
}

static napi_value make_f64(napi_env env, double v) {
  napi_value r;
  napi_create_double(env, v, &r);
  return r;
}

static napi_value make_ptr(napi_env env, const void* p) {
  napi_value r;
  napi_create_bigint_uint64(env, (uint64_t)(uintptr_t)p, &r);
  return r;
}

/* ------------------------------------------------------------------------ */
/* Scenes: device copies of a store's packed buffers (GaussianData.ts:10-33,
 * 108-138), owned by the addon and leased to pipelines. */

typedef struct Scene {
  void* means;  /* float32[count][4] */
  void* shape;  /* uint32[count][2] */
  void* rot;    /* uint32[count] */
  void* sh;     /* uint32[count * C + count]: rgb8e8 + active-slot tail */
  size_t bytes[4];
  gs3d_gaussian_data data;
} Scene;

static void scene_free(Scene* s) {
  if (!s) return;
  cudaFree(s->means);
  cudaFree(s->shape);
  cudaFree(s->rot);
  cudaFree(s->sh);
  free(s);
}

static void scene_finalize(napi_env env, void* data, void* hint) {
  (void)env;
  (void)hint;
  scene_free((Scene*)data);
}

static const char* const kSceneFields[4] = {"means", "scalesOpacity", "rotations", "shCoefficients"};

/* createScene({means, scalesOpacity, rotations, shCoefficients, count,
 * activeCount, shDegree}) -> opaque scene. */
static napi_value create_scene(napi_env env, napi_callback_info info) {
  size_t argc = 1;
  napi_value argv[1];
  CHECK_NAPI(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  if (argc < 1) return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
  Scene* s = (Scene*)calloc(1, sizeof(Scene));
  if (!s) return throw_status(env, GS3D_ERROR_OUT_OF_MEMORY, NULL);
  uint32_t count = 0, active = 0, degree = 0;
  if (!get_u32(env, argv[0], "count", &count) || !get_u32(env, argv[0], "activeCount", &active) ||
      !get_u32(env, argv[0], "shDegree", &degree)) {
    free(s);
    return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
  }
  void** slots[4] = {&s->means, &s->shape, &s->rot, &s->sh};
  for (int i = 0; i < 4; ++i) {
    void* host = NULL;
    size_t bytes = 0;
    if (!typed_field(env, argv[0], kSceneFields[i], &host, &bytes) || bytes == 0) {
      scene_free(s);
      return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
    }
    cudaError_t e = cudaMalloc(slots[i], bytes);
    if (e == cudaSuccess) e = cudaMemcpy(*slots[i], host, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      scene_free(s);
      return throw_cuda(env, e, "uploading the packed Gaussian buffers");
    }
    s->bytes[i] = bytes;
  }
  s->data.count = count;
  s->data.active_count = active;
  s->data.sh_degree = degree;
  s->data.means = s->means;
  s->data.scales_opacity = s->shape;
  s->data.rotations = s->rot;
  s->data.sh_coefficients = s->sh;
  napi_value obj;
  CHECK_NAPI(env, napi_create_object(env, &obj));
  CHECK_NAPI(env, napi_wrap(env, obj, s, scene_finalize, NULL, NULL));
  return obj;
}

/* updateScene(scene, field, byteOffset, typedArray[, activeCount]): writes a
 * streamed patch (slots or the active-slot tail) into the device copy. */
static napi_value update_scene(napi_env env, napi_callback_info info) {
  size_t argc = 5;
  napi_value argv[5];
  CHECK_NAPI(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  if (argc < 4) return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
  Scene* s = NULL;
  CHECK_NAPI(env, napi_unwrap(env, argv[0], (void**)&s));
  uint32_t field = 0;
  double offset = 0;
  void* host = NULL;
  size_t bytes = 0;
  if (napi_get_value_uint32(env, argv[1], &field) != napi_ok || field > 3 ||
      napi_get_value_double(env, argv[2], &offset) != napi_ok || offset < 0 ||
      !typed_bytes(env, argv[3], &host, &bytes))
    return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
  if ((size_t)offset + bytes > s->bytes[field]) return throw_status(env, GS3D_ERROR_RANGE, NULL);
  void* dst[4] = {s->means, s->shape, s->rot, s->sh};
  cudaError_t e = cudaMemcpy((char*)dst[field] + (size_t)offset, host, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return throw_cuda(env, e, "writing a scene patch");
  if (argc >= 5) {
    uint32_t active = 0;
    if (napi_get_value_uint32(env, argv[4], &active) != napi_ok || active > s->data.count)
      return throw_status(env, GS3D_ERROR_RANGE, NULL);
    s->data.active_count = active;
  }
  return NULL;
}

/* ------------------------------------------------------------------------ */
/* Pipelines */

typedef struct Pipeline {
  gs3d_pipeline* p;
  cudaStream_t stream;
  napi_ref scene_ref;       /* the leased scene (GaussianData.retain) */
  Scene* scene;
  void* color;              /* rgba16f, owned by this pipeline */
  float* depth;             /* float32 or NULL (outputDepth = false) */
  size_t color_bytes, depth_bytes;
  uint32_t width, height, output_depth;
  gs3d_camera camera;
  float* objects;           /* host copy of the object table */
  uint32_t object_cap;
  int stats_pending, image_pending;
  void* pinned;             /* read-back of the colour target */
  size_t pinned_bytes;
} Pipeline;

static void pipeline_release(Pipeline* pl) {
  if (!pl) return;
  if (pl->stream) cudaStreamSynchronize(pl->stream);
  gs3d_pipeline_destroy(pl->p);
  pl->p = NULL;
  cudaFree(pl->color);
  cudaFree(pl->depth);
  if (pl->pinned) cudaFreeHost(pl->pinned);
  pl->color = NULL;
  pl->depth = NULL;
  pl->pinned = NULL;
  if (pl->stream) cudaStreamDestroy(pl->stream);
  pl->stream = NULL;
  free(pl->objects);
  pl->objects = NULL;
}

static void pipeline_finalize(napi_env env, void* data, void* hint) {
  (void)hint;
  Pipeline* pl = (Pipeline*)data;
  if (pl->scene_ref) napi_delete_reference(env, pl->scene_ref);
  pipeline_release(pl);
  free(pl);
}

static Pipeline* this_pipeline(napi_env env, napi_callback_info info, size_t* argc, napi_value* argv) {
  napi_value self;
  Pipeline* pl = NULL;
  if (napi_get_cb_info(env, info, argc, argv, &self, NULL) != napi_ok) return NULL;
  if (napi_unwrap(env, self, (void**)&pl) != napi_ok || !pl || !pl->p) {
    napi_throw_error(env, NULL, "TiledGaussianPipeline is disposed");
    return NULL;
  }
  return pl;
}

static const char* const kDepthModes[2] = {"float32", "packed16"};
static const char* const kAntialias[2] = {"compensated", "classic"};
static const char* const kBoundaries[3] = {"clip", "repeat-x", "repeat-y"};
static const char* const kRasterForms[3] = {"fp32", "exact", "half2"};

static int get_enum(napi_env env, napi_value obj, const char* name, const char* const* names, uint32_t n,
                    uint32_t* out) {
  napi_value v;
  bool has = false;
  if (napi_has_named_property(env, obj, name, &has) != napi_ok || !has) return 1; /* keep the default */
  if (napi_get_named_property(env, obj, name, &v) != napi_ok) return 0;
  char buf[32];
  size_t len = 0;
  if (napi_get_value_string_utf8(env, v, buf, sizeof(buf), &len) != napi_ok) return 0;
  for (uint32_t i = 0; i < n; ++i)
    if (strcmp(buf, names[i]) == 0) {
      *out = i;
      return 1;
    }
  return 0;
}

static int get_opt_f32(napi_env env, napi_value obj, const char* name, float* out) {
  bool has = false;
  if (napi_has_named_property(env, obj, name, &has) != napi_ok || !has) return 1;
  double d = 0;
  if (!get_f64(env, obj, name, &d)) return 0;
  *out = (float)d;
  return 1;
}

static int get_opt_u32(napi_env env, napi_value obj, const char* name, uint32_t* out) {
  bool has = false;
  if (napi_has_named_property(env, obj, name, &has) != napi_ok || !has) return 1;
  return get_u32(env, obj, name, out);
}

/* new Pipeline(scene, options): options use the reference's names
 * (GaussianPass.ts:170-256): depthSortMode, antialiasMode, intersectionCapacity,
 * background [r,g,b,a], maxRasterizedSplatsPerTile, rasterChunkSize,
 * subpixelSampleCulling, rasterTransmittanceThreshold, depthAlphaThreshold,
 * filterVariance, boundaryPolicy, rasterStats, plus rasterForm
 * ("fp32" | "exact" | "half2") and device. */
static napi_value pipeline_new(napi_env env, napi_callback_info info) {
  size_t argc = 2;
  napi_value argv[2], self;
  CHECK_NAPI(env, napi_get_cb_info(env, info, &argc, argv, &self, NULL));
  if (argc < 1) return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
  Scene* scene = NULL;
  if (napi_unwrap(env, argv[0], (void**)&scene) != napi_ok || !scene)
    return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
  gs3d_pipeline_desc d;
  gs3d_pipeline_desc_defaults(&d);
  if (argc >= 2) {
    napi_value o = argv[1];
    double cap = (double)d.intersection_capacity;
    bool has = false, flag = false;
    uint32_t stats = 0, subpixel = d.subpixel_sample_culling, chunk = d.raster_chunk_size, dev = 0;
    if (!get_enum(env, o, "depthSortMode", kDepthModes, 2, &d.depth_sort_mode) ||
        !get_enum(env, o, "antialiasMode", kAntialias, 2, &d.antialias_mode) ||
        !get_enum(env, o, "boundaryPolicy", kBoundaries, 3, &d.boundary_policy) ||
        !get_enum(env, o, "rasterForm", kRasterForms, 3, &d.raster_precision) ||
        !get_opt_f32(env, o, "rasterTransmittanceThreshold", &d.raster_transmittance_threshold) ||
        !get_opt_f32(env, o, "depthAlphaThreshold", &d.depth_alpha_threshold) ||
        !get_opt_f32(env, o, "filterVariance", &d.filter_variance) ||
        !get_opt_u32(env, o, "maxRasterizedSplatsPerTile", &d.max_rasterized_splats_per_tile) ||
        !get_opt_u32(env, o, "rasterChunkSize", &chunk) || !get_opt_u32(env, o, "device", &dev))
      return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
    d.raster_chunk_size = chunk;
    d.device = (int32_t)dev;
    if (napi_has_named_property(env, o, "intersectionCapacity", &has) == napi_ok && has &&
        get_f64(env, o, "intersectionCapacity", &cap))
      d.intersection_capacity = (uint64_t)cap;
    napi_value v;
    if (napi_has_named_property(env, o, "subpixelSampleCulling", &has) == napi_ok && has &&
        napi_get_named_property(env, o, "subpixelSampleCulling", &v) == napi_ok &&
        napi_get_value_bool(env, v, &flag) == napi_ok)
      subpixel = flag ? 1u : 0u;
    d.subpixel_sample_culling = subpixel;
    if (napi_has_named_property(env, o, "rasterStats", &has) == napi_ok && has &&
        napi_get_named_property(env, o, "rasterStats", &v) == napi_ok && napi_get_value_bool(env, v, &flag) == napi_ok)
      stats = flag ? 1u : 0u;
    d.raster_stats = stats;
    if (napi_has_named_property(env, o, "background", &has) == napi_ok && has &&
        napi_get_named_property(env, o, "background", &v) == napi_ok) {
      for (uint32_t i = 0; i < 4; ++i) {
        napi_value e;
        double x = 0;
        if (napi_get_element(env, v, i, &e) != napi_ok || napi_get_value_double(env, e, &x) != napi_ok)
          return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
        d.background[i] = (float)x;
      }
    }
  }
  Pipeline* pl = (Pipeline*)calloc(1, sizeof(Pipeline));
  if (!pl) return throw_status(env, GS3D_ERROR_OUT_OF_MEMORY, NULL);
  if (cudaSetDevice(d.device) != cudaSuccess || cudaStreamCreateWithFlags(&pl->stream, cudaStreamNonBlocking) != cudaSuccess) {
    free(pl);
    return throw_status(env, GS3D_ERROR_CUDA, NULL);
  }
  gs3d_status s = gs3d_pipeline_create(&d, &scene->data, &pl->p);
  if (s != GS3D_OK) {
    cudaStreamDestroy(pl->stream);
    free(pl);
    return throw_status(env, s, NULL);
  }
  pl->scene = scene;
  napi_create_reference(env, argv[0], 1, &pl->scene_ref);
  CHECK_NAPI(env, napi_wrap(env, self, pl, pipeline_finalize, NULL, NULL));
  return self;
}

/* updateData(scene) (TiledGaussianPipeline.ts:203-218). */
static napi_value pipeline_update_data(napi_env env, napi_callback_info info) {
  size_t argc = 1;
  napi_value argv[1];
  Pipeline* pl = this_pipeline(env, info, &argc, argv);
  if (!pl) return NULL;
  Scene* scene = NULL;
  if (argc < 1 || napi_unwrap(env, argv[0], (void**)&scene) != napi_ok || !scene)
    return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, pl->p);
  gs3d_status s = gs3d_pipeline_update_data(pl->p, &scene->data);
  if (s != GS3D_OK) return throw_status(env, s, pl->p);
  if (pl->scene_ref) napi_delete_reference(env, pl->scene_ref);
  napi_create_reference(env, argv[0], 1, &pl->scene_ref);
  pl->scene = scene;
  return NULL;
}

/* resizeIntersections(capacity) (TiledGaussianPipeline.ts:220-231). */
static napi_value pipeline_resize(napi_env env, napi_callback_info info) {
  size_t argc = 1;
  napi_value argv[1];
  Pipeline* pl = this_pipeline(env, info, &argc, argv);
  if (!pl) return NULL;
  double cap = 0;
  if (argc < 1 || napi_get_value_double(env, argv[0], &cap) != napi_ok || !(cap >= 0))
    return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, pl->p);
  gs3d_status s = gs3d_pipeline_resize_intersections(pl->p, (uint64_t)cap);
  if (s != GS3D_OK) return throw_status(env, s, pl->p);
  return NULL;
}

/* prepareFrame(width, height, outputDepth) (TiledGaussianPipeline.ts:286-322):
 * sizes the pipeline's own rgba16f colour and float32 depth targets. */
static napi_value pipeline_prepare(napi_env env, napi_callback_info info) {
  size_t argc = 3;
  napi_value argv[3];
  Pipeline* pl = this_pipeline(env, info, &argc, argv);
  if (!pl) return NULL;
  uint32_t w = 0, h = 0;
  bool depth = false;
  if (argc < 2 || napi_get_value_uint32(env, argv[0], &w) != napi_ok ||
      napi_get_value_uint32(env, argv[1], &h) != napi_ok)
    return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, pl->p);
  if (argc >= 3) napi_get_value_bool(env, argv[2], &depth);
  gs3d_status s = gs3d_pipeline_prepare_frame(pl->p, w, h);
  if (s != GS3D_OK) return throw_status(env, s, pl->p);
  const size_t cbytes = (size_t)w * h * 8, dbytes = depth ? (size_t)w * h * 4 : 0;
  if (cbytes != pl->color_bytes || dbytes != pl->depth_bytes) {
    cudaStreamSynchronize(pl->stream); /* the previous frame may still write the old targets */
    cudaFree(pl->color);
    cudaFree(pl->depth);
    pl->color = NULL;
    pl->depth = NULL;
    pl->color_bytes = pl->depth_bytes = 0;
    cudaError_t e = cudaMalloc(&pl->color, cbytes);
    if (e == cudaSuccess && dbytes) e = cudaMalloc((void**)&pl->depth, dbytes);
    if (e != cudaSuccess) return throw_cuda(env, e, "allocating render targets");
    pl->color_bytes = cbytes;
    pl->depth_bytes = dbytes;
  }
  pl->width = w;
  pl->height = h;
  pl->output_depth = depth ? 1u : 0u;
  return NULL;
}

/* setCamera(projection[16], view[16], near, far, objectTable): the state
 * FrameUniforms.update and ObjectFrameState.update write each frame
 * (FrameUniforms.ts:41-58, ObjectFrameState.ts:97-119); column-major
 * matrices, 40 floats per object. */
static napi_value pipeline_set_camera(napi_env env, napi_callback_info info) {
  size_t argc = 5;
  napi_value argv[5];
  Pipeline* pl = this_pipeline(env, info, &argc, argv);
  if (!pl) return NULL;
  void *proj = NULL, *view = NULL, *table = NULL;
  size_t pb = 0, vb = 0, tb = 0;
  double nearv = 0, farv = 0;
  if (argc < 5 || !typed_bytes(env, argv[0], &proj, &pb) || pb != 64 || !typed_bytes(env, argv[1], &view, &vb) ||
      vb != 64 || napi_get_value_double(env, argv[2], &nearv) != napi_ok ||
      napi_get_value_double(env, argv[3], &farv) != napi_ok || !typed_bytes(env, argv[4], &table, &tb) ||
      tb % 160 != 0)
    return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, pl->p);
  const uint32_t objects = (uint32_t)(tb / 160);
  if (objects > pl->object_cap) {
    float* grown = (float*)realloc(pl->objects, tb);
    if (!grown) return throw_status(env, GS3D_ERROR_OUT_OF_MEMORY, pl->p);
    pl->objects = grown;
    pl->object_cap = objects;
  }
  if (tb) memcpy(pl->objects, table, tb);
  memcpy(pl->camera.projection, proj, 64);
  memcpy(pl->camera.view, view, 64);
  pl->camera.depth_near = (float)nearv;
  pl->camera.depth_far = (float)farv;
  pl->camera.object_table = pl->objects;
  pl->camera.object_count = objects;
  return NULL;
}

/* render(attempt, resetValid) (TiledGaussianPipeline.ts:324-341): enqueues
 * the pass on the pipeline's stream and returns. */
static napi_value pipeline_render(napi_env env, napi_callback_info info) {
  size_t argc = 2;
  napi_value argv[2];
  Pipeline* pl = this_pipeline(env, info, &argc, argv);
  if (!pl) return NULL;
  uint32_t attempt = 1;
  bool reset = false;
  if (argc >= 1) napi_get_value_uint32(env, argv[0], &attempt);
  if (argc >= 2) napi_get_value_bool(env, argv[1], &reset);
  if (!pl->color) return throw_status(env, GS3D_ERROR_NOT_PREPARED, pl->p);
  gs3d_targets t;
  memset(&t, 0, sizeof(t));
  t.color = pl->color;
  t.color_format = GS3D_COLOR_RGBA16F;
  t.depth = pl->output_depth ? pl->depth : NULL;
  gs3d_status s = gs3d_pipeline_render(pl->p, &pl->camera, attempt, reset ? 1 : 0, &t, pl->stream);
  if (s != GS3D_OK) return throw_status(env, s, pl->p);
  return NULL;
}

/* Asynchronous read-backs: a libuv worker waits for the copy, the JS thread
 * resolves the Promise. */
typedef struct Readback {
  Pipeline* pl;
  napi_deferred deferred;
  napi_async_work work;
  napi_ref self_ref;    /* keeps the pipeline object alive while in flight */
  int kind;             /* 0: stats, 1: image */
  gs3d_status status;
  gs3d_stats stats;
  cudaError_t cuda;
} Readback;

static void readback_execute(napi_env env, void* data) {
  (void)env;
  Readback* rb = (Readback*)data;
  if (rb->kind == 0) rb->status = gs3d_pipeline_poll_stats(rb->pl->p, &rb->stats, 1);
  else rb->cuda = cudaStreamSynchronize(rb->pl->stream);
}

static napi_value stats_object(napi_env env, const gs3d_stats* s) {
  napi_value o, work, state;
  napi_create_object(env, &o);
  napi_set_named_property(env, o, "visibleGaussianCount", make_u32(env, s->visible_gaussian_count));
  napi_set_named_property(env, o, "intersectionCount", make_u32(env, s->intersection_count));
  napi_set_named_property(env, o, "requestedIntersections", make_u32(env, s->requested_intersections));
  napi_set_named_property(env, o, "intersectionCapacity", make_f64(env, (double)s->intersection_capacity));
  napi_value overflow;
  napi_get_boolean(env, s->overflow != 0, &overflow);
  napi_set_named_property(env, o, "overflow", overflow);
  napi_create_object(env, &work);
  napi_set_named_property(env, work, "checked", make_f64(env, (double)s->raster_checked));
  napi_set_named_property(env, work, "blended", make_f64(env, (double)s->raster_blended));
  napi_set_named_property(env, work, "pixels", make_f64(env, (double)s->raster_pixels));
  napi_set_named_property(env, work, "alphaStopped", make_f64(env, (double)s->raster_alpha_stopped));
  napi_set_named_property(env, o, "rasterWork", work);
  napi_create_array_with_length(env, 4, &state);
  for (uint32_t i = 0; i < 4; ++i) napi_set_element(env, state, i, make_u32(env, s->output_state[i]));
  napi_set_named_property(env, o, "outputState", state);
  return o;
}

static void readback_complete(napi_env env, napi_status status, void* data) {
  Readback* rb = (Readback*)data;
  Pipeline* pl = rb->pl;
  napi_value result = NULL, msg;
  int ok = status == napi_ok;
  if (rb->kind == 0) {
    pl->stats_pending = 0;
    ok = ok && rb->status == GS3D_OK;
    if (ok) result = stats_object(env, &rb->stats);
    else {
      const char* m = gs3d_pipeline_last_error(pl->p);
      napi_create_string_utf8(env, m && m[0] ? m : gs3d_status_string(rb->status), NAPI_AUTO_LENGTH, &msg);
      napi_create_error(env, NULL, msg, &result);
    }
  } else {
    pl->image_pending = 0;
    ok = ok && rb->cuda == cudaSuccess;
    if (ok) {
      void* bytes = NULL;
      napi_create_arraybuffer(env, pl->color_bytes, &bytes, &result);
      memcpy(bytes, pl->pinned, pl->color_bytes);
    } else {
      napi_create_string_utf8(env, cudaGetErrorString(rb->cuda), NAPI_AUTO_LENGTH, &msg);
      napi_create_error(env, NULL, msg, &result);
    }
  }
  if (ok) napi_resolve_deferred(env, rb->deferred, result);
  else napi_reject_deferred(env, rb->deferred, result);
  napi_delete_async_work(env, rb->work);
  napi_delete_reference(env, rb->self_ref);
  free(rb);
}

static napi_value start_readback(napi_env env, napi_callback_info info, int kind) {
  size_t argc = 0;
  napi_value self;
  Pipeline* pl = NULL;
  CHECK_NAPI(env, napi_get_cb_info(env, info, &argc, NULL, &self, NULL));
  if (napi_unwrap(env, self, (void**)&pl) != napi_ok || !pl || !pl->p) {
    napi_throw_error(env, NULL, "TiledGaussianPipeline is disposed");
    return NULL;
  }
  if (kind == 0) {
    if (pl->stats_pending) {
      napi_throw_error(env, NULL, "a stats read-back is already in flight");
      return NULL;
    }
    gs3d_status s = gs3d_pipeline_request_stats(pl->p, pl->stream);
    if (s != GS3D_OK) return throw_status(env, s, pl->p);
    pl->stats_pending = 1;
  } else {
    if (pl->image_pending) {
      napi_throw_error(env, NULL, "an image read-back is already in flight");
      return NULL;
    }
    if (!pl->color) return throw_status(env, GS3D_ERROR_NOT_PREPARED, pl->p);
    if (pl->pinned_bytes < pl->color_bytes) {
      if (pl->pinned) cudaFreeHost(pl->pinned);
      pl->pinned = NULL;
      pl->pinned_bytes = 0;
      cudaError_t e = cudaMallocHost(&pl->pinned, pl->color_bytes);
      if (e != cudaSuccess) return throw_cuda(env, e, "allocating the pinned image buffer");
      pl->pinned_bytes = pl->color_bytes;
    }
    cudaError_t e = cudaMemcpyAsync(pl->pinned, pl->color, pl->color_bytes, cudaMemcpyDeviceToHost, pl->stream);
    if (e != cudaSuccess) return throw_cuda(env, e, "enqueueing the image read-back");
    pl->image_pending = 1;
  }
  Readback* rb = (Readback*)calloc(1, sizeof(Readback));
  napi_value promise, name;
  rb->pl = pl;
  rb->kind = kind;
  CHECK_NAPI(env, napi_create_promise(env, &rb->deferred, &promise));
  CHECK_NAPI(env, napi_create_reference(env, self, 1, &rb->self_ref));
  CHECK_NAPI(env, napi_create_string_utf8(env, kind ? "gs3d.readImage" : "gs3d.readStats", NAPI_AUTO_LENGTH, &name));
  CHECK_NAPI(env, napi_create_async_work(env, NULL, name, readback_execute, readback_complete, rb, &rb->work));
  CHECK_NAPI(env, napi_queue_async_work(env, rb->work));
  return promise;
}

/* readStats(): Promise of the last render's counters and 16-byte output
 * state (TiledGaussianPipeline.ts:353-366, GaussianPass.ts:1019-1079). */
static napi_value pipeline_read_stats(napi_env env, napi_callback_info info) { return start_readback(env, info, 0); }

/* readImage(): Promise of the rgba16f colour target as an ArrayBuffer. */
static napi_value pipeline_read_image(napi_env env, napi_callback_info info) { return start_readback(env, info, 1); }

/* getResources() (TiledGaussianPipeline.ts:391-406): device addresses as
 * BigInts, for CUDA interop. */
static napi_value pipeline_get_resources(napi_env env, napi_callback_info info) {
  size_t argc = 0;
  Pipeline* pl = this_pipeline(env, info, &argc, NULL);
  if (!pl) return NULL;
  gs3d_resources r;
  gs3d_status s = gs3d_pipeline_get_resources(pl->p, &r);
  if (s != GS3D_OK) return throw_status(env, s, pl->p);
  napi_value o;
  napi_create_object(env, &o);
  napi_set_named_property(env, o, "projectedMean", make_ptr(env, r.projected_mean));
  napi_set_named_property(env, o, "projectedConic", make_ptr(env, r.projected_conic));
  napi_set_named_property(env, o, "projectedColor", make_ptr(env, r.projected_color));
  napi_set_named_property(env, o, "tileCounts", make_ptr(env, r.tile_counts));
  napi_set_named_property(env, o, "visibleOffsets", make_ptr(env, r.visible_offsets));
  napi_set_named_property(env, o, "depthSortedKeys", make_ptr(env, r.depth_sorted_keys));
  napi_set_named_property(env, o, "depthSortedIds", make_ptr(env, r.depth_sorted_ids));
  napi_set_named_property(env, o, "intersectionOffsets", make_ptr(env, r.intersection_offsets));
  napi_set_named_property(env, o, "sortedTileIds", make_ptr(env, r.sorted_tile_ids));
  napi_set_named_property(env, o, "sortedGaussianIds", make_ptr(env, r.sorted_gaussian_ids));
  napi_set_named_property(env, o, "tileOffsets", make_ptr(env, r.tile_offsets));
  napi_set_named_property(env, o, "outputState", make_ptr(env, r.output_state));
  napi_set_named_property(env, o, "color", make_ptr(env, pl->color));
  napi_set_named_property(env, o, "depth", make_ptr(env, pl->output_depth ? pl->depth : NULL));
  napi_set_named_property(env, o, "tilesX", make_u32(env, r.tiles_x));
  napi_set_named_property(env, o, "tilesY", make_u32(env, r.tiles_y));
  napi_set_named_property(env, o, "intersectionCapacity", make_f64(env, (double)r.intersection_capacity));
  return o;
}

/* dispose() (TiledGaussianPipeline.ts:408-425). */
static napi_value pipeline_dispose(napi_env env, napi_callback_info info) {
  size_t argc = 0;
  napi_value self;
  Pipeline* pl = NULL;
  CHECK_NAPI(env, napi_get_cb_info(env, info, &argc, NULL, &self, NULL));
  if (napi_unwrap(env, self, (void**)&pl) == napi_ok && pl) {
    if (pl->stats_pending || pl->image_pending) {
      napi_throw_error(env, NULL, "dispose() while a read-back is in flight");
      return NULL;
    }
    pipeline_release(pl);
    if (pl->scene_ref) napi_delete_reference(env, pl->scene_ref); /* GaussianData.release */
    pl->scene_ref = NULL;
  }
  return NULL;
}

/* capacityNext(maximum, growth, headroom, current, demand): the capacity
 * policy (IntersectionCapacityPolicy.ts:90-100); null above the maximum. */
static napi_value capacity_next(napi_env env, napi_callback_info info) {
  size_t argc = 5;
  napi_value argv[5], r;
  double a[5] = {0, 0, 0, 0, 0};
  CHECK_NAPI(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  if (argc < 5) return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
  for (int i = 0; i < 5; ++i)
    if (napi_get_value_double(env, argv[i], &a[i]) != napi_ok)
      return throw_status(env, GS3D_ERROR_INVALID_ARGUMENT, NULL);
  const uint64_t next = gs3d_capacity_next((uint64_t)a[0], a[1], a[2], (uint64_t)a[3], (uint64_t)a[4]);
  if (next == 0) {
    napi_get_null(env, &r);
    return r;
  }
  return make_f64(env, (double)next);
}

static napi_value init(napi_env env, napi_value exports) {
  napi_property_descriptor methods[] = {
      {"updateData", NULL, pipeline_update_data, NULL, NULL, NULL, napi_default, NULL},
      {"resizeIntersections", NULL, pipeline_resize, NULL, NULL, NULL, napi_default, NULL},
      {"prepareFrame", NULL, pipeline_prepare, NULL, NULL, NULL, napi_default, NULL},
      {"setCamera", NULL, pipeline_set_camera, NULL, NULL, NULL, napi_default, NULL},
      {"render", NULL, pipeline_render, NULL, NULL, NULL, napi_default, NULL},
      {"readStats", NULL, pipeline_read_stats, NULL, NULL, NULL, napi_default, NULL},
      {"readImage", NULL, pipeline_read_image, NULL, NULL, NULL, napi_default, NULL},
      {"getResources", NULL, pipeline_get_resources, NULL, NULL, NULL, napi_default, NULL},
      {"dispose", NULL, pipeline_dispose, NULL, NULL, NULL, napi_default, NULL},
  };
  napi_value cls, fn;
  if (gs3d_abi_version() != GS3D_ABI_VERSION) {
    napi_throw_error(env, NULL, "libgs3d ABI version differs from the addon's header");
    return NULL;
  }
  CHECK_NAPI(env, napi_define_class(env, "Pipeline", NAPI_AUTO_LENGTH, pipeline_new, NULL,
                                    sizeof(methods) / sizeof(methods[0]), methods, &cls));
  CHECK_NAPI(env, napi_set_named_property(env, exports, "Pipeline", cls));
  CHECK_NAPI(env, napi_create_function(env, "createScene", NAPI_AUTO_LENGTH, create_scene, NULL, &fn));
  CHECK_NAPI(env, napi_set_named_property(env, exports, "createScene", fn));
  CHECK_NAPI(env, napi_create_function(env, "updateScene", NAPI_AUTO_LENGTH, update_scene, NULL, &fn));
  CHECK_NAPI(env, napi_set_named_property(env, exports, "updateScene", fn));
  CHECK_NAPI(env, napi_create_function(env, "capacityNext", NAPI_AUTO_LENGTH, capacity_next, NULL, &fn));
  CHECK_NAPI(env, napi_set_named_property(env, exports, "capacityNext", fn));
  return exports;
}

NAPI_MODULE(NODE_GYP_MODULE_NAME, init)
