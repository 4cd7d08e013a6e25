/*
 * caustic_addon.c - Node-API addon binding the reference's TypeScript host to
 * libcaustic_gb300 (include/caustic.h).
 *
 * The reference's module surface it serves (src/tracer/index.ts:5-20):
 *   renderImage(ps, frame, opts)                       tracer.ts:348-355
 *   accumulatePass(ps, frame, w, h, frameIndex, opts, accum)   tracer.ts:361-395
 *   intersectClosest / occluded, batched over many rays        intersect.ts:202,368
 * plus sceneCreate / sceneDestroy, which upload a PackedScene (pack.ts:46-59)
 * once and keep it on the GPU. Typed arrays are borrowed without copying
 * (napi_get_typedarray_info); renderImage returns a new Float32Array.
 *
 * Errors: a wrong argument type throws TypeError, an array of the wrong length
 * RangeError, and a failed library call Error with `code` set to the status
 * name (CT_ERR_...) and the library's ct_last_error() message. Every Node-API
 * call's status is checked; a failed one throws (unless an exception is
 * already pending) and the function returns NULL (undefined).
 *
 * Numbers follow the reference's JavaScript semantics where it converts
 * them: frameIndex and seed go through ToUint32 as rng.ts does (pcgHash and
 * seedFor work on uint32), so frameIndex = s + seed * 7919 wraps as it does
 * there for integer seeds.
 */
#ifdef CT_NODE_HEADERS
#include <node_api.h>
#else
#include "node_api_min.h"
#endif

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "caustic.h"

#if defined(__GNUC__)
#define CT_EXPORT __attribute__((visibility("default")))
#else
#define CT_EXPORT
#endif

/* ---- Node-API status handling ------------------------------------------ */

static void throw_once(napi_env env, const char* code, const char* msg, int kind) {
  bool pending = false;
  if (napi_is_exception_pending(env, &pending) == napi_ok && pending) return;
  if (kind == 1)
    napi_throw_type_error(env, code, msg);
  else if (kind == 2)
    napi_throw_range_error(env, code, msg);
  else
    napi_throw_error(env, code, msg);
}

/* Evaluates a Node-API call; on failure throws and returns 0 from the helper. */
#define NAPI_OK(env, call)                                                   \
  do {                                                                       \
    napi_status st_ = (call);                                                \
    if (st_ != napi_ok) {                                                    \
      char m_[160];                                                          \
      snprintf(m_, sizeof m_, "Node-API call failed (status %d): %s", (int)st_, #call); \
      throw_once(env, "CT_NAPI", m_, 0);                                     \
      return 0;                                                              \
    }                                                                        \
  } while (0)

static int type_error(napi_env env, const char* what, const char* expected) {
  char m[200];
  snprintf(m, sizeof m, "%s must be %s", what, expected);
  throw_once(env, "ERR_INVALID_ARG_TYPE", m, 1);
  return 0;
}

static int range_error(napi_env env, const char* what, const char* detail) {
  char m[240];
  snprintf(m, sizeof m, "%s %s", what, detail);
  throw_once(env, "ERR_OUT_OF_RANGE", m, 2);
  return 0;
}

static const char* status_name(ct_status s) {
  switch (s) {
    case CT_OK: return "CT_OK";
    case CT_ERR_INVALID_ARGUMENT: return "CT_ERR_INVALID_ARGUMENT";
    case CT_ERR_CUDA: return "CT_ERR_CUDA";
    case CT_ERR_OUT_OF_MEMORY: return "CT_ERR_OUT_OF_MEMORY";
    case CT_ERR_UNSUPPORTED: return "CT_ERR_UNSUPPORTED";
    case CT_ERR_TIMEOUT: return "CT_ERR_TIMEOUT";
    case CT_ERR_BUDGET: return "CT_ERR_BUDGET";
    case CT_ERR_CANCELLED: return "CT_ERR_CANCELLED";
    case CT_ERR_NOT_FOUND: return "CT_ERR_NOT_FOUND";
  }
  return "CT_ERR_UNKNOWN";
}

/* A failed ct_* call: Error with code = status name, message = ct_last_error(). */
static napi_value library_error(napi_env env, ct_status s) {
  const char* msg = ct_last_error();
  throw_once(env, status_name(s), msg && msg[0] ? msg : status_name(s), 0);
  return NULL;
}

/* ---- reading JavaScript values ----------------------------------------- */

static int get_prop(napi_env env, napi_value obj, const char* key, napi_value* out) {
  napi_valuetype t;
  NAPI_OK(env, napi_typeof(env, obj, &t));
  if (t != napi_object) return type_error(env, key, "read from an object");
  NAPI_OK(env, napi_get_named_property(env, obj, key, out));
  return 1;
}

static int as_number(napi_env env, napi_value v, const char* what, double* out) {
  napi_valuetype t;
  NAPI_OK(env, napi_typeof(env, v, &t));
  if (t != napi_number) return type_error(env, what, "a number");
  NAPI_OK(env, napi_get_value_double(env, v, out));
  return 1;
}

static int prop_number(napi_env env, napi_value obj, const char* key, double* out) {
  napi_value v;
  return get_prop(env, obj, key, &v) && as_number(env, v, key, out);
}

static int prop_bool(napi_env env, napi_value obj, const char* key, int32_t* out) {
  napi_value v;
  napi_valuetype t;
  bool b = false;
  if (!get_prop(env, obj, key, &v)) return 0;
  NAPI_OK(env, napi_typeof(env, v, &t));
  if (t != napi_boolean) return type_error(env, key, "a boolean");
  NAPI_OK(env, napi_get_value_bool(env, v, &b));
  *out = b ? 1 : 0;
  return 1;
}

/* An integer in [lo, hi] (image sizes, spp, bounce counts). */
static int prop_int(napi_env env, napi_value obj, const char* key, double lo, double hi, int32_t* out) {
  double d;
  if (!prop_number(env, obj, key, &d)) return 0;
  if (!(d == floor(d)) || d < lo || d > hi) {
    char m[96];
    snprintf(m, sizeof m, "must be an integer in [%.0f, %.0f], got %g", lo, hi, d);
    return range_error(env, key, m);
  }
  *out = (int32_t)d;
  return 1;
}

/* ECMAScript ToUint32: truncate, then modulo 2^32 (NaN and infinities give 0). */
static uint32_t to_uint32(double d) {
  if (!isfinite(d)) return 0;
  double m = fmod(trunc(d), 4294967296.0);
  if (m < 0) m += 4294967296.0;
  return (uint32_t)m;
}

/* A typed array of the given element type; pointer and element count, no copy. */
static int typed(napi_env env, napi_value v, napi_typedarray_type want, const char* what, const char* tname,
                 void** data, size_t* length) {
  bool is = false;
  napi_typedarray_type t;
  napi_value buf;
  size_t off;
  NAPI_OK(env, napi_is_typedarray(env, v, &is));
  if (!is) return type_error(env, what, tname);
  NAPI_OK(env, napi_get_typedarray_info(env, v, &t, length, data, &buf, &off));
  if (t != want) return type_error(env, what, tname);
  return 1;
}

static int prop_typed(napi_env env, napi_value obj, const char* key, napi_typedarray_type want, const char* tname,
                      void** data, size_t* length) {
  napi_value v;
  return get_prop(env, obj, key, &v) && typed(env, v, want, key, tname, data, length);
}

static int vec3(napi_env env, napi_value obj, const char* key, double out[3]) { /* Vec3 {x, y, z} */
  napi_value v;
  return get_prop(env, obj, key, &v) && prop_number(env, v, "x", &out[0]) && prop_number(env, v, "y", &out[1]) &&
         prop_number(env, v, "z", &out[2]);
}

static int color(napi_env env, napi_value obj, const char* key, double out[3]) { /* Color {r, g, b} */
  napi_value v;
  return get_prop(env, obj, key, &v) && prop_number(env, v, "r", &out[0]) && prop_number(env, v, "g", &out[1]) &&
         prop_number(env, v, "b", &out[2]);
}

/* CameraFrame (camera.ts:8-20). */
static int frame_of(napi_env env, napi_value f, ct_camera_frame* out) {
  return vec3(env, f, "origin", out->origin) && vec3(env, f, "right", out->right) && vec3(env, f, "up", out->up) &&
         vec3(env, f, "forward", out->forward) && prop_number(env, f, "tanHalfFov", &out->tan_half_fov) &&
         prop_number(env, f, "aspect", &out->aspect) && prop_number(env, f, "lensRadius", &out->lens_radius) &&
         prop_number(env, f, "focusDistance", &out->focus_distance);
}

/* TraceOptions (tracer.ts:27-31). */
static int trace_of(napi_env env, napi_value o, ct_trace_options* out) {
  return prop_int(env, o, "maxBounces", 0, 1 << 20, &out->max_bounces) &&
         prop_bool(env, o, "russianRoulette", &out->russian_roulette) && prop_bool(env, o, "nee", &out->nee);
}

/* Sky (scene.ts:50-52): { kind: 'none' } | { kind: 'gradient', zenith, horizon, strength }. */
static int sky_of(napi_env env, napi_value ps, ct_sky* out) {
  napi_value sky, kind;
  napi_valuetype t;
  char k[16] = {0};
  size_t len = 0;
  memset(out, 0, sizeof *out);
  if (!get_prop(env, ps, "sky", &sky) || !get_prop(env, sky, "kind", &kind)) return 0;
  NAPI_OK(env, napi_typeof(env, kind, &t));
  if (t != napi_string) return type_error(env, "sky.kind", "'none' or 'gradient'");
  NAPI_OK(env, napi_get_value_string_utf8(env, kind, k, sizeof k, &len));
  if (strcmp(k, "none") == 0) return 1;
  if (strcmp(k, "gradient") != 0) return range_error(env, "sky.kind", "must be 'none' or 'gradient'");
  out->kind = 1;
  return color(env, sky, "zenith", out->zenith) && color(env, sky, "horizon", out->horizon) &&
         prop_number(env, sky, "strength", &out->strength);
}

/* ---- scene handles ------------------------------------------------------ */

typedef struct scene_box {
  ct_scene* scene; /* NULL once sceneDestroy released it */
} scene_box;

static void scene_finalize(napi_env env, void* data, void* hint) {
  scene_box* box = (scene_box*)data;
  (void)env;
  (void)hint;
  if (box->scene) ct_scene_destroy(box->scene);
  free(box);
}

static int scene_of(napi_env env, napi_value v, scene_box** out) {
  napi_valuetype t;
  void* p = NULL;
  NAPI_OK(env, napi_typeof(env, v, &t));
  if (t != napi_external) return type_error(env, "scene", "a handle returned by sceneCreate");
  NAPI_OK(env, napi_get_value_external(env, v, &p));
  *out = (scene_box*)p;
  if (!(*out)->scene) return range_error(env, "scene", "was destroyed by sceneDestroy");
  return 1;
}

static int args(napi_env env, napi_callback_info info, size_t want, napi_value* argv) {
  size_t argc = want;
  NAPI_OK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  if (argc < want) {
    char m[96];
    snprintf(m, sizeof m, "expects %zu arguments, got %zu", want, argc);
    throw_once(env, "ERR_MISSING_ARGS", m, 1);
    return 0;
  }
  return 1;
}

static napi_value undefined(napi_env env) {
  napi_value u = NULL;
  if (napi_get_undefined(env, &u) != napi_ok) return NULL;
  return u;
}

/* sceneCreate(ps: PackedScene): External. Validates the arrays and copies them to the GPU. */
static napi_value scene_create(napi_env env, napi_callback_info info) {
  napi_value ps;
  ct_packed_scene_view v;
  double prim_count, node_count, mat_count;
  size_t n_prims, n_nodes, n_mats, n_lights, n_obj;
  void *prims, *nodes, *mats, *lights, *obj;
  memset(&v, 0, sizeof v);
  if (!args(env, info, 1, &ps)) return NULL;
  if (!prop_typed(env, ps, "prims", napi_float32_array, "a Float32Array", &prims, &n_prims) ||
      !prop_number(env, ps, "primCount", &prim_count) ||
      !prop_typed(env, ps, "nodes", napi_float32_array, "a Float32Array", &nodes, &n_nodes) ||
      !prop_number(env, ps, "nodeCount", &node_count) ||
      !prop_typed(env, ps, "mats", napi_float32_array, "a Float32Array", &mats, &n_mats) ||
      !prop_number(env, ps, "matCount", &mat_count) ||
      !prop_typed(env, ps, "lights", napi_int32_array, "an Int32Array", &lights, &n_lights) ||
      !prop_typed(env, ps, "primObject", napi_uint32_array, "a Uint32Array", &obj, &n_obj) || !sky_of(env, ps, &v.sky))
    return NULL;
  if (prim_count < 0 || prim_count != floor(prim_count) || prim_count > 4294967295.0 ||
      n_prims < (size_t)prim_count * CT_PRIM_STRIDE || n_obj < (size_t)prim_count)
    return range_error(env, "primCount", "does not fit prims (16 floats each) and primObject"), NULL;
  if (node_count < 0 || node_count != floor(node_count) || n_nodes < (size_t)node_count * CT_NODE_STRIDE)
    return range_error(env, "nodeCount", "does not fit nodes (8 floats each)"), NULL;
  if (mat_count < 0 || mat_count != floor(mat_count) ||
      n_mats < (size_t)(mat_count > 0 ? mat_count : 1) * CT_MAT_STRIDE)
    return range_error(env, "matCount", "does not fit mats (16 floats each)"), NULL;
  if (n_lights > 0xFFFFFFFFu) return range_error(env, "lights", "is too long"), NULL;
  v.prims = (const float*)prims;
  v.prim_count = (uint32_t)prim_count;
  v.nodes = (const float*)nodes;
  v.node_count = (uint32_t)node_count;
  v.mats = (const float*)mats;
  v.mat_count = (uint32_t)mat_count;
  v.lights = (const int32_t*)lights;
  v.light_count = (uint32_t)n_lights;
  v.prim_object = (const uint32_t*)obj;

  scene_box* box = (scene_box*)calloc(1, sizeof *box);
  if (!box) return library_error(env, CT_ERR_OUT_OF_MEMORY);
  ct_status st = ct_scene_create(&v, &box->scene);
  if (st != CT_OK) {
    free(box);
    return library_error(env, st);
  }
  napi_value ext;
  if (napi_create_external(env, box, scene_finalize, NULL, &ext) != napi_ok) {
    ct_scene_destroy(box->scene);
    free(box);
    throw_once(env, "CT_NAPI", "napi_create_external failed", 0);
    return NULL;
  }
  return ext;
}

/* sceneDestroy(scene): releases the GPU copy now instead of at garbage collection. */
static napi_value scene_destroy(napi_env env, napi_callback_info info) {
  napi_value a;
  napi_valuetype t;
  void* p = NULL;
  if (!args(env, info, 1, &a)) return NULL;
  if (napi_typeof(env, a, &t) != napi_ok || t != napi_external)
    return type_error(env, "scene", "a handle returned by sceneCreate"), NULL;
  if (napi_get_value_external(env, a, &p) != napi_ok) return NULL;
  scene_box* box = (scene_box*)p;
  if (box->scene) ct_scene_destroy(box->scene);
  box->scene = NULL;
  return undefined(env);
}

/* renderImage(scene, frame: CameraFrame, opts: RenderOptions): Float32Array (tracer.ts:348-355). */
static napi_value render_image(napi_env env, napi_callback_info info) {
  napi_value a[3];
  scene_box* box;
  ct_camera_frame f;
  ct_trace_options t;
  ct_render_options o;
  if (!args(env, info, 3, a) || !scene_of(env, a[0], &box) || !frame_of(env, a[1], &f) || !trace_of(env, a[2], &t))
    return NULL;
  memset(&o, 0, sizeof o);
  if (!prop_int(env, a[2], "width", 1, 1 << 16, &o.width) || !prop_int(env, a[2], "height", 1, 1 << 16, &o.height) ||
      !prop_int(env, a[2], "spp", 1, 1 << 24, &o.spp))
    return NULL;
  bool has_seed = false;
  if (napi_has_named_property(env, a[2], "seed", &has_seed) != napi_ok) return NULL;
  if (has_seed) { /* seed?: number, default 0 (tracer.ts:351: opts.seed ?? 0) */
    napi_value sv;
    napi_valuetype st;
    double seed = 0;
    if (!get_prop(env, a[2], "seed", &sv)) return NULL;
    if (napi_typeof(env, sv, &st) != napi_ok) return NULL;
    if (st != napi_undefined && st != napi_null) {
      if (!as_number(env, sv, "seed", &seed)) return NULL;
      o.seed = to_uint32(seed);
    }
  }
  o.max_bounces = t.max_bounces;
  o.russian_roulette = t.russian_roulette;
  o.nee = t.nee;
  const size_t n = (size_t)o.width * (size_t)o.height * 3;
  void* px = NULL;
  napi_value ab, out;
  if (napi_create_arraybuffer(env, n * sizeof(float), &px, &ab) != napi_ok) {
    throw_once(env, "CT_NAPI", "cannot allocate the image", 2);
    return NULL;
  }
  ct_status st = ct_render_image(box->scene, &f, &o, (float*)px, NULL);
  if (st != CT_OK) return library_error(env, st);
  if (napi_create_typedarray(env, napi_float32_array, n, ab, 0, &out) != napi_ok) {
    throw_once(env, "CT_NAPI", "napi_create_typedarray failed", 0);
    return NULL;
  }
  return out;
}

/* accumulatePass(scene, frame, width, height, frameIndex, opts: TraceOptions, accum: Float32Array)
 * (tracer.ts:361-395): adds one sample per pixel into accum in place (a sum, not a mean). */
static napi_value accumulate_pass(napi_env env, napi_callback_info info) {
  napi_value a[7];
  scene_box* box;
  ct_camera_frame f;
  ct_trace_options t;
  double w, h, fi;
  void* accum;
  size_t n;
  if (!args(env, info, 7, a) || !scene_of(env, a[0], &box) || !frame_of(env, a[1], &f) ||
      !as_number(env, a[2], "width", &w) || !as_number(env, a[3], "height", &h) ||
      !as_number(env, a[4], "frameIndex", &fi) || !trace_of(env, a[5], &t) ||
      !typed(env, a[6], napi_float32_array, "accum", "a Float32Array", &accum, &n))
    return NULL;
  if (w != floor(w) || h != floor(h) || w < 1 || h < 1 || w > 65536 || h > 65536)
    return range_error(env, "width and height", "must be integers in [1, 65536]"), NULL;
  if (n != (size_t)w * (size_t)h * 3) return range_error(env, "accum", "must hold width * height * 3 floats"), NULL;
  ct_status st = ct_accumulate_pass(box->scene, &f, (int32_t)w, (int32_t)h, to_uint32(fi), &t, (float*)accum, NULL);
  if (st != CT_OK) return library_error(env, st);
  return undefined(env);
}

/* intersectClosestMany(scene, rays: Float32Array (8 floats per ray: origin, direction, tMin, tMax),
 * prim: Int32Array, t: Float32Array[, u: Float32Array, v: Float32Array]): intersectClosest
 * (intersect.ts:202-282) for every ray; prim -1 and t Infinity for a miss. */
static napi_value intersect_closest_many(napi_env env, napi_callback_info info) {
  napi_value a[6];
  size_t argc = 6;
  scene_box* box;
  void *rays, *prim, *t, *u = NULL, *v = NULL;
  size_t nr, np, nt, nu = 0, nv = 0;
  if (napi_get_cb_info(env, info, &argc, a, NULL, NULL) != napi_ok) return NULL;
  if (argc < 4) return type_error(env, "intersectClosestMany", "called with (scene, rays, prim, t[, u, v])"), NULL;
  if (!scene_of(env, a[0], &box) || !typed(env, a[1], napi_float32_array, "rays", "a Float32Array", &rays, &nr) ||
      !typed(env, a[2], napi_int32_array, "prim", "an Int32Array", &prim, &np) ||
      !typed(env, a[3], napi_float32_array, "t", "a Float32Array", &t, &nt))
    return NULL;
  if (argc >= 6 && (!typed(env, a[4], napi_float32_array, "u", "a Float32Array", &u, &nu) ||
                    !typed(env, a[5], napi_float32_array, "v", "a Float32Array", &v, &nv)))
    return NULL;
  const size_t n = nr / CT_RAY_FLOATS;
  if (nr % CT_RAY_FLOATS) return range_error(env, "rays", "must hold 8 floats per ray"), NULL;
  if (n > 0xFFFFFFFFu) return range_error(env, "rays", "holds more than 2^32 - 1 rays"), NULL;
  if (np != n || nt != n || (u && (nu != n || nv != n)))
    return range_error(env, "prim, t, u and v", "must hold one entry per ray"), NULL;
  ct_status st = ct_trace_closest(box->scene, (const float*)rays, (uint32_t)n, (int32_t*)prim, (float*)t, (float*)u,
                                  (float*)v, NULL);
  if (st != CT_OK) return library_error(env, st);
  return undefined(env);
}

/* occludedMany(scene, rays: Float32Array, blocked: Uint8Array): occluded (intersect.ts:368-420)
 * on (tMin, tMax) of every ray, 1 where blocked. */
static napi_value occluded_many(napi_env env, napi_callback_info info) {
  napi_value a[3];
  scene_box* box;
  void *rays, *out;
  size_t nr, no;
  if (!args(env, info, 3, a) || !scene_of(env, a[0], &box) ||
      !typed(env, a[1], napi_float32_array, "rays", "a Float32Array", &rays, &nr) ||
      !typed(env, a[2], napi_uint8_array, "blocked", "a Uint8Array", &out, &no))
    return NULL;
  const size_t n = nr / CT_RAY_FLOATS;
  if (nr % CT_RAY_FLOATS) return range_error(env, "rays", "must hold 8 floats per ray"), NULL;
  if (n > 0xFFFFFFFFu) return range_error(env, "rays", "holds more than 2^32 - 1 rays"), NULL;
  if (no != n) return range_error(env, "blocked", "must hold one entry per ray"), NULL;
  ct_status st = ct_trace_occluded(box->scene, (const float*)rays, (uint32_t)n, (uint8_t*)out, NULL);
  if (st != CT_OK) return library_error(env, st);
  return undefined(env);
}

/* ---- module registration ----------------------------------------------- */

CT_EXPORT int32_t node_api_module_get_api_version_v1(void) { return NAPI_VERSION; }

CT_EXPORT napi_value napi_register_module_v1(napi_env env, napi_value exports) {
  const napi_property_descriptor d[] = {
      {"sceneCreate", NULL, scene_create, NULL, NULL, NULL, napi_default, NULL},
      {"sceneDestroy", NULL, scene_destroy, NULL, NULL, NULL, napi_default, NULL},
      {"renderImage", NULL, render_image, NULL, NULL, NULL, napi_default, NULL},
      {"accumulatePass", NULL, accumulate_pass, NULL, NULL, NULL, napi_default, NULL},
      {"intersectClosestMany", NULL, intersect_closest_many, NULL, NULL, NULL, napi_default, NULL},
      {"occludedMany", NULL, occluded_many, NULL, NULL, NULL, napi_default, NULL},
  };
  if (napi_define_properties(env, exports, sizeof d / sizeof d[0], d) != napi_ok) {
    throw_once(env, "CT_NAPI", "napi_define_properties failed", 0);
    return NULL;
  }
  return exports;
}
