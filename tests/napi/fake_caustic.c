/*
 * fake_caustic.c - a recording stand-in for libcaustic_gb300, for testing the
 * Node-API addon's argument handling on a machine without a GPU.
 *
 * TEST INFRASTRUCTURE. It defines the ct_* entry points the addon calls
 * (include/caustic.h), records the arguments each received, fills outputs with
 * values that identify the call, and fails on request with a given status and
 * ct_last_error() message (fake_fail_next).
 */
#include <stdlib.h>
#include <string.h>

#include "caustic.h"

struct ct_scene {
  int id;
};

static ct_packed_scene_view g_view;
static float g_first_prim[16];
static ct_camera_frame g_frame;
static ct_render_options g_ropts;
static ct_trace_options g_topts;
static int32_t g_width, g_height;
static uint32_t g_frame_index, g_rays;
static int g_created, g_destroyed, g_uv;
static ct_status g_fail = CT_OK;
static char g_msg[256];

void fake_fail_next(ct_status st, const char* msg) {
  g_fail = st;
  strncpy(g_msg, msg ? msg : "", sizeof g_msg - 1);
}

static ct_status consume_failure(void) {
  ct_status st = g_fail;
  g_fail = CT_OK;
  return st;
}

const ct_packed_scene_view* fake_view(void) { return &g_view; }
const float* fake_first_prim(void) { return g_first_prim; }
const ct_camera_frame* fake_frame(void) { return &g_frame; }
const ct_render_options* fake_render_options(void) { return &g_ropts; }
const ct_trace_options* fake_trace_options(void) { return &g_topts; }
void fake_pass_args(int32_t* w, int32_t* h, uint32_t* frame_index) {
  *w = g_width;
  *h = g_height;
  *frame_index = g_frame_index;
}
uint32_t fake_rays(void) { return g_rays; }
int fake_uv(void) { return g_uv; }
void fake_counts(int* created, int* destroyed) {
  *created = g_created;
  *destroyed = g_destroyed;
}

const char* ct_last_error(void) { return g_msg; }

ct_status ct_scene_create(const ct_packed_scene_view* ps, ct_scene** out) {
  ct_status st = consume_failure();
  if (st != CT_OK) return st;
  g_view = *ps;
  if (ps->prim_count) memcpy(g_first_prim, ps->prims, sizeof g_first_prim);
  *out = (ct_scene*)calloc(1, sizeof(ct_scene));
  (*out)->id = ++g_created;
  return CT_OK;
}

void ct_scene_destroy(ct_scene* scene) {
  if (scene) g_destroyed++;
  free(scene);
}

ct_status ct_render_image(ct_scene* scene, const ct_camera_frame* frame, const ct_render_options* o, float* out,
                          ct_stats* stats) {
  (void)scene;
  (void)stats;
  ct_status st = consume_failure();
  if (st != CT_OK) return st;
  g_frame = *frame;
  g_ropts = *o;
  const size_t n = (size_t)o->width * o->height * 3;
  for (size_t i = 0; i < n; i++) out[i] = (float)(i % 7) + 0.25f * (float)o->spp;
  return CT_OK;
}

ct_status ct_accumulate_pass(ct_scene* scene, const ct_camera_frame* frame, int32_t width, int32_t height,
                             uint32_t frame_index, const ct_trace_options* opts, float* accum, ct_stats* stats) {
  (void)scene;
  (void)stats;
  ct_status st = consume_failure();
  if (st != CT_OK) return st;
  g_frame = *frame;
  g_topts = *opts;
  g_width = width;
  g_height = height;
  g_frame_index = frame_index;
  const size_t n = (size_t)width * height * 3;
  for (size_t i = 0; i < n; i++) accum[i] += 1.0f + (float)(frame_index % 5);
  return CT_OK;
}

ct_status ct_trace_closest(ct_scene* scene, const float* rays, uint32_t count, int32_t* prim, float* t, float* u,
                           float* v, ct_stats* stats) {
  (void)scene;
  (void)stats;
  ct_status st = consume_failure();
  if (st != CT_OK) return st;
  g_rays = count;
  g_uv = u != NULL && v != NULL;
  for (uint32_t i = 0; i < count; i++) {
    prim[i] = (int32_t)i - 1;
    t[i] = rays[(size_t)CT_RAY_FLOATS * i + 7];
    if (u) u[i] = 0.25f;
    if (v) v[i] = 0.5f;
  }
  return CT_OK;
}

ct_status ct_trace_occluded(ct_scene* scene, const float* rays, uint32_t count, uint8_t* blocked, ct_stats* stats) {
  (void)scene;
  (void)rays;
  (void)stats;
  ct_status st = consume_failure();
  if (st != CT_OK) return st;
  g_rays = count;
  for (uint32_t i = 0; i < count; i++) blocked[i] = (uint8_t)(i & 1u);
  return CT_OK;
}
