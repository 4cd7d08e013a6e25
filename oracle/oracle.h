/*
 * C ABI of the oracle library (oracle/_build/liboracle.so).
 *
 * TEST INFRASTRUCTURE ONLY: the CPU restatement of the reference path tracer
 * that the tests, the smoke check and the benchmark's CPU-baseline leg use as
 * the checker. The product library never links or loads it.
 */
#ifndef CAUSTIC_ORACLE_H
#define CAUSTIC_ORACLE_H

#include <stdint.h>

#include "../include/caustic.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CameraSettings (scene.ts:55-67). */
typedef struct or_camera_settings {
  double target[3];
  double yaw, pitch, distance, fov_deg, lens_radius, focus_distance;
} or_camera_settings;

typedef struct or_packed or_packed; /* oracle-owned packed scene */

/* rng.ts */
uint32_t or_pcg_hash(uint32_t x);
uint32_t or_seed_for(uint32_t pixel, uint32_t frame);
/* n draws of Rng(seed).next() (kind 0), nextU32() (kind 1) or range(lo,hi) (kind 2) */
void or_rng_stream(uint32_t seed, uint32_t n, int32_t kind, double lo, double hi, double* out);
/* The same draws continuing from a raw xorshift state; returns the state reached. */
uint32_t or_rng_stream_state(uint32_t state, uint64_t n, int32_t kind, double lo, double hi, double* out);

/* packScene (pack.ts:195-223) of a scene description or of the CORNELL_BOX preset. */
or_packed* or_pack(const ct_object* objects, uint32_t count, const ct_sky* sky);
or_packed* or_pack_cornell(or_camera_settings* camera_out);
void or_packed_view(const or_packed* p, ct_packed_scene_view* view, const uint32_t** order);
void or_packed_free(or_packed* p);
/* validateBvh (bvh.ts:319-381): out = {ok, maxLeafSize, leafCount, depth, errors} */
void or_validate_bvh(const ct_packed_scene_view* v, const uint32_t* order, uint32_t order_len,
                     uint32_t out[5]);

/* Batched ray queries over CT_RAY_FLOATS-float rays.
 * mode 0 = intersectClosest (ordered walk), 1 = intersectClosestStackless,
 * 2 = intersectBruteForce. counters = {aabb, tri, sphere, nodes} (may be NULL). */
void or_trace(const ct_packed_scene_view* v, const float* rays, uint64_t count, int32_t mode,
              int32_t* prim, double* t, double* u, double* vv, uint64_t counters[4],
              int32_t threads);
void or_occluded(const ct_packed_scene_view* v, const float* rays, uint64_t count,
                 uint8_t* blocked, uint64_t counters[4], int32_t threads);
/* float64 distance at which `prim` is hit by a ray (-1 = not hit in (tmin,tmax)). */
double or_prim_hit_t(const ct_packed_scene_view* v, int32_t prim, const float ray[8]);

/* camera.ts */
void or_camera_frame(const or_camera_settings* cam, double aspect, ct_camera_frame* out);
void or_generate_ray(const ct_camera_frame* f, double sx, double sy, double lx, double ly,
                     double out[6]);

/* tracer.ts: renderImage / accumulatePass. sumsq (may be NULL) accumulates the
 * squared per-pixel samples. rays_out (may be NULL) = {closest, shadow}.   */
void or_render_image(const ct_packed_scene_view* v, const ct_camera_frame* f,
                     const ct_render_options* o, int32_t threads, float* out, double* sumsq);
void or_accumulate_pass(const ct_packed_scene_view* v, const ct_camera_frame* f, int32_t width,
                        int32_t height, uint32_t frame_index, const ct_trace_options* o,
                        float* accum, int32_t threads);
/* radiance of the single path of pixel `pixel` in pass `frame_index`; work (may
 * be NULL) = {closest rays, shadow rays, closest-query box/triangle/sphere
 * tests and nodes, shadow-query box/triangle/sphere tests and nodes}.      */
void or_pixel_radiance(const ct_packed_scene_view* v, const ct_camera_frame* f, int32_t width,
                       int32_t height, uint32_t pixel, uint32_t frame_index,
                       const ct_trace_options* o, double out[3], uint64_t work[10]);

/* renderCornellReference (reference.ts:20-43) with its defaults (RR on, NEE on,
 * 8 bounces, seed 1, ACES, EV 0): linear w*h*3, rgba w*h*4.              */
void or_cornell_reference(int32_t width, int32_t height, int32_t spp, int32_t threads,
                          float* linear, uint8_t* rgba);
/* tonemap.ts / materials.ts scalar helpers for the known-answer tests. */
void or_tonemap(const float* accum, int32_t width, int32_t height, double samples, double ev,
                int32_t aces, uint8_t* rgba);
double or_scalar(int32_t fn, double a, double b, double c);
void or_vector(int32_t fn, const double* in, double* out);

#ifdef __cplusplus
}
#endif

#endif
