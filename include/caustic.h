/*
 * caustic.h - C ABI of the GB300 (sm_103a) path tracer library `libcaustic_gb300.so`.
 *
 * This is the drop-in boundary for the reference's CPU path tracer
 * (caustic-tracer, src/tracer/). A host written in any language binds these
 * functions through its FFI: the reference's TypeScript host through an
 * N-API addon, the Python host in this repository through ctypes.
 *
 * Conventions
 *   - Every function returns a ct_status; on failure ct_last_error() returns a
 *     message for the calling thread. No C++ exception crosses this boundary.
 *   - The caller owns every array passed in. Host arrays are borrowed for the
 *     duration of the call only; a ct_scene keeps its own device copies.
 *   - A ct_scene owns one CUDA stream. Calls on the same handle are serialised
 *     by an internal lock; distinct handles may be used from distinct threads.
 *   - "_device" entry points take device pointers and a cudaStream_t (passed as
 *     void*); they enqueue work and return without synchronising.
 *
 * Array layouts are the reference's packed layouts (pack.ts:6-17, bvh.ts:6-15):
 *   prims  float[16 * prim_count]  [a.xyz,type | b.xyz(r),object | c.xyz,area | n.xyz,0]
 *   nodes  float[8 * node_count]   [min.xyz,skip | max.xyz,leaf]  leaf = start*8+count or -1
 *   mats   float[16 * max(1,mat_count)] [rgb,type | param,checkerScale,checkerOn,0 | rgb2,0 | e.rgb,0]
 *   lights int32[light_count]      packed indices of emitting primitives
 *   prim_object uint32[prim_count] packed primitive -> scene object
 */
#ifndef CAUSTIC_H
#define CAUSTIC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CT_ABI_VERSION 1

/* Layout constants: pack.ts:30-44 and bvh.ts:18-20. */
#define CT_PRIM_STRIDE 16
#define CT_NODE_STRIDE 8
#define CT_MAT_STRIDE 16
#define CT_MAX_LEAF_PRIMS 4
#define CT_SAH_BUCKETS 12
#define CT_PRIM_SPHERE 0
#define CT_PRIM_TRIANGLE 1
#define CT_MAT_LAMBERTIAN 0
#define CT_MAT_METAL 1
#define CT_MAT_DIELECTRIC 2
#define CT_MAT_EMISSIVE 3

/* Ray record for the batched queries: 8 floats = 32 bytes per ray. */
#define CT_RAY_FLOATS 8 /* ox oy oz dx dy dz tmin tmax */

typedef enum ct_status {
  CT_OK = 0,
  CT_ERR_INVALID_ARGUMENT = 1,
  CT_ERR_CUDA = 2,
  CT_ERR_OUT_OF_MEMORY = 3,
  CT_ERR_UNSUPPORTED = 4,
  CT_ERR_TIMEOUT = 5,
  CT_ERR_BUDGET = 6,
  CT_ERR_CANCELLED = 7,
  CT_ERR_NOT_FOUND = 8
} ct_status;

/* Sky (scene.ts:50-52): kind 0 = none, 1 = gradient. */
typedef struct ct_sky {
  int32_t kind;
  double zenith[3];
  double horizon[3];
  double strength;
} ct_sky;

/* CameraFrame (camera.ts:8-20): world-space thin-lens camera. */
typedef struct ct_camera_frame {
  double origin[3];
  double right[3];
  double up[3];
  double forward[3];
  double tan_half_fov;
  double aspect;
  double lens_radius;
  double focus_distance;
} ct_camera_frame;

/* TraceOptions (tracer.ts:27-31). Booleans are 0/1. */
typedef struct ct_trace_options {
  int32_t max_bounces;
  int32_t russian_roulette;
  int32_t nee;
} ct_trace_options;

/* RenderOptions (tracer.ts:337-342): TraceOptions + image size, spp, seed. */
typedef struct ct_render_options {
  int32_t width;
  int32_t height;
  int32_t spp;
  int32_t max_bounces;
  int32_t russian_roulette;
  int32_t nee;
  uint32_t seed;
} ct_render_options;

/* PackedScene (pack.ts:46-59) as borrowed host arrays. */
typedef struct ct_packed_scene_view {
  const float* prims;
  uint32_t prim_count;
  const float* nodes;
  uint32_t node_count;
  const float* mats;
  uint32_t mat_count;
  const int32_t* lights;
  uint32_t light_count;
  const uint32_t* prim_object;
  ct_sky sky;
} ct_packed_scene_view;

/* Scene description consumed by the host packer (scene.ts:21-74).
 * Shape kinds: 0 sphere (p[0..2] centre, p[3] radius), 1 triangle (p = a,b,c),
 * 2 quad (p = origin,u,v), 3 mesh (vertices xyz triples + index triples).   */
typedef struct ct_shape {
  int32_t kind;
  double p[9];
  const double* vertices;
  uint32_t vertex_count;
  const uint32_t* indices;
  uint32_t index_count;
} ct_shape;

/* Material (scene.ts:21-31). type uses CT_MAT_*; color is albedo (lambertian,
 * metal), tint (dielectric, default 1,1,1) or colour (emissive); param is
 * roughness | ior | strength.                                              */
typedef struct ct_material {
  int32_t type;
  double color[3];
  double param;
  int32_t has_checker;
  double checker_color2[3];
  double checker_scale;
  int32_t has_emission;
  double emission[3];
} ct_material;

typedef struct ct_object {
  ct_shape shape;
  ct_material material;
} ct_object;

/* Host-side packed scene produced by ct_pack_scene; arrays owned by the library. */
typedef struct ct_packed_scene {
  ct_packed_scene_view view;
  const uint32_t* order; /* order[i] = scene-order primitive stored at packed slot i */
} ct_packed_scene;

typedef struct ct_scene ct_scene; /* device-resident scene (opaque) */

/* Per-call statistics filled by the query/render entry points when non-NULL. */
typedef struct ct_stats {
  double kernel_ms;       /* device time of the dominant kernel(s), CUDA events */
  double total_ms;        /* device time of the whole call */
  uint64_t rays;          /* closest-hit + shadow rays traced */
  uint64_t fp64_fallbacks;/* primitive tests re-run in float64 at a decision boundary */
  uint32_t launches;      /* kernels launched by the call */
} ct_stats;

/* ---- library ---------------------------------------------------------- */

/* ABI version of the loaded library (== CT_ABI_VERSION). */
int32_t ct_abi_version(void);

/* Message describing the last failure on the calling thread ("" if none). */
const char* ct_last_error(void);

/* ---- host packer --------------------------------------------------------
 * packScene (pack.ts:195-223): enumerate primitives in scene order, build the
 * binned-SAH BVH (bvh.ts:111-296), reorder primitives into leaf order and
 * collect emitters. Runs on the host; the result is bit-identical to the
 * reference's Float32 arrays.                                              */
ct_status ct_pack_scene(const ct_object* objects, uint32_t object_count, const ct_sky* sky,
                        ct_packed_scene** out);
void ct_packed_scene_free(ct_packed_scene* ps);

/* Rng (rng.ts:25-65) for host-side scene generators: writes n draws of
 * next() (kind 0), nextU32() (kind 1) or range(lo, hi) (kind 2). The stream
 * starts from Rng(seed) when is_state == 0, else from the raw xorshift state
 * `seed_or_state`; the state reached is returned so a stream can continue. */
uint32_t ct_rng_stream(uint32_t seed_or_state, int32_t is_state, uint64_t n, int32_t kind,
                       double lo, double hi, double* out);

/* ---- device scene -------------------------------------------------------
 * Uploads a PackedScene (pack.ts:46-59) and derives the GPU traversal layout.
 * Replaces the implicit "arrays are readable" contract of the reference's
 * tracer (tracer.ts:348, intersect.ts:202).                                 */
ct_status ct_scene_create(const ct_packed_scene_view* ps, ct_scene** out);
/* Waits for the scene's own stream and returns its arrays (one allocation
 * from the per-device pool) to the pool. Batches that read the scene must be
 * finished or destroyed first (ct_batch_destroy waits for its run).       */
void ct_scene_destroy(ct_scene* scene);
/* Device bytes held by the scene (for admission budgets). Path state of a
 * render or batch is not part of it: it comes from a per-device
 * stream-ordered pool for the duration of the call's work, and the pool
 * keeps its high-water mark for reuse (168 bytes per path in flight: a
 * render of several waves holds up to four sets of 48 Mi paths, 33 GiB, and
 * so does a batch of several waves).                                     */
uint64_t ct_scene_device_bytes(const ct_scene* scene);

/* Per-scene tuning knobs, set by callers or an autotuner. No counterpart in
 * the reference (its CPU loop has nothing to tune).
 *   CT_OPT_WALK        integrator trace walk: -1 chosen from the tree (default),
 *                      0 ordered walk per thread, 1 ordered walk with persistent
 *                      lane refill, 2 stackless skip-link walk (intersect.ts:290)
 *   CT_OPT_WAVE_PATHS  paths per wave (0 = library default: half the render's
 *                      paths, at least 16 Mi and at most 48 Mi)
 *   CT_OPT_TRACE_BLOCKS  resident 128-thread blocks per SM of the integrator's
 *                      trace (or whole-path) launches of a single-scene render,
 *                      1..64, capped at the kernel's occupancy (0 = as many as
 *                      fit, the default). Changes timing only, not images.   */
#define CT_OPT_WALK 1
#define CT_OPT_WAVE_PATHS 2
#define CT_OPT_TRACE_BLOCKS 3
/*   CT_OPT_PATH_KERNEL 1 (default): single-scene renders of scenes of at most
 *                      32 primitives run each path whole in one lane; 0: they
 *                      run the wavefront kernels like every other scene. The
 *                      images are the same bit for bit.                      */
#define CT_OPT_PATH_KERNEL 4
ct_status ct_scene_set_option(ct_scene* scene, int32_t option, int64_t value);
/* Trace walk the integrator uses for the scene (0, 1 or 2 as above: the
 * CT_OPT_WALK value, or the choice from the tree); -1 for a NULL scene. A
 * scheduler groups jobs by it (ct_batch gives each walk waves of its own). */
int32_t ct_scene_walk(const ct_scene* scene);

/* ---- ray queries --------------------------------------------------------
 * intersectClosest (intersect.ts:202-282) over a batch of rays. rays holds
 * CT_RAY_FLOATS floats per ray. prim receives the packed primitive index or
 * -1, t the hit distance (+inf on a miss); u, v (may be NULL) the triangle
 * barycentrics (0 for sphere hits). Host pointers. Batches of at least 8 Mi
 * rays run in 4 Mi-ray chunks whose copies overlap the previous chunk's
 * trace (pinned host memory lets the copies run asynchronously); stats then
 * count one launch per chunk and kernel_ms spans the first chunk's trace to
 * the last one's end.                                                      */
ct_status ct_trace_closest(ct_scene* scene, const float* rays, uint32_t count, int32_t* prim,
                           float* t, float* u, float* v, ct_stats* stats);
/* occluded (intersect.ts:368-420): blocked[i] = 1 when anything is hit in
 * (tmin, tmax). Host pointers.                                              */
ct_status ct_trace_occluded(ct_scene* scene, const float* rays, uint32_t count, uint8_t* blocked,
                            ct_stats* stats);
/* Device-pointer variants; enqueue on `stream` (cudaStream_t, NULL = the
 * scene's stream) without synchronising. u and v may be NULL.               */
ct_status ct_trace_closest_device(ct_scene* scene, const float* rays, uint32_t count,
                                  int32_t* prim, float* t, float* u, float* v, void* stream);
ct_status ct_trace_occluded_device(ct_scene* scene, const float* rays, uint32_t count,
                                   uint8_t* blocked, void* stream);

/* Traversal variant used by the query entry points:
 * 0 = ordered short-stack walk (near child first) with persistent lane
 * refill, 1 = stackless skip-link walk (intersect.ts:290-365), 2 = ordered
 * walk, one query per thread. Returns the previous value.                  */
int32_t ct_set_traversal(int32_t variant);

/* ---- integrator ---------------------------------------------------------
 * accumulatePass (tracer.ts:361-395): one sample per pixel, seeded by
 * Rng.fromPixel(pixel, frame_index), added into accum (sum, not mean;
 * width*height*3 floats, row 0 = top). Host pointer, read and written.      */
ct_status ct_accumulate_pass(ct_scene* scene, const ct_camera_frame* frame, int32_t width,
                             int32_t height, uint32_t frame_index, const ct_trace_options* opts,
                             float* accum, ct_stats* stats);
/* renderImage (tracer.ts:348-355): opts->spp passes with frame index
 * s + seed*7919, then scaled by 1/spp. out: width*height*3 floats (host).   */
ct_status ct_render_image(ct_scene* scene, const ct_camera_frame* frame,
                          const ct_render_options* opts, float* out, ct_stats* stats);
/* Device-pointer variants. accum/out are device arrays; sumsq (may be NULL)
 * receives the per-pixel sum of squared samples for variance estimates.     */
ct_status ct_accumulate_passes_device(ct_scene* scene, const ct_camera_frame* frame,
                                      int32_t width, int32_t height, uint32_t first_frame_index,
                                      int32_t passes, const ct_trace_options* opts, float* accum,
                                      float* sumsq, void* stream);
ct_status ct_render_image_device(ct_scene* scene, const ct_camera_frame* frame,
                                 const ct_render_options* opts, float* out, void* stream);

/* ---- batched rendering ----------------------------------------------------
 * Many scenes, cameras and image sizes rendered together. No single
 * counterpart in the reference: each job is `passes` calls of accumulatePass
 * (tracer.ts:361-395) with frame indices first_frame_index + k, adding into
 * the job's device sum buffer `accum` (width*height*3 floats). Results equal
 * those of the single-scene entry points for the same frame indices.
 * The paths of all jobs share waves of up to wave_paths paths (0 = 48 Mi),
 * up to four waves in flight on as many streams, added in pass order;
 * walk selects the trace walk: -1 = each job the walk its scene uses alone
 * (so every result equals its single-scene render bit for bit; a wave holds
 * jobs of one walk), or 0 ordered per thread, 1 ordered with persistent lane
 * refill, 2 stackless skip-link for all jobs. ct_batch_info reports 3 for -1.
 * The first ct_batch_run captures the whole launch sequence in a CUDA graph;
 * later runs replay it. Scenes must outlive the batch and must not be used
 * by other calls while a run is in flight.                                  */
typedef struct ct_batch_job {
  ct_scene* scene;
  ct_camera_frame frame;
  int32_t width;
  int32_t height;
  uint32_t first_frame_index;
  int32_t passes;
  float* accum;
} ct_batch_job;

typedef struct ct_batch ct_batch;

ct_status ct_batch_create(const ct_batch_job* jobs, uint32_t count, const ct_trace_options* opts,
                          int64_t wave_paths, int32_t walk, ct_batch** out);
/* Replaces every job's first frame index (one per job) for the next run. */
ct_status ct_batch_set_first_frames(ct_batch* batch, const uint32_t* first_frame_index);
/* Enqueues the batch on `stream` (NULL = the batch's own stream). */
ct_status ct_batch_run(ct_batch* batch, void* stream);
/* Same work launched directly, without capturing a graph: for batches run
 * once (a serving step whose set of jobs changes every time).              */
ct_status ct_batch_run_direct(ct_batch* batch, void* stream);
/* ct_batch_run_direct whose sums are added only after those of the most
 * recent run of `after` (NULL: none), which may run on another stream: two
 * batches that add passes of the same jobs (consecutive serving steps) then
 * overlap on the GPU while every pixel's passes stay in pass order. `after`
 * must have been run and must not be destroyed before this call returns.
 * No counterpart in the reference: accumulatePass (tracer.ts:361) in order. */
ct_status ct_batch_run_direct_after(ct_batch* batch, void* stream, const ct_batch* after);
ct_status ct_batch_info(const ct_batch* batch, uint32_t* waves, uint64_t* paths, uint64_t* graph_nodes,
                        int32_t* walk);
void ct_batch_destroy(ct_batch* batch);

/* ---- accumulatePass without allocation ------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device
 * memory when they render: real-time loops that forbid allocation per frame
 * (an allocation can stall on the device and miss the frame), plugin hosts
 * that hand the library a fixed memory budget at load time and own every
 * later allocation, and deployments that must reserve all device memory up
 * front. Same work as ct_accumulate_pass (one sample per pixel, seeded by
 * Rng.fromPixel(pixel, frame_index), added into accum, through the same
 * kernels and launch shapes the scene's options select), but all scratch
 * lives in one static device array of the library, sized for
 * CT_NOALLOC_MAX_PIXELS pixels (42 MiB; every GPU that loads the library
 * holds it until the process exits). Larger images are rejected with
 * CT_ERR_INVALID_ARGUMENT. accum is a device array (width*height*3 floats);
 * the scene comes from ct_scene_create. The first call on a device (and the
 * first after that device's context was reset) looks the array's address up
 * for that device; make that first call before any stream capture. All calls
 * share the one array and it keeps the last call's contents (each call clears
 * the queue counters it needs), so calls that overlap on the GPU (on
 * different streams or different scenes) race: order them on one stream.  */
#define CT_NOALLOC_MAX_PIXELS (512u * 512u)
ct_status ct_accumulate_pass_noalloc(ct_scene* scene, const ct_camera_frame* frame, int32_t width,
                                     int32_t height, uint32_t frame_index, const ct_trace_options* opts,
                                     float* accum, void* stream);

/* ---- either side of the path ----------------------------------------------
 * tonemapBuffer (tonemap.ts:41-62) on the device: the sum buffer `accum`
 * (width*height*3 floats, device) divided by `samples`, scaled by
 * 2^exposure_ev, tone mapped (mode 0 = ACES fit, 1 = Reinhard), sRGB encoded
 * and rounded like Math.round into `rgba` (width*height*4 bytes, device,
 * 4-byte aligned, alpha 255). Every byte equals the reference's float64
 * result (float32 with a float64 recomputation near rounding boundaries).
 * Enqueued on `stream` (cudaStream_t, NULL = default stream).              */
ct_status ct_tonemap_device(const float* accum, int32_t width, int32_t height, double samples,
                            double exposure_ev, int32_t mode, uint8_t* rgba, void* stream);
/* tonemapBuffer then encodePPM (ppm.ts:4-16) on the device: writes the
 * binary PPM file (header "P6\n<w> <h>\n255\n", then RGB rows from the top)
 * into `ppm` (device, `capacity` bytes); *size receives the file size. A
 * buffer that is too small is rejected (CT_ERR_INVALID_ARGUMENT, *size set). */
ct_status ct_ppm_device(const float* accum, int32_t width, int32_t height, double samples, double exposure_ev,
                        int32_t mode, uint8_t* ppm, uint64_t capacity, uint64_t* size, void* stream);
/* pick (picking.ts:21-33) for `count` screen positions (sx, sy in [0, 1],
 * sy = 1 at the top): the pinhole ray of primaryRay (camera.ts:75) in
 * float64, rounded to the float32 ray record, tMin = T_MIN; closest hit as
 * ct_trace_closest. object[i] = primObject[prim] or -1, prim[i], t[i]
 * (+inf on a miss), point[3i..3i+2] = origin + dir * t in float64 (NaN on a
 * miss; `point` may be NULL). Host pointers.                               */
ct_status ct_pick(ct_scene* scene, const ct_camera_frame* frame, uint32_t count, const double* sx,
                  const double* sy, int32_t* object, int32_t* prim, float* t, double* point);

/* ---- profiling ------------------------------------------------------------
 * No counterpart in the reference (which times with performance.now(),
 * reference.ts:28,42). While enabled, every kernel launch is bracketed by
 * CUDA events on its stream; ct_profile_read sums device time and launch
 * counts per kernel name (static strings) and returns the number of kernels. */
void ct_profile_enable(int32_t on);
void ct_profile_reset(void);
int32_t ct_profile_read(const char** names, double* ms, uint64_t* launches, int32_t capacity);

#ifdef __cplusplus
}
#endif

#endif /* CAUSTIC_H */
