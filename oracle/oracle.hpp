// Oracle: CPU restatement of the caustic-tracer reference path tracer.
//
// TEST INFRASTRUCTURE ONLY. This code is the checker for the GPU library: the
// tests, the smoke check and the benchmark's CPU-baseline leg call it; the
// product never links, loads or falls back to it.
//
// Every function restates the reference's TypeScript (src/tracer/*.ts) with
// the same float64 arithmetic in the same operation order over the same
// Float32 storage, so outputs match the reference bit for bit except where the
// C library's transcendental functions (sin, cos, tan, cbrt, pow) round
// differently from V8's. Build with -ffp-contract=off and without fast-math.
// Parity is pinned by the reference's golden render out/cornell.ppm and the
// assertions of its test files (bvh/furnace/materials/reference.test.ts).
#pragma once

#include <cstdint>
#include <cstddef>
#include <vector>

#include "../include/caustic.h"

namespace oracle {

// ---- rng.ts:10-65 -------------------------------------------------------
uint32_t pcg_hash(uint32_t input);
uint32_t seed_for(uint32_t pixel_index, uint32_t frame);

struct Rng {
  uint32_t state;
  explicit Rng(uint32_t seed);
  static Rng from_pixel(uint32_t pixel_index, uint32_t frame);
  uint32_t next_u32();
  double next();
  double range(double lo, double hi);
  int32_t integer(int32_t n);
};

// ---- vec3.ts ---------------------------------------------------------------
struct V3 {
  double x, y, z;
};
inline V3 v3(double x, double y, double z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 scale(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
V3 normalize(V3 a);

// ---- scene.ts --------------------------------------------------------------
enum ShapeKind { SHAPE_SPHERE = 0, SHAPE_TRIANGLE = 1, SHAPE_QUAD = 2, SHAPE_MESH = 3 };

struct Shape {
  ShapeKind kind = SHAPE_SPHERE;
  V3 a{0, 0, 0}, b{0, 0, 0}, c{0, 0, 0};  // sphere: a = centre; quad: a=origin b=u c=v
  double radius = 0;
  std::vector<V3> vertices;
  std::vector<uint32_t> indices;
};

struct Material {
  int type = CT_MAT_LAMBERTIAN;
  V3 color{1, 1, 1};  // albedo | tint | emissive colour
  double param = 0;   // roughness | ior | strength
  bool checker = false;
  V3 color2{0, 0, 0};
  double checker_scale = 0;
  bool has_emission = false;
  V3 emission{0, 0, 0};
};

struct Sky {
  bool gradient = false;
  V3 zenith{0, 0, 0}, horizon{0, 0, 0};
  double strength = 0;
};

struct CameraSettings {
  V3 target{0, 0, 0};
  double yaw = 0, pitch = 0, distance = 1, fov_deg = 40, lens_radius = 0, focus_distance = 1;
};

struct Scene {
  std::vector<Shape> shapes;
  std::vector<Material> materials;
  CameraSettings camera;
  Sky sky;
};

struct Tri {
  V3 a, b, c;
};

// scene.ts:85-127,176-185
void shape_triangles(const Shape& s, std::vector<Tri>& out);
uint32_t primitive_count(const Shape& s);
V3 triangle_normal(const Tri& t);
double triangle_area(const Tri& t);
bool material_emission(const Material& m, V3* out);

// scenes.ts:26-40
CameraSettings camera_at(V3 eye, V3 target, double fov_deg, double lens_radius,
                         double focus_distance, bool has_focus);
// scenes.ts:45-67
Scene cornell_box();

// ---- bvh.ts / pack.ts ------------------------------------------------------
struct Packed {
  std::vector<float> prims, nodes, mats;
  uint32_t prim_count = 0, node_count = 0, mat_count = 0;
  std::vector<int32_t> lights;
  std::vector<uint32_t> prim_object;
  std::vector<uint32_t> order;
  Sky sky;
};

Packed pack_scene(const Scene& scene);  // pack.ts:195-223

struct BvhReport {
  bool ok;
  uint32_t max_leaf_size, leaf_count, depth, errors;
};
BvhReport validate_bvh(const float* nodes, uint32_t node_count, const uint32_t* order,
                       uint32_t order_len, uint32_t prim_count);  // bvh.ts:319-381

// ---- packed-scene view used by traversal and tracing ----------------------
struct View {
  const float* prims;
  uint32_t prim_count;
  const float* nodes;
  uint32_t node_count;
  const float* mats;
  uint32_t mat_count;
  const int32_t* lights;
  uint32_t light_count;
  const uint32_t* prim_object;
  Sky sky;
};
View view_of(const Packed& p);
View view_of(const ct_packed_scene_view& v);

// ---- intersect.ts ------------------------------------------------------------
constexpr double T_MIN = 1e-4;

struct Hit {
  double t;
  int32_t prim;
  double u, v;
};

// Work counters of one query: box tests, triangle tests, sphere tests, nodes visited.
struct Counters {
  uint64_t aabb = 0, tri = 0, sphere = 0, nodes = 0;
};

double ray_sphere(double ox, double oy, double oz, double dx, double dy, double dz, double cx,
                  double cy, double cz, double r, double tmin, double tmax);
bool ray_triangle(double ox, double oy, double oz, double dx, double dy, double dz, double ax,
                  double ay, double az, double bx, double by, double bz, double cx, double cy,
                  double cz, double tmin, double tmax, double* t, double* u, double* v);
double ray_aabb(double ox, double oy, double oz, double idx, double idy, double idz, double minx,
                double miny, double minz, double maxx, double maxy, double maxz, double tmax);

bool intersect_closest(const View& ps, double ox, double oy, double oz, double dx, double dy,
                       double dz, double tmin, double tmax, Hit* hit, Counters* c = nullptr);
bool intersect_closest_stackless(const View& ps, double ox, double oy, double oz, double dx,
                                 double dy, double dz, double tmin, double tmax, Hit* hit,
                                 Counters* c = nullptr);
bool occluded(const View& ps, double ox, double oy, double oz, double dx, double dy, double dz,
              double tmin, double tmax, Counters* c = nullptr);
bool intersect_brute_force(const View& ps, double ox, double oy, double oz, double dx, double dy,
                           double dz, double tmin, double tmax, Hit* hit);

// ---- materials.ts ------------------------------------------------------------
extern const double INV_PI;
extern const double TWO_PI;
void basis_into(double nx, double ny, double nz, double out[6]);
void cosine_hemisphere_into(double nx, double ny, double nz, double u1, double u2, double out[3]);
void unit_vector_into(double u1, double u2, double out[3]);
double schlick(double cos_theta, double eta_i, double eta_t);
double dielectric_reflectance(double cos_i, double eta_i, double eta_t);
void metal_into(double dx, double dy, double dz, double nx, double ny, double nz, double roughness,
                double u1, double u2, double u3, double out[3]);
bool dielectric_into(double dx, double dy, double dz, double nx, double ny, double nz, double ior,
                     bool front_face, double u, double out[3]);
double power_heuristic(double a, double b);
bool checker_primary(double px, double py, double pz, double cells);

// ---- camera.ts -----------------------------------------------------------------
struct Frame {
  V3 origin, right, up, forward;
  double tan_half_fov, aspect, lens_radius, focus_distance;
};
V3 camera_position(const CameraSettings& cam);
Frame camera_frame(const CameraSettings& cam, double aspect);
void generate_ray(const Frame& f, double sx, double sy, double lx, double ly, V3* origin, V3* dir);

// ---- tracer.ts -----------------------------------------------------------------
struct TraceOptions {
  int max_bounces = 8;
  bool russian_roulette = true;
  bool nee = true;
};

double light_pdf(const View& ps, double px, double py, double pz, double hx, double hy, double hz,
                 double hnx, double hny, double hnz, int32_t prim);
bool sample_light(const View& ps, double px, double py, double pz, Rng& rng, double out[8]);
// Radiance of one path; also counts closest-hit and shadow rays when given.
void radiance(const View& ps, double ox, double oy, double oz, double dx, double dy, double dz,
              Rng& rng, const TraceOptions& opts, double out[3], uint64_t* closest_rays = nullptr,
              uint64_t* shadow_rays = nullptr, Counters* closest_work = nullptr,
              Counters* shadow_work = nullptr);
// accumulatePass over rows [y0, y1); sumsq (optional) gets squared samples.
void accumulate_pass_rows(const View& ps, const Frame& f, int width, int height,
                          uint32_t frame_index, const TraceOptions& opts, float* accum,
                          double* sumsq, int y0, int y1);
void accumulate_pass(const View& ps, const Frame& f, int width, int height, uint32_t frame_index,
                     const TraceOptions& opts, float* accum);
// renderImage with `threads` workers splitting rows (results do not depend on it).
std::vector<float> render_image(const View& ps, const Frame& f, int width, int height, int spp,
                                uint32_t seed, const TraceOptions& opts, int threads = 1,
                                double* sumsq = nullptr);

// ---- tonemap.ts / ppm.ts ---------------------------------------------------------
double aces_fitted(double x);
double reinhard(double x);
double linear_to_srgb(double x);
double js_round(double x);
void tonemap_buffer(const float* accum, int width, int height, double samples, double exposure_ev,
                    bool aces, uint8_t* rgba);
std::vector<uint8_t> encode_ppm(int width, int height, const uint8_t* rgba);

}  // namespace oracle
