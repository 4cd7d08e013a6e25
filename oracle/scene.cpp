// Oracle (test infrastructure): RNG, vector helpers, scene model and the
// Cornell preset. Restates src/tracer/rng.ts, vec3.ts, scene.ts and
// scenes.ts of the reference.
#include <cmath>

#include "oracle.hpp"

namespace oracle {

// rng.ts:10-15. JS Math.imul/`>>> 0` arithmetic is uint32 arithmetic.
uint32_t pcg_hash(uint32_t input) {
  uint32_t state = input * 747796405u + 2891336453u;
  uint32_t shifted = (state >> ((state >> 28) + 4u)) ^ state;
  uint32_t word = shifted * 277803737u;
  return (word >> 22) ^ word;
}

// rng.ts:18-23
uint32_t seed_for(uint32_t pixel_index, uint32_t frame) {
  uint32_t a = pcg_hash(pixel_index);
  uint32_t b = pcg_hash(frame ^ 0x9e3779b9u);
  uint32_t s = pcg_hash(a ^ (b * 0x85ebca6bu));
  return s == 0 ? 0x1234567u : s;
}

// rng.ts:28-31
Rng::Rng(uint32_t seed) {
  uint32_t s = pcg_hash(seed);
  state = s == 0 ? 0x9e3779b9u : s;
}

// rng.ts:33-37
Rng Rng::from_pixel(uint32_t pixel_index, uint32_t frame) {
  Rng r(0);
  r.state = seed_for(pixel_index, frame);
  return r;
}

// rng.ts:40-49: xorshift32 with shifts 13, 17, 5.
uint32_t Rng::next_u32() {
  uint32_t x = state;
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  state = x;
  return x;
}

// rng.ts:52-54
double Rng::next() { return (double)next_u32() / 4294967296.0; }

// rng.ts:57-59
double Rng::range(double lo, double hi) { return lo + (hi - lo) * next(); }

// rng.ts:62-64
int32_t Rng::integer(int32_t n) {
  double f = std::floor(next() * (double)n);
  double m = (double)(n - 1);
  return (int32_t)(m < f ? m : f);
}

// vec3.ts:29-32
V3 normalize(V3 a) {
  double len = std::sqrt(dot(a, a));
  return len > 0 ? scale(a, 1.0 / len) : v3(0, 0, 0);
}

// scene.ts:85-94 (quadTriangles), 96-105 (meshTriangles), 107-118 (shapeTriangles)
void shape_triangles(const Shape& s, std::vector<Tri>& out) {
  switch (s.kind) {
    case SHAPE_SPHERE:
      return;
    case SHAPE_TRIANGLE:
      out.push_back(Tri{s.a, s.b, s.c});
      return;
    case SHAPE_QUAD: {
      V3 p0 = s.a;
      V3 p1 = add(s.a, s.b);
      V3 p2 = add(add(s.a, s.b), s.c);
      V3 p3 = add(s.a, s.c);
      out.push_back(Tri{p0, p1, p2});
      out.push_back(Tri{p0, p2, p3});
      return;
    }
    case SHAPE_MESH:
      for (size_t i = 0; i + 2 < s.indices.size(); i += 3)
        out.push_back(Tri{s.vertices[s.indices[i]], s.vertices[s.indices[i + 1]],
                          s.vertices[s.indices[i + 2]]});
      return;
  }
}

// scene.ts:129-140
uint32_t primitive_count(const Shape& s) {
  switch (s.kind) {
    case SHAPE_SPHERE:
    case SHAPE_TRIANGLE:
      return 1;
    case SHAPE_QUAD:
      return 2;
    case SHAPE_MESH:
      return (uint32_t)(s.indices.size() / 3);
  }
  return 0;
}

// scene.ts:120-122
V3 triangle_normal(const Tri& t) { return normalize(cross(sub(t.b, t.a), sub(t.c, t.a))); }

// scene.ts:124-127
double triangle_area(const Tri& t) {
  V3 c = cross(sub(t.b, t.a), sub(t.c, t.a));
  return 0.5 * std::sqrt(c.x * c.x + c.y * c.y + c.z * c.z);
}

// scene.ts:176-185
bool material_emission(const Material& m, V3* out) {
  if (m.type == CT_MAT_EMISSIVE) {
    *out = v3(m.color.x * m.param, m.color.y * m.param, m.color.z * m.param);
    return true;
  }
  if (m.type == CT_MAT_LAMBERTIAN && m.has_emission) {
    const V3& e = m.emission;
    if (e.x > 0 || e.y > 0 || e.z > 0) {
      *out = e;
      return true;
    }
  }
  return false;
}

// scenes.ts:26-40
CameraSettings camera_at(V3 eye, V3 target, double fov_deg, double lens_radius,
                         double focus_distance, bool has_focus) {
  double dx = eye.x - target.x, dy = eye.y - target.y, dz = eye.z - target.z;
  double distance = std::sqrt(dx * dx + dy * dy + dz * dz);
  CameraSettings c;
  c.target = target;
  c.yaw = std::atan2(dx, dz);
  c.pitch = std::asin(dy / distance);
  c.distance = distance;
  c.fov_deg = fov_deg;
  c.lens_radius = lens_radius;
  c.focus_distance = has_focus ? focus_distance : distance;
  return c;
}

static Shape quad_shape(V3 o, V3 u, V3 v) {
  Shape s;
  s.kind = SHAPE_QUAD;
  s.a = o;
  s.b = u;
  s.c = v;
  return s;
}
static Shape sphere_shape(V3 c, double r) {
  Shape s;
  s.kind = SHAPE_SPHERE;
  s.a = c;
  s.radius = r;
  return s;
}
static Material lambert(V3 albedo) {
  Material m;
  m.type = CT_MAT_LAMBERTIAN;
  m.color = albedo;
  return m;
}

// scenes.ts:45-67: the reference's CORNELL_BOX preset.
Scene cornell_box() {
  Scene s;
  const double W = 0.75;
  Material white = lambert(v3(0.73, 0.73, 0.73));
  Material red = lambert(v3(0.65, 0.05, 0.05));
  Material green = lambert(v3(0.12, 0.45, 0.15));
  Material light;
  light.type = CT_MAT_EMISSIVE;
  light.color = v3(1, 0.86, 0.7);
  light.param = 12;
  Material metal;
  metal.type = CT_MAT_METAL;
  metal.color = v3(0.9, 0.9, 0.92);
  metal.param = 0.02;
  Material glass;
  glass.type = CT_MAT_DIELECTRIC;
  glass.color = v3(1, 1, 1);
  glass.param = 1.5;
  auto push = [&](Shape sh, Material m) {
    s.shapes.push_back(sh);
    s.materials.push_back(m);
  };
  push(quad_shape(v3(-W, 0, -0.5), v3(2 * W, 0, 0), v3(0, 0, 1)), white);
  push(quad_shape(v3(-W, 1, -0.5), v3(2 * W, 0, 0), v3(0, 0, 1)), white);
  push(quad_shape(v3(-W, 0, -0.5), v3(2 * W, 0, 0), v3(0, 1, 0)), white);
  push(quad_shape(v3(-W, 0, -0.5), v3(0, 0, 1), v3(0, 1, 0)), red);
  push(quad_shape(v3(W, 0, -0.5), v3(0, 0, 1), v3(0, 1, 0)), green);
  push(quad_shape(v3(-0.2, 0.998, -0.15), v3(0.4, 0, 0), v3(0, 0, 0.3)), light);
  push(sphere_shape(v3(-0.33, 0.24, -0.12), 0.24), metal);
  push(sphere_shape(v3(0.3, 0.2, 0.17), 0.2), glass);
  s.camera = camera_at(v3(0, 0.5, 1.6), v3(0, 0.5, 0), 32, 0, 1.6, true);
  s.sky.gradient = false;
  return s;
}

}  // namespace oracle
