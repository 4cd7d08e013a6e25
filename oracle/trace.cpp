// Oracle (test infrastructure): ray queries, material sampling, camera and
// the path integrator. Restates src/tracer/intersect.ts, materials.ts,
// camera.ts and tracer.ts of the reference in float64.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <string>
#include <thread>

#include "oracle.hpp"

namespace oracle {

namespace {
constexpr double INF = std::numeric_limits<double>::infinity();
constexpr double PI = 3.14159265358979323846;
constexpr double SHADOW_SHORTEN = 1 - 1e-3;  // tracer.ts:36
inline double safe_inv(double d) { return 1 / (d == 0 ? 1e-20 : d); }  // intersect.ts:142
}  // namespace

const double INV_PI = 1 / PI;
const double TWO_PI = 2 * PI;

View view_of(const Packed& p) {
  View v;
  v.prims = p.prims.data();
  v.prim_count = p.prim_count;
  v.nodes = p.nodes.data();
  v.node_count = p.node_count;
  v.mats = p.mats.data();
  v.mat_count = p.mat_count;
  v.lights = p.lights.data();
  v.light_count = (uint32_t)p.lights.size();
  v.prim_object = p.prim_object.data();
  v.sky = p.sky;
  return v;
}

View view_of(const ct_packed_scene_view& s) {
  View v;
  v.prims = s.prims;
  v.prim_count = s.prim_count;
  v.nodes = s.nodes;
  v.node_count = s.node_count;
  v.mats = s.mats;
  v.mat_count = s.mat_count;
  v.lights = s.lights;
  v.light_count = s.light_count;
  v.prim_object = s.prim_object;
  v.sky.gradient = s.sky.kind == 1;
  v.sky.zenith = v3(s.sky.zenith[0], s.sky.zenith[1], s.sky.zenith[2]);
  v.sky.horizon = v3(s.sky.horizon[0], s.sky.horizon[1], s.sky.horizon[2]);
  v.sky.strength = s.sky.strength;
  return v;
}

// ---- intersect.ts ------------------------------------------------------------

// intersect.ts:20-39
double ray_sphere(double ox, double oy, double oz, double dx, double dy, double dz, double cx,
                  double cy, double cz, double r, double tmin, double tmax) {
  double lx = ox - cx, ly = oy - cy, lz = oz - cz;
  double a = dx * dx + dy * dy + dz * dz;
  double half_b = lx * dx + ly * dy + lz * dz;
  double c = lx * lx + ly * ly + lz * lz - r * r;
  double disc = half_b * half_b - a * c;
  if (disc < 0) return -1;
  double s = std::sqrt(disc);
  double t = (-half_b - s) / a;
  if (t <= tmin || t >= tmax) {
    t = (-half_b + s) / a;
    if (t <= tmin || t >= tmax) return -1;
  }
  return t;
}

// intersect.ts:52-85: two-sided Moller-Trumbore.
bool ray_triangle(double ox, double oy, double oz, double dx, double dy, double dz, double ax,
                  double ay, double az, double bx, double by, double bz, double cx, double cy,
                  double cz, double tmin, double tmax, double* t_out, double* u_out,
                  double* v_out) {
  double e1x = bx - ax, e1y = by - ay, e1z = bz - az;
  double e2x = cx - ax, e2y = cy - ay, e2z = cz - az;
  double px = dy * e2z - dz * e2y;
  double py = dz * e2x - dx * e2z;
  double pz = dx * e2y - dy * e2x;
  double det = e1x * px + e1y * py + e1z * pz;
  if (det > -1e-12 && det < 1e-12) return false;
  double inv_det = 1 / det;
  double tx = ox - ax, ty = oy - ay, tz = oz - az;
  double u = (tx * px + ty * py + tz * pz) * inv_det;
  if (u < 0 || u > 1) return false;
  double qx = ty * e1z - tz * e1y;
  double qy = tz * e1x - tx * e1z;
  double qz = tx * e1y - ty * e1x;
  double v = (dx * qx + dy * qy + dz * qz) * inv_det;
  if (v < 0 || u + v > 1) return false;
  double t = (e2x * qx + e2y * qy + e2z * qz) * inv_det;
  if (t <= tmin || t >= tmax) return false;
  *t_out = t;
  *u_out = u;
  *v_out = v;
  return true;
}

// intersect.ts:92-123
double ray_aabb(double ox, double oy, double oz, double idx, double idy, double idz, double minx,
                double miny, double minz, double maxx, double maxy, double maxz, double tmax) {
  double t0 = (minx - ox) * idx;
  double t1 = (maxx - ox) * idx;
  double tn = t0 < t1 ? t0 : t1;
  double tf = t0 < t1 ? t1 : t0;
  t0 = (miny - oy) * idy;
  t1 = (maxy - oy) * idy;
  if (t0 < t1) {
    if (t0 > tn) tn = t0;
    if (t1 < tf) tf = t1;
  } else {
    if (t1 > tn) tn = t1;
    if (t0 < tf) tf = t0;
  }
  t0 = (minz - oz) * idz;
  t1 = (maxz - oz) * idz;
  if (t0 < t1) {
    if (t0 > tn) tn = t0;
    if (t1 < tf) tf = t1;
  } else {
    if (t1 > tn) tn = t1;
    if (t0 < tf) tf = t0;
  }
  if (tn > tf || tf < 0 || tn > tmax) return INF;
  return tn < 0 ? 0 : tn;
}

namespace {

inline double node_aabb(const float* nodes, uint32_t node, double ox, double oy, double oz,
                        double idx, double idy, double idz, double tmax) {
  const float* n = nodes + (size_t)node * CT_NODE_STRIDE;
  return ray_aabb(ox, oy, oz, idx, idy, idz, n[0], n[1], n[2], n[4], n[5], n[6], tmax);
}

// intersect.ts:155-193 (testLeaf). `prim`, `u`, `v` persist across leaves the
// way the reference's shared leafScratch record does.
inline double test_leaf(const float* prims, double leaf, double ox, double oy, double oz,
                        double dx, double dy, double dz, double tmin, double closest,
                        int32_t* prim, double* u, double* v, Counters* c) {
  int32_t li = (int32_t)leaf;
  int32_t count = li & 7, start = li >> 3;
  for (int32_t p = start; p < start + count; p++) {
    const float* q = prims + (size_t)p * CT_PRIM_STRIDE;
    if (q[3] == CT_PRIM_SPHERE) {
      if (c) c->sphere++;
      double t = ray_sphere(ox, oy, oz, dx, dy, dz, q[0], q[1], q[2], q[4], tmin, closest);
      if (t > 0) {
        closest = t;
        *prim = p;
      }
    } else {
      if (c) c->tri++;
      double t, tu, tv;
      if (ray_triangle(ox, oy, oz, dx, dy, dz, q[0], q[1], q[2], q[4], q[5], q[6], q[8], q[9],
                       q[10], tmin, closest, &t, &tu, &tv)) {
        closest = t;
        *prim = p;
        *u = tu;
        *v = tv;
      }
    }
  }
  return closest;
}

}  // namespace

// intersect.ts:202-282: ordered front-to-back walk with a 512-entry stack.
bool intersect_closest(const View& ps, double ox, double oy, double oz, double dx, double dy,
                       double dz, double tmin, double tmax, Hit* hit, Counters* c) {
  const float* nodes = ps.nodes;
  if (ps.node_count == 0) {
    hit->t = INF;
    hit->prim = -1;
    return false;
  }
  double idx = safe_inv(dx), idy = safe_inv(dy), idz = safe_inv(dz);
  double closest = tmax;
  int32_t best = -1;
  double bu = 0, bv = 0;
  if (c) {
    c->aabb++;
    c->nodes++;
  }
  if (node_aabb(nodes, 0, ox, oy, oz, idx, idy, idz, closest) == INF) {
    hit->t = INF;
    hit->prim = -1;
    return false;
  }
  int32_t stack_node[512];
  double stack_entry[512];
  int sp = 0;
  uint32_t node = 0;
  for (;;) {
    const float* nb = nodes + (size_t)node * CT_NODE_STRIDE;
    double leaf = nb[7];
    if (leaf >= 0) {
      closest = test_leaf(ps.prims, leaf, ox, oy, oz, dx, dy, dz, tmin, closest, &best, &bu, &bv, c);
    } else {
      uint32_t left = node + 1;
      uint32_t right = (uint32_t)(int32_t)nodes[(size_t)left * CT_NODE_STRIDE + 3];
      double tl = node_aabb(nodes, left, ox, oy, oz, idx, idy, idz, closest);
      double tr = node_aabb(nodes, right, ox, oy, oz, idx, idy, idz, closest);
      if (c) c->aabb += 2;
      if (tl != INF) {
        if (tr != INF) {
          if (tl <= tr) {
            stack_node[sp] = (int32_t)right;
            stack_entry[sp++] = tr;
            node = left;
          } else {
            stack_node[sp] = (int32_t)left;
            stack_entry[sp++] = tl;
            node = right;
          }
        } else {
          node = left;
        }
        if (c) c->nodes++;
        continue;
      }
      if (tr != INF) {
        node = right;
        if (c) c->nodes++;
        continue;
      }
    }
    // pop, skipping entries the shrinking bound has already excluded
    do {
      if (sp == 0) {
        if (best < 0) {
          hit->t = INF;
          hit->prim = -1;
          return false;
        }
        hit->t = closest;
        hit->prim = best;
        hit->u = bu;
        hit->v = bv;
        return true;
      }
      sp--;
    } while (stack_entry[sp] >= closest);
    node = (uint32_t)stack_node[sp];
    if (c) c->nodes++;
  }
}

// intersect.ts:290-365: literal skip-link loop.
bool intersect_closest_stackless(const View& ps, double ox, double oy, double oz, double dx,
                                 double dy, double dz, double tmin, double tmax, Hit* hit,
                                 Counters* c) {
  double idx = safe_inv(dx), idy = safe_inv(dy), idz = safe_inv(dz);
  double closest = tmax;
  int32_t best = -1;
  double bu = 0, bv = 0;
  uint32_t node = 0;
  while (node < ps.node_count) {
    const float* nb = ps.nodes + (size_t)node * CT_NODE_STRIDE;
    if (c) {
      c->aabb++;
      c->nodes++;
    }
    double entry = ray_aabb(ox, oy, oz, idx, idy, idz, nb[0], nb[1], nb[2], nb[4], nb[5], nb[6],
                            closest);
    if (entry == INF) {
      node = (uint32_t)(int32_t)nb[3];
      continue;
    }
    double leaf = nb[7];
    if (leaf >= 0)
      closest = test_leaf(ps.prims, leaf, ox, oy, oz, dx, dy, dz, tmin, closest, &best, &bu, &bv, c);
    node++;
  }
  if (best < 0) {
    hit->t = INF;
    hit->prim = -1;
    return false;
  }
  hit->t = closest;
  hit->prim = best;
  hit->u = bu;
  hit->v = bv;
  return true;
}

// intersect.ts:368-420: stackless any-hit on (tmin, tmax).
bool occluded(const View& ps, double ox, double oy, double oz, double dx, double dy, double dz,
              double tmin, double tmax, Counters* c) {
  double idx = safe_inv(dx), idy = safe_inv(dy), idz = safe_inv(dz);
  uint32_t node = 0;
  while (node < ps.node_count) {
    const float* nb = ps.nodes + (size_t)node * CT_NODE_STRIDE;
    if (c) {
      c->aabb++;
      c->nodes++;
    }
    double entry = ray_aabb(ox, oy, oz, idx, idy, idz, nb[0], nb[1], nb[2], nb[4], nb[5], nb[6],
                            tmax);
    if (entry == INF) {
      node = (uint32_t)(int32_t)nb[3];
      continue;
    }
    double leaf = nb[7];
    if (leaf >= 0) {
      int32_t li = (int32_t)leaf;
      int32_t count = li & 7, start = li >> 3;
      for (int32_t p = start; p < start + count; p++) {
        const float* q = ps.prims + (size_t)p * CT_PRIM_STRIDE;
        if (q[3] == CT_PRIM_SPHERE) {
          if (c) c->sphere++;
          if (ray_sphere(ox, oy, oz, dx, dy, dz, q[0], q[1], q[2], q[4], tmin, tmax) > 0)
            return true;
        } else {
          if (c) c->tri++;
          double t, u, v;
          if (ray_triangle(ox, oy, oz, dx, dy, dz, q[0], q[1], q[2], q[4], q[5], q[6], q[8], q[9],
                           q[10], tmin, tmax, &t, &u, &v))
            return true;
        }
      }
    }
    node++;
  }
  return false;
}

// intersect.ts:423-468
bool intersect_brute_force(const View& ps, double ox, double oy, double oz, double dx, double dy,
                           double dz, double tmin, double tmax, Hit* hit) {
  double closest = tmax;
  int32_t best = -1;
  double bu = 0, bv = 0;
  for (uint32_t p = 0; p < ps.prim_count; p++) {
    const float* q = ps.prims + (size_t)p * CT_PRIM_STRIDE;
    if (q[3] == CT_PRIM_SPHERE) {
      double t = ray_sphere(ox, oy, oz, dx, dy, dz, q[0], q[1], q[2], q[4], tmin, closest);
      if (t > 0) {
        closest = t;
        best = (int32_t)p;
      }
    } else {
      double t, u, v;
      if (ray_triangle(ox, oy, oz, dx, dy, dz, q[0], q[1], q[2], q[4], q[5], q[6], q[8], q[9],
                       q[10], tmin, closest, &t, &u, &v)) {
        closest = t;
        best = (int32_t)p;
        bu = u;
        bv = v;
      }
    }
  }
  hit->t = best < 0 ? INF : closest;
  hit->prim = best;
  hit->u = bu;
  hit->v = bv;
  return best >= 0;
}

// ---- materials.ts ------------------------------------------------------------

// materials.ts:20-42
void basis_into(double nx, double ny, double nz, double out[6]) {
  double hx = 1, hy = 0, hz = 0;
  if (std::fabs(nx) > 0.9) {
    hx = 0;
    hy = 1;
  }
  double tx = hy * nz - hz * ny;
  double ty = hz * nx - hx * nz;
  double tz = hx * ny - hy * nx;
  double inv = 1 / std::sqrt(tx * tx + ty * ty + tz * tz);
  tx *= inv;
  ty *= inv;
  tz *= inv;
  out[0] = tx;
  out[1] = ty;
  out[2] = tz;
  out[3] = ny * tz - nz * ty;
  out[4] = nz * tx - nx * tz;
  out[5] = nx * ty - ny * tx;
}

// materials.ts:47-64
void cosine_hemisphere_into(double nx, double ny, double nz, double u1, double u2, double out[3]) {
  double r = std::sqrt(u1);
  double phi = TWO_PI * u2;
  double x = r * std::cos(phi);
  double y = r * std::sin(phi);
  double z = std::sqrt(u1 < 1 ? 1 - u1 : 0);
  double b[6];
  basis_into(nx, ny, nz, b);
  double dx = b[0] * x + b[3] * y + nx * z;
  double dy = b[1] * x + b[4] * y + ny * z;
  double dz = b[2] * x + b[5] * y + nz * z;
  double inv = 1 / std::sqrt(dx * dx + dy * dy + dz * dz);
  out[0] = dx * inv;
  out[1] = dy * inv;
  out[2] = dz * inv;
}

// materials.ts:67-74
void unit_vector_into(double u1, double u2, double out[3]) {
  double z = 1 - 2 * u1;
  double r = std::sqrt(z * z < 1 ? 1 - z * z : 0);
  double phi = TWO_PI * u2;
  out[0] = r * std::cos(phi);
  out[1] = r * std::sin(phi);
  out[2] = z;
}

// materials.ts:77-81
double schlick(double cos_theta, double eta_i, double eta_t) {
  double q = (eta_i - eta_t) / (eta_i + eta_t);
  double r0 = q * q;
  double m = 1 - std::fmax(0.0, std::fmin(1.0, cos_theta));
  return r0 + (1 - r0) * m * m * m * m * m;
}

// materials.ts:89-95
double dielectric_reflectance(double cos_i, double eta_i, double eta_t) {
  double eta = eta_i / eta_t;
  double sin2t = eta * eta * (1 - cos_i * cos_i);
  if (sin2t >= 1) return 1;
  if (eta_i > eta_t) return schlick(std::sqrt(1 - sin2t), eta_i, eta_t);
  return schlick(cos_i, eta_i, eta_t);
}

// materials.ts:102-124
void metal_into(double dx, double dy, double dz, double nx, double ny, double nz, double roughness,
                double u1, double u2, double u3, double out[3]) {
  double k = 2 * (dx * nx + dy * ny + dz * nz);
  double rx = dx - k * nx, ry = dy - k * ny, rz = dz - k * nz;
  if (roughness > 0) {
    unit_vector_into(u1, u2, out);
    double rad = std::cbrt(u3) * roughness;
    rx += out[0] * rad;
    ry += out[1] * rad;
    rz += out[2] * rad;
  }
  double inv = 1 / std::sqrt(rx * rx + ry * ry + rz * rz);
  out[0] = rx * inv;
  out[1] = ry * inv;
  out[2] = rz * inv;
}

// materials.ts:131-166
bool dielectric_into(double dx, double dy, double dz, double nx, double ny, double nz, double ior,
                     bool front_face, double u, double out[3]) {
  double eta_i = front_face ? 1 : ior;
  double eta_t = front_face ? ior : 1;
  double eta = eta_i / eta_t;
  double cos_i = -(dx * nx + dy * ny + dz * nz);
  if (cos_i > 1) cos_i = 1;
  double refl = dielectric_reflectance(cos_i, eta_i, eta_t);
  double sin2t = eta * eta * (1 - cos_i * cos_i);
  if (u < refl || sin2t > 1) {
    double k = 2 * (dx * nx + dy * ny + dz * nz);
    out[0] = dx - k * nx;
    out[1] = dy - k * ny;
    out[2] = dz - k * nz;
    return true;
  }
  double cos_t = std::sqrt(1 - sin2t);
  double s = eta * cos_i - cos_t;
  double tx = dx * eta + nx * s, ty = dy * eta + ny * s, tz = dz * eta + nz * s;
  double inv = 1 / std::sqrt(tx * tx + ty * ty + tz * tz);
  out[0] = tx * inv;
  out[1] = ty * inv;
  out[2] = tz * inv;
  return false;
}

// materials.ts:169-174
double power_heuristic(double a, double b) {
  double a2 = a * a, b2 = b * b, denom = a2 + b2;
  return denom > 0 ? a2 / denom : 0;
}

// materials.ts:177-181
bool checker_primary(double px, double py, double pz, double cells) {
  double sum = std::floor(px * cells + 0.5) + std::floor(py * cells + 0.5) +
               std::floor(pz * cells + 0.5);
  double m = std::fmod(std::fmod(sum, 2) + 2, 2);  // JS `%` is fmod
  return m == 0;
}

// ---- camera.ts -----------------------------------------------------------------

// camera.ts:25-31
V3 camera_position(const CameraSettings& cam) {
  double cp = std::cos(cam.pitch);
  return add(cam.target, scale(v3(cp * std::sin(cam.yaw), std::sin(cam.pitch),
                                  cp * std::cos(cam.yaw)),
                               cam.distance));
}

// camera.ts:33-51
Frame camera_frame(const CameraSettings& cam, double aspect) {
  V3 origin = camera_position(cam);
  V3 forward = normalize(sub(cam.target, origin));
  V3 right = cross(forward, v3(0, 1, 0));
  if (right.x * right.x + right.y * right.y + right.z * right.z < 1e-12) right = v3(1, 0, 0);
  right = normalize(right);
  V3 up = cross(right, forward);
  Frame f;
  f.origin = origin;
  f.right = right;
  f.up = up;
  f.forward = forward;
  f.tan_half_fov = std::tan((cam.fov_deg * PI) / 360);
  f.aspect = aspect;
  f.lens_radius = cam.lens_radius;
  f.focus_distance = std::fmax(1e-3, cam.focus_distance);
  return f;
}

// camera.ts:62-72
void generate_ray(const Frame& f, double sx, double sy, double lx, double ly, V3* origin, V3* dir) {
  double px = (2 * sx - 1) * f.tan_half_fov * f.aspect;
  double py = (2 * sy - 1) * f.tan_half_fov;
  V3 focus = add(f.origin, scale(add(add(scale(f.right, px), scale(f.up, py)), f.forward),
                                 f.focus_distance));
  V3 offset = add(scale(f.right, lx * f.lens_radius), scale(f.up, ly * f.lens_radius));
  *origin = add(f.origin, offset);
  *dir = normalize(sub(focus, *origin));
}

// ---- tracer.ts -----------------------------------------------------------------

// tracer.ts:61-90
double light_pdf(const View& ps, double px, double py, double pz, double hx, double hy, double hz,
                 double hnx, double hny, double hnz, int32_t prim) {
  uint32_t light_count = ps.light_count;
  if (light_count == 0) return 0;
  const float* q = ps.prims + (size_t)prim * CT_PRIM_STRIDE;
  double tx = hx - px, ty = hy - py, tz = hz - pz;
  double dist2 = tx * tx + ty * ty + tz * tz;
  if (dist2 <= 0) return 0;
  double inv = 1 / std::sqrt(dist2);
  double wx = tx * inv, wy = ty * inv, wz = tz * inv;
  if (q[3] == CT_PRIM_SPHERE) {
    double cx = q[0] - px, cy = q[1] - py, cz = q[2] - pz;
    double r = q[4];
    double d2 = cx * cx + cy * cy + cz * cz;
    if (d2 > r * r) {
      double cos_max = std::sqrt(std::fmax(0.0, 1 - (r * r) / d2));
      double solid = TWO_PI * (1 - cos_max);
      return solid > 0 ? 1 / (solid * light_count) : 0;
    }
  }
  double cos_l = std::fabs(hnx * wx + hny * wy + hnz * wz);
  if (cos_l < 1e-6) return 0;
  return dist2 / (q[11] * cos_l * light_count);
}

// tracer.ts:93-180. out: [0..2] direction, [3] distance, [4] pdf, [5..7] emission.
bool sample_light(const View& ps, double px, double py, double pz, Rng& rng, double out[8]) {
  uint32_t light_count = ps.light_count;
  if (light_count == 0) return false;
  int32_t prim = ps.lights[rng.integer((int32_t)light_count)];
  const float* q = ps.prims + (size_t)prim * CT_PRIM_STRIDE;
  const float* m = ps.mats + (size_t)ps.prim_object[prim] * CT_MAT_STRIDE;
  out[5] = m[12];
  out[6] = m[13];
  out[7] = m[14];
  if (q[3] == CT_PRIM_SPHERE) {
    double cx = q[0] - px, cy = q[1] - py, cz = q[2] - pz;
    double r = q[4];
    double d2 = cx * cx + cy * cy + cz * cz;
    if (d2 > r * r) {
      double cos_max = std::sqrt(std::fmax(0.0, 1 - (r * r) / d2));
      double cos_t = 1 - rng.next() * (1 - cos_max);
      double sin_t = std::sqrt(std::fmax(0.0, 1 - cos_t * cos_t));
      double phi = TWO_PI * rng.next();
      double inv_d = 1 / std::sqrt(d2);
      double ax = cx * inv_d, ay = cy * inv_d, az = cz * inv_d;
      double b[6];
      basis_into(ax, ay, az, b);
      double sx = sin_t * std::cos(phi), sy = sin_t * std::sin(phi);
      double wx = b[0] * sx + b[3] * sy + ax * cos_t;
      double wy = b[1] * sx + b[4] * sy + ay * cos_t;
      double wz = b[2] * sx + b[5] * sy + az * cos_t;
      double inv_w = 1 / std::sqrt(wx * wx + wy * wy + wz * wz);
      wx *= inv_w;
      wy *= inv_w;
      wz *= inv_w;
      double half_b = -(cx * wx + cy * wy + cz * wz);
      double disc = half_b * half_b - (d2 - r * r);
      if (disc < 0) return false;
      double dist = -half_b - std::sqrt(disc);
      if (dist <= 0) return false;
      out[0] = wx;
      out[1] = wy;
      out[2] = wz;
      out[3] = dist;
      out[4] = 1 / (TWO_PI * (1 - cos_max) * light_count);
      return true;
    }
    double u1 = rng.next();
    double u2 = rng.next();
    double n[3];
    unit_vector_into(u1, u2, n);
    double tx = cx + n[0] * r, ty = cy + n[1] * r, tz = cz + n[2] * r;
    double dist2 = tx * tx + ty * ty + tz * tz;
    if (dist2 <= 0) return false;
    double dist = std::sqrt(dist2);
    double wx = tx / dist, wy = ty / dist, wz = tz / dist;
    double cos_l = std::fabs(n[0] * wx + n[1] * wy + n[2] * wz);
    if (cos_l < 1e-6) return false;
    out[0] = wx;
    out[1] = wy;
    out[2] = wz;
    out[3] = dist;
    out[4] = dist2 / (q[11] * cos_l * light_count);
    return true;
  }
  double u1 = rng.next();
  double u2 = rng.next();
  if (u1 + u2 > 1) {
    u1 = 1 - u1;
    u2 = 1 - u2;
  }
  double ax = q[0], ay = q[1], az = q[2];
  double qx = ax + (q[4] - ax) * u1 + (q[8] - ax) * u2;
  double qy = ay + (q[5] - ay) * u1 + (q[9] - ay) * u2;
  double qz = az + (q[6] - az) * u1 + (q[10] - az) * u2;
  double tx = qx - px, ty = qy - py, tz = qz - pz;
  double dist2 = tx * tx + ty * ty + tz * tz;
  if (dist2 <= 0) return false;
  double dist = std::sqrt(dist2);
  double wx = tx / dist, wy = ty / dist, wz = tz / dist;
  double cos_l = std::fabs(q[12] * wx + q[13] * wy + q[14] * wz);
  if (cos_l < 1e-6) return false;
  out[0] = wx;
  out[1] = wy;
  out[2] = wz;
  out[3] = dist;
  out[4] = dist2 / (q[11] * cos_l * light_count);
  return true;
}

// tracer.ts:191-328
void radiance(const View& ps, double ox, double oy, double oz, double dx, double dy, double dz,
              Rng& rng, const TraceOptions& opts, double out[3], uint64_t* closest_rays,
              uint64_t* shadow_rays, Counters* closest_work, Counters* shadow_work) {
  double lr = 0, lg = 0, lb = 0;
  double br = 1, bg = 1, bb = 1;
  bool specular = true;
  double prev_pdf = 0;
  double prevx = ox, prevy = oy, prevz = oz;
  const float* prims = ps.prims;
  const float* mats = ps.mats;
  bool use_nee = opts.nee && ps.light_count > 0;
  const Sky& sky = ps.sky;
  double light[8];
  for (int bounce = 0; bounce <= opts.max_bounces; bounce++) {
    Hit hit;
    if (closest_rays) (*closest_rays)++;
    if (!intersect_closest(ps, ox, oy, oz, dx, dy, dz, T_MIN, INF, &hit, closest_work)) {
      if (sky.gradient) {
        double t = 0.5 * (dy + 1);
        lr += br * (sky.horizon.x + (sky.zenith.x - sky.horizon.x) * t) * sky.strength;
        lg += bg * (sky.horizon.y + (sky.zenith.y - sky.horizon.y) * t) * sky.strength;
        lb += bb * (sky.horizon.z + (sky.zenith.z - sky.horizon.z) * t) * sky.strength;
      }
      break;
    }
    int32_t prim = hit.prim;
    double t = hit.t;
    const float* q = prims + (size_t)prim * CT_PRIM_STRIDE;
    double px = ox + dx * t, py = oy + dy * t, pz = oz + dz * t;
    double nx, ny, nz;
    if (q[3] == CT_PRIM_SPHERE) {
      double inv_r = 1 / (double)q[4];
      nx = (px - q[0]) * inv_r;
      ny = (py - q[1]) * inv_r;
      nz = (pz - q[2]) * inv_r;
    } else {
      nx = q[12];
      ny = q[13];
      nz = q[14];
    }
    bool front = dx * nx + dy * ny + dz * nz < 0;
    double sx = front ? nx : -nx, sy = front ? ny : -ny, sz = front ? nz : -nz;
    const float* m = mats + (size_t)ps.prim_object[prim] * CT_MAT_STRIDE;
    double type = m[3];
    double er = m[12], eg = m[13], eb = m[14];
    if (er > 0 || eg > 0 || eb > 0) {
      double w = 1;
      if (use_nee && !specular) {
        double pl = light_pdf(ps, prevx, prevy, prevz, px, py, pz, nx, ny, nz, prim);
        w = power_heuristic(prev_pdf, pl);
      }
      lr += br * er * w;
      lg += bg * eg * w;
      lb += bb * eb * w;
    }
    if (type == CT_MAT_EMISSIVE) break;
    double ndx, ndy, ndz;
    double dir[3];
    if (type == CT_MAT_LAMBERTIAN) {
      double ar = m[0], ag = m[1], ab = m[2];
      if (m[6] > 0.5 && !checker_primary(px, py, pz, m[5])) {
        ar = m[8];
        ag = m[9];
        ab = m[10];
      }
      if (use_nee && sample_light(ps, px, py, pz, rng, light)) {
        double wx = light[0], wy = light[1], wz = light[2];
        double pdf_l = light[4];
        double cos_s = sx * wx + sy * wy + sz * wz;
        if (cos_s > 0 && pdf_l > 0) {
          if (shadow_rays) (*shadow_rays)++;
          if (!occluded(ps, px, py, pz, wx, wy, wz, T_MIN, light[3] * SHADOW_SHORTEN, shadow_work)) {
            double pdf_b = cos_s * INV_PI;
            double k = (cos_s * INV_PI * power_heuristic(pdf_l, pdf_b)) / pdf_l;
            lr += br * ar * light[5] * k;
            lg += bg * ag * light[6] * k;
            lb += bb * ab * light[7] * k;
          }
        }
      }
      double u1 = rng.next();
      double u2 = rng.next();
      cosine_hemisphere_into(sx, sy, sz, u1, u2, dir);
      ndx = dir[0];
      ndy = dir[1];
      ndz = dir[2];
      prev_pdf = std::fmax(0.0, sx * ndx + sy * ndy + sz * ndz) * INV_PI;
      br *= ar;
      bg *= ag;
      bb *= ab;
      specular = false;
    } else if (type == CT_MAT_METAL) {
      double u1 = rng.next();
      double u2 = rng.next();
      double u3 = rng.next();
      metal_into(dx, dy, dz, sx, sy, sz, m[4], u1, u2, u3, dir);
      ndx = dir[0];
      ndy = dir[1];
      ndz = dir[2];
      if (ndx * sx + ndy * sy + ndz * sz <= 0) break;
      br *= m[0];
      bg *= m[1];
      bb *= m[2];
      specular = true;
    } else {
      double u = rng.next();
      dielectric_into(dx, dy, dz, sx, sy, sz, m[4], front, u, dir);
      ndx = dir[0];
      ndy = dir[1];
      ndz = dir[2];
      br *= m[0];
      bg *= m[1];
      bb *= m[2];
      specular = true;
    }
    if (opts.russian_roulette && bounce >= 3) {
      double max_b = br > bg ? (br > bb ? br : bb) : bg > bb ? bg : bb;
      double p_survive = max_b > 1 ? 1 : max_b < 0.05 ? 0.05 : max_b;
      if (rng.next() > p_survive) break;
      br /= p_survive;
      bg /= p_survive;
      bb /= p_survive;
    }
    prevx = px;
    prevy = py;
    prevz = pz;
    ox = px;
    oy = py;
    oz = pz;
    dx = ndx;
    dy = ndy;
    dz = ndz;
  }
  out[0] = lr;
  out[1] = lg;
  out[2] = lb;
}

// tracer.ts:361-395 over rows [y0, y1).
void accumulate_pass_rows(const View& ps, const Frame& f, int width, int height,
                          uint32_t frame_index, const TraceOptions& opts, float* accum,
                          double* sumsq, int y0, int y1) {
  bool use_lens = f.lens_radius > 0;
  for (int y = y0; y < y1; y++) {
    for (int x = 0; x < width; x++) {
      uint32_t pixel = (uint32_t)(y * width + x);
      Rng rng = Rng::from_pixel(pixel, frame_index);
      double sx = (x + rng.next()) / width;
      double sy = 1 - (y + rng.next()) / height;
      double lx = 0, ly = 0;
      if (use_lens) {
        double r = std::sqrt(rng.next());
        double theta = TWO_PI * rng.next();
        lx = r * std::cos(theta);
        ly = r * std::sin(theta);
      }
      V3 o, d;
      generate_ray(f, sx, sy, lx, ly, &o, &d);
      double c[3];
      radiance(ps, o.x, o.y, o.z, d.x, d.y, d.z, rng, opts, c);
      size_t i = (size_t)pixel * 3;
      if (std::isfinite(c[0]) && std::isfinite(c[1]) && std::isfinite(c[2])) {
        accum[i] = (float)((double)accum[i] + c[0]);
        accum[i + 1] = (float)((double)accum[i + 1] + c[1]);
        accum[i + 2] = (float)((double)accum[i + 2] + c[2]);
        if (sumsq) {
          sumsq[i] += c[0] * c[0];
          sumsq[i + 1] += c[1] * c[1];
          sumsq[i + 2] += c[2] * c[2];
        }
      }
    }
  }
}

void accumulate_pass(const View& ps, const Frame& f, int width, int height, uint32_t frame_index,
                     const TraceOptions& opts, float* accum) {
  accumulate_pass_rows(ps, f, width, height, frame_index, opts, accum, nullptr, 0, height);
}

// tracer.ts:348-355. Rows are split among threads; every pixel still sums its
// passes in pass order, so the result does not depend on the thread count.
std::vector<float> render_image(const View& ps, const Frame& f, int width, int height, int spp,
                                uint32_t seed, const TraceOptions& opts, int threads,
                                double* sumsq) {
  std::vector<float> out((size_t)width * height * 3, 0.0f);
  auto work = [&](int y0, int y1) {
    for (int s = 0; s < spp; s++)
      accumulate_pass_rows(ps, f, width, height, (uint32_t)(s + seed * 7919u), opts, out.data(),
                           sumsq, y0, y1);
  };
  if (threads <= 1 || height < 2) {
    work(0, height);
  } else {
    if (threads > height) threads = height;
    std::vector<std::thread> pool;
    // Interleave row blocks so threads get similar amounts of work.
    const int block = 4;
    std::atomic_int next{0};
    auto worker = [&]() {
      for (;;) {
        int y0 = next.fetch_add(block);
        if (y0 >= height) break;
        work(y0, std::min(height, y0 + block));
      }
    };
    for (int t = 0; t < threads; t++) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
  }
  double inv = 1.0 / spp;
  for (float& v : out) v = (float)((double)v * inv);
  return out;
}

// ---- tonemap.ts / ppm.ts ---------------------------------------------------------

// tonemap.ts:7-15
double aces_fitted(double x) {
  const double a = 2.51, b = 0.03, c = 2.43, d = 0.59, e = 0.14;
  double v = (x * (a * x + b)) / (x * (c * x + d) + e);
  return v < 0 ? 0 : v > 1 ? 1 : v;
}

// tonemap.ts:18-20
double reinhard(double x) { return x <= 0 ? 0 : x / (1 + x); }

// tonemap.ts:27-31
double linear_to_srgb(double x) {
  if (x <= 0) return 0;
  if (x >= 1) return 1;
  return x <= 0.0031308 ? 12.92 * x : 1.055 * std::pow(x, 1 / 2.4) - 0.055;
}

// JS Math.round: nearest integer, halves toward +infinity.
double js_round(double x) {
  double f = std::floor(x);
  return (x - f >= 0.5) ? f + 1 : f;
}

// tonemap.ts:41-62
void tonemap_buffer(const float* accum, int width, int height, double samples, double exposure_ev,
                    bool aces, uint8_t* rgba) {
  double inv = samples > 0 ? std::pow(2.0, exposure_ev) / samples : 0;
  for (int i = 0; i < width * height; i++) {
    for (int k = 0; k < 3; k++) {
      double x = accum[(size_t)i * 3 + k] * inv;
      double mapped = aces ? aces_fitted(x) : reinhard(x);
      double v = js_round(linear_to_srgb(mapped) * 255);
      // Uint8ClampedArray store: clamp to [0, 255], NaN -> 0
      rgba[(size_t)i * 4 + k] = (uint8_t)(v >= 0 && v <= 255 ? v : v > 255 ? 255 : 0);
    }
    rgba[(size_t)i * 4 + 3] = 255;
  }
}

// ppm.ts:4-16
std::vector<uint8_t> encode_ppm(int width, int height, const uint8_t* rgba) {
  std::string header = "P6\n" + std::to_string(width) + " " + std::to_string(height) + "\n255\n";
  std::vector<uint8_t> out(header.begin(), header.end());
  out.reserve(header.size() + (size_t)width * height * 3);
  for (int i = 0; i < width * height; i++) {
    out.push_back(rgba[(size_t)i * 4]);
    out.push_back(rgba[(size_t)i * 4 + 1]);
    out.push_back(rgba[(size_t)i * 4 + 2]);
  }
  return out;
}

}  // namespace oracle
