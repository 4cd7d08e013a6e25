// Oracle (test infrastructure): C ABI over the restatement, for ctypes.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "oracle.h"
#include "oracle.hpp"

using namespace oracle;

struct or_packed {
  Packed p;
};

namespace {

Scene scene_from(const ct_object* objs, uint32_t count, const ct_sky* sky) {
  Scene s;
  s.shapes.reserve(count);
  s.materials.reserve(count);
  for (uint32_t i = 0; i < count; i++) {
    const ct_shape& cs = objs[i].shape;
    Shape sh;
    sh.kind = (ShapeKind)cs.kind;
    sh.a = v3(cs.p[0], cs.p[1], cs.p[2]);
    sh.b = v3(cs.p[3], cs.p[4], cs.p[5]);
    sh.c = v3(cs.p[6], cs.p[7], cs.p[8]);
    if (cs.kind == SHAPE_SPHERE) sh.radius = cs.p[3];
    if (cs.kind == SHAPE_MESH) {
      sh.vertices.resize(cs.vertex_count);
      for (uint32_t k = 0; k < cs.vertex_count; k++)
        sh.vertices[k] = v3(cs.vertices[3 * k], cs.vertices[3 * k + 1], cs.vertices[3 * k + 2]);
      sh.indices.assign(cs.indices, cs.indices + cs.index_count);
    }
    const ct_material& cm = objs[i].material;
    Material m;
    m.type = cm.type;
    m.color = v3(cm.color[0], cm.color[1], cm.color[2]);
    m.param = cm.param;
    m.checker = cm.has_checker != 0;
    m.color2 = v3(cm.checker_color2[0], cm.checker_color2[1], cm.checker_color2[2]);
    m.checker_scale = cm.checker_scale;
    m.has_emission = cm.has_emission != 0;
    m.emission = v3(cm.emission[0], cm.emission[1], cm.emission[2]);
    s.shapes.push_back(std::move(sh));
    s.materials.push_back(m);
  }
  if (sky) {
    s.sky.gradient = sky->kind == 1;
    s.sky.zenith = v3(sky->zenith[0], sky->zenith[1], sky->zenith[2]);
    s.sky.horizon = v3(sky->horizon[0], sky->horizon[1], sky->horizon[2]);
    s.sky.strength = sky->strength;
  }
  return s;
}

Frame frame_from(const ct_camera_frame* f) {
  Frame r;
  r.origin = v3(f->origin[0], f->origin[1], f->origin[2]);
  r.right = v3(f->right[0], f->right[1], f->right[2]);
  r.up = v3(f->up[0], f->up[1], f->up[2]);
  r.forward = v3(f->forward[0], f->forward[1], f->forward[2]);
  r.tan_half_fov = f->tan_half_fov;
  r.aspect = f->aspect;
  r.lens_radius = f->lens_radius;
  r.focus_distance = f->focus_distance;
  return r;
}

CameraSettings settings_from(const or_camera_settings* c) {
  CameraSettings s;
  s.target = v3(c->target[0], c->target[1], c->target[2]);
  s.yaw = c->yaw;
  s.pitch = c->pitch;
  s.distance = c->distance;
  s.fov_deg = c->fov_deg;
  s.lens_radius = c->lens_radius;
  s.focus_distance = c->focus_distance;
  return s;
}

// Runs fn(begin, end, counters) over [0, n) on `threads` workers.
template <class F>
void parallel_for(uint64_t n, int32_t threads, uint64_t counters[4], F fn) {
  if (threads < 1) threads = 1;
  std::vector<Counters> cs((size_t)threads);
  if (threads == 1 || n < 1024) {
    fn((uint64_t)0, n, &cs[0]);
  } else {
    std::atomic<uint64_t> next{0};
    const uint64_t chunk = 256;
    std::vector<std::thread> pool;
    for (int32_t t = 0; t < threads; t++)
      pool.emplace_back([&, t]() {
        for (;;) {
          uint64_t b = next.fetch_add(chunk);
          if (b >= n) break;
          fn(b, std::min(n, b + chunk), &cs[(size_t)t]);
        }
      });
    for (auto& th : pool) th.join();
  }
  if (counters) {
    for (int k = 0; k < 4; k++) counters[k] = 0;
    for (const Counters& c : cs) {
      counters[0] += c.aabb;
      counters[1] += c.tri;
      counters[2] += c.sphere;
      counters[3] += c.nodes;
    }
  }
}

}  // namespace

extern "C" {

uint32_t or_pcg_hash(uint32_t x) { return pcg_hash(x); }
uint32_t or_seed_for(uint32_t pixel, uint32_t frame) { return seed_for(pixel, frame); }

void or_rng_stream(uint32_t seed, uint32_t n, int32_t kind, double lo, double hi, double* out) {
  Rng r(seed);
  for (uint32_t i = 0; i < n; i++)
    out[i] = kind == 0 ? r.next() : kind == 1 ? (double)r.next_u32() : r.range(lo, hi);
}

uint32_t or_rng_stream_state(uint32_t state, uint64_t n, int32_t kind, double lo, double hi, double* out) {
  Rng r(0);
  r.state = state;
  for (uint64_t i = 0; i < n; i++)
    out[i] = kind == 0 ? r.next() : kind == 1 ? (double)r.next_u32() : r.range(lo, hi);
  return r.state;
}

or_packed* or_pack(const ct_object* objects, uint32_t count, const ct_sky* sky) {
  or_packed* h = new or_packed;
  h->p = pack_scene(scene_from(objects, count, sky));
  return h;
}

or_packed* or_pack_cornell(or_camera_settings* camera_out) {
  Scene s = cornell_box();
  or_packed* h = new or_packed;
  h->p = pack_scene(s);
  if (camera_out) {
    camera_out->target[0] = s.camera.target.x;
    camera_out->target[1] = s.camera.target.y;
    camera_out->target[2] = s.camera.target.z;
    camera_out->yaw = s.camera.yaw;
    camera_out->pitch = s.camera.pitch;
    camera_out->distance = s.camera.distance;
    camera_out->fov_deg = s.camera.fov_deg;
    camera_out->lens_radius = s.camera.lens_radius;
    camera_out->focus_distance = s.camera.focus_distance;
  }
  return h;
}

void or_packed_view(const or_packed* h, ct_packed_scene_view* v, const uint32_t** order) {
  const Packed& p = h->p;
  v->prims = p.prims.data();
  v->prim_count = p.prim_count;
  v->nodes = p.nodes.data();
  v->node_count = p.node_count;
  v->mats = p.mats.data();
  v->mat_count = p.mat_count;
  v->lights = p.lights.data();
  v->light_count = (uint32_t)p.lights.size();
  v->prim_object = p.prim_object.data();
  v->sky.kind = p.sky.gradient ? 1 : 0;
  v->sky.zenith[0] = p.sky.zenith.x;
  v->sky.zenith[1] = p.sky.zenith.y;
  v->sky.zenith[2] = p.sky.zenith.z;
  v->sky.horizon[0] = p.sky.horizon.x;
  v->sky.horizon[1] = p.sky.horizon.y;
  v->sky.horizon[2] = p.sky.horizon.z;
  v->sky.strength = p.sky.strength;
  if (order) *order = p.order.data();
}

void or_packed_free(or_packed* h) { delete h; }

void or_validate_bvh(const ct_packed_scene_view* v, const uint32_t* order, uint32_t order_len,
                     uint32_t out[5]) {
  BvhReport r = validate_bvh(v->nodes, v->node_count, order, order_len, v->prim_count);
  out[0] = r.ok;
  out[1] = r.max_leaf_size;
  out[2] = r.leaf_count;
  out[3] = r.depth;
  out[4] = r.errors;
}

void or_trace(const ct_packed_scene_view* sv, const float* rays, uint64_t count, int32_t mode,
              int32_t* prim, double* t, double* u, double* vv, uint64_t counters[4],
              int32_t threads) {
  View v = view_of(*sv);
  parallel_for(count, threads, counters, [&](uint64_t b, uint64_t e, Counters* c) {
    for (uint64_t i = b; i < e; i++) {
      const float* r = rays + i * CT_RAY_FLOATS;
      Hit h{0, -1, 0, 0};
      bool hit;
      if (mode == 0)
        hit = intersect_closest(v, r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], &h, c);
      else if (mode == 1)
        hit = intersect_closest_stackless(v, r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], &h, c);
      else
        hit = intersect_brute_force(v, r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], &h);
      prim[i] = hit ? h.prim : -1;
      if (t) t[i] = hit ? h.t : INFINITY;
      if (u) u[i] = hit ? h.u : 0;
      if (vv) vv[i] = hit ? h.v : 0;
    }
  });
}

void or_occluded(const ct_packed_scene_view* sv, const float* rays, uint64_t count,
                 uint8_t* blocked, uint64_t counters[4], int32_t threads) {
  View v = view_of(*sv);
  parallel_for(count, threads, counters, [&](uint64_t b, uint64_t e, Counters* c) {
    for (uint64_t i = b; i < e; i++) {
      const float* r = rays + i * CT_RAY_FLOATS;
      blocked[i] = occluded(v, r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], c) ? 1 : 0;
    }
  });
}

double or_prim_hit_t(const ct_packed_scene_view* sv, int32_t prim, const float* r) {
  const float* q = sv->prims + (size_t)prim * CT_PRIM_STRIDE;
  if (q[3] == CT_PRIM_SPHERE)
    return ray_sphere(r[0], r[1], r[2], r[3], r[4], r[5], q[0], q[1], q[2], q[4], r[6], r[7]);
  double t, u, v;
  if (ray_triangle(r[0], r[1], r[2], r[3], r[4], r[5], q[0], q[1], q[2], q[4], q[5], q[6], q[8],
                   q[9], q[10], r[6], r[7], &t, &u, &v))
    return t;
  return -1;
}

void or_camera_frame(const or_camera_settings* cam, double aspect, ct_camera_frame* out) {
  Frame f = camera_frame(settings_from(cam), aspect);
  const V3* src[4] = {&f.origin, &f.right, &f.up, &f.forward};
  double* dst[4] = {out->origin, out->right, out->up, out->forward};
  for (int k = 0; k < 4; k++) {
    dst[k][0] = src[k]->x;
    dst[k][1] = src[k]->y;
    dst[k][2] = src[k]->z;
  }
  out->tan_half_fov = f.tan_half_fov;
  out->aspect = f.aspect;
  out->lens_radius = f.lens_radius;
  out->focus_distance = f.focus_distance;
}

void or_generate_ray(const ct_camera_frame* f, double sx, double sy, double lx, double ly,
                     double out[6]) {
  V3 o, d;
  generate_ray(frame_from(f), sx, sy, lx, ly, &o, &d);
  out[0] = o.x;
  out[1] = o.y;
  out[2] = o.z;
  out[3] = d.x;
  out[4] = d.y;
  out[5] = d.z;
}

void or_render_image(const ct_packed_scene_view* sv, const ct_camera_frame* f,
                     const ct_render_options* o, int32_t threads, float* out, double* sumsq) {
  TraceOptions opts;
  opts.max_bounces = o->max_bounces;
  opts.russian_roulette = o->russian_roulette != 0;
  opts.nee = o->nee != 0;
  std::vector<float> img = render_image(view_of(*sv), frame_from(f), o->width, o->height, o->spp,
                                        o->seed, opts, threads, sumsq);
  std::copy(img.begin(), img.end(), out);
}

void or_accumulate_pass(const ct_packed_scene_view* sv, const ct_camera_frame* f, int32_t width,
                        int32_t height, uint32_t frame_index, const ct_trace_options* o,
                        float* accum, int32_t threads) {
  TraceOptions opts;
  opts.max_bounces = o->max_bounces;
  opts.russian_roulette = o->russian_roulette != 0;
  opts.nee = o->nee != 0;
  View v = view_of(*sv);
  Frame fr = frame_from(f);
  if (threads <= 1) {
    accumulate_pass_rows(v, fr, width, height, frame_index, opts, accum, nullptr, 0, height);
    return;
  }
  std::atomic_int next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++)
    pool.emplace_back([&]() {
      for (;;) {
        int y0 = next.fetch_add(4);
        if (y0 >= height) break;
        accumulate_pass_rows(v, fr, width, height, frame_index, opts, accum, nullptr, y0,
                             std::min(height, y0 + 4));
      }
    });
  for (auto& th : pool) th.join();
}

void or_pixel_radiance(const ct_packed_scene_view* sv, const ct_camera_frame* f, int32_t width,
                       int32_t height, uint32_t pixel, uint32_t frame_index,
                       const ct_trace_options* o, double out[3], uint64_t rays_out[10]) {
  TraceOptions opts;
  opts.max_bounces = o->max_bounces;
  opts.russian_roulette = o->russian_roulette != 0;
  opts.nee = o->nee != 0;
  Frame fr = frame_from(f);
  View v = view_of(*sv);
  int x = (int)(pixel % (uint32_t)width), y = (int)(pixel / (uint32_t)width);
  Rng rng = Rng::from_pixel(pixel, frame_index);
  double sx = (x + rng.next()) / width;
  double sy = 1 - (y + rng.next()) / height;
  double lx = 0, ly = 0;
  if (fr.lens_radius > 0) {
    double r = std::sqrt(rng.next());
    double theta = TWO_PI * rng.next();
    lx = r * std::cos(theta);
    ly = r * std::sin(theta);
  }
  V3 ro, rd;
  generate_ray(fr, sx, sy, lx, ly, &ro, &rd);
  uint64_t cr = 0, sr = 0;
  Counters cw, sw;
  radiance(v, ro.x, ro.y, ro.z, rd.x, rd.y, rd.z, rng, opts, out, &cr, &sr, &cw, &sw);
  if (rays_out) {
    const uint64_t vals[10] = {cr, sr, cw.aabb, cw.tri, cw.sphere, cw.nodes, sw.aabb, sw.tri, sw.sphere, sw.nodes};
    for (int k = 0; k < 10; k++) rays_out[k] = vals[k];
  }
}

void or_cornell_reference(int32_t width, int32_t height, int32_t spp, int32_t threads,
                          float* linear, uint8_t* rgba) {
  Scene s = cornell_box();
  Packed p = pack_scene(s);
  Frame f = camera_frame(s.camera, (double)width / (double)height);
  TraceOptions opts;  // maxBounces 8, RR on, NEE on (reference.ts:31-39)
  std::vector<float> img = render_image(view_of(p), f, width, height, spp, 1, opts, threads);
  std::copy(img.begin(), img.end(), linear);
  tonemap_buffer(img.data(), width, height, 1, 0, true, rgba);
}

void or_tonemap(const float* accum, int32_t width, int32_t height, double samples, double ev,
                int32_t aces, uint8_t* rgba) {
  tonemap_buffer(accum, width, height, samples, ev, aces != 0, rgba);
}

double or_scalar(int32_t fn, double a, double b, double c) {
  switch (fn) {
    case 0: return aces_fitted(a);
    case 1: return reinhard(a);
    case 2: return linear_to_srgb(a);
    case 3: return schlick(a, b, c);
    case 4: return dielectric_reflectance(a, b, c);
    case 5: return power_heuristic(a, b);
    case 6: return js_round(a);
    default: return NAN;
  }
}

// fn 0 cosine hemisphere (n3,u1,u2), 1 unit vector (u1,u2), 2 metal (d3,n3,rough,u1,u2,u3),
// 3 dielectric (d3,n3,ior,front,u -> out3 + reflected flag), 4 basis (n3 -> 6),
// 5 checker (p3, cells -> out[0] = primary ? 1 : 0).
void or_vector(int32_t fn, const double* in, double* out) {
  switch (fn) {
    case 0: cosine_hemisphere_into(in[0], in[1], in[2], in[3], in[4], out); break;
    case 1: unit_vector_into(in[0], in[1], out); break;
    case 2: metal_into(in[0], in[1], in[2], in[3], in[4], in[5], in[6], in[7], in[8], in[9], out); break;
    case 3:
      out[3] = dielectric_into(in[0], in[1], in[2], in[3], in[4], in[5], in[6], in[7] != 0, in[8], out) ? 1 : 0;
      break;
    case 4: basis_into(in[0], in[1], in[2], out); break;
    case 5: out[0] = checker_primary(in[0], in[1], in[2], in[3]) ? 1 : 0; break;
    default: break;
  }
}

}  // extern "C"
