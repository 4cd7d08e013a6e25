// Device-side path-tracing helpers in float32 (tracer.ts, materials.ts,
// camera.ts, rng.ts of the reference). Random numbers are drawn in the
// reference's order so every path consumes the same uint32 stream.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "traverse.cuh"

namespace ctk {

constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kTMin = 1e-4f;                 // intersect.ts:14
constexpr float kShadowShorten = 1.0f - 1e-3f; // tracer.ts:36

// ---- rng.ts -------------------------------------------------------------------
__device__ __forceinline__ uint32_t pcg_hash(uint32_t x) {
  const uint32_t state = x * 747796405u + 2891336453u;
  const uint32_t word = ((state >> ((state >> 28) + 4u)) ^ state) * 277803737u;
  return (word >> 22) ^ word;
}

__device__ __forceinline__ uint32_t seed_for(uint32_t pixel, uint32_t frame) {
  const uint32_t a = pcg_hash(pixel);
  const uint32_t b = pcg_hash(frame ^ 0x9e3779b9u);
  const uint32_t s = pcg_hash(a ^ (b * 0x85ebca6bu));
  return s == 0 ? 0x1234567u : s;
}

__device__ __forceinline__ uint32_t next_u32(uint32_t& s) {
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  return s;
}

// next() = u32 / 2^32, truncated to 24 bits so the float stays below 1.
__device__ __forceinline__ float next_f(uint32_t& s) { return (float)(next_u32(s) >> 8) * 5.9604645e-8f; }

// int(n) = min(n-1, floor(next()*n)) exactly, in integers.
__device__ __forceinline__ uint32_t next_int(uint32_t& s, uint32_t n) {
  const uint32_t r = (uint32_t)(((uint64_t)next_u32(s) * n) >> 32);
  return r < n - 1 ? r : n - 1;
}

// ---- small vector helpers --------------------------------------------------------
struct V3f {
  float x, y, z;
};
__device__ __forceinline__ V3f mk(float x, float y, float z) { return V3f{x, y, z}; }
// Fused forms are written out (device code is compiled with -fmad=false).
__device__ __forceinline__ float dot3(V3f a, V3f b) { return __fmaf_rn(a.x, b.x, __fmaf_rn(a.y, b.y, a.z * b.z)); }
// a + b * s per component
__device__ __forceinline__ V3f madd3(V3f a, V3f b, float s) {
  return mk(__fmaf_rn(b.x, s, a.x), __fmaf_rn(b.y, s, a.y), __fmaf_rn(b.z, s, a.z));
}
__device__ __forceinline__ V3f normalize3(V3f a) {
  const float l2 = dot3(a, a);
  const float inv = l2 > 0.0f ? rsqrtf(l2) : 0.0f;
  return mk(a.x * inv, a.y * inv, a.z * inv);
}

// ---- materials.ts --------------------------------------------------------------
// basisInto (materials.ts:20-42): t = normalize(h x n), b = n x t.
__device__ __forceinline__ void basis(V3f n, V3f& t, V3f& b) {
  const float hx = fabsf(n.x) > 0.9f ? 0.0f : 1.0f, hy = 1.0f - hx;
  V3f tt = mk(hy * n.z, -hx * n.z, hx * n.y - hy * n.x);
  tt = normalize3(tt);
  t = tt;
  b = mk(n.y * tt.z - n.z * tt.y, n.z * tt.x - n.x * tt.z, n.x * tt.y - n.y * tt.x);
}

// sin and cos of the angle 2 pi u through __sincosf, evaluated at 2 pi u - pi
// (inside [-pi, pi], where its documented absolute error is 2^-21.41) and
// negated back.
__device__ __forceinline__ void sincos_turn(float u, float& s, float& c) {
  __sincosf(6.28318530718f * u - 3.14159265359f, &s, &c);
  s = -s;
  c = -c;
}

// cosineHemisphereInto (materials.ts:47-64)
__device__ __forceinline__ V3f cosine_hemisphere(V3f n, float u1, float u2) {
  const float r = sqrtf(u1);
  float sp, cp;
  sincos_turn(u2, sp, cp);
  const float x = r * cp, y = r * sp;
  const float z = sqrtf(u1 < 1.0f ? 1.0f - u1 : 0.0f);
  V3f t, b;
  basis(n, t, b);
  return normalize3(madd3(madd3(mk(n.x * z, n.y * z, n.z * z), b, y), t, x));
}

// unitVectorInto (materials.ts:67-74)
__device__ __forceinline__ V3f unit_vector(float u1, float u2) {
  const float z = 1.0f - 2.0f * u1;
  const float r = sqrtf(z * z < 1.0f ? 1.0f - z * z : 0.0f);
  float sp, cp;
  sincos_turn(u2, sp, cp);
  return mk(r * cp, r * sp, z);
}

// Divisions in the shading code use __fdividef (a reciprocal and a multiply,
// within 2 ulp for the ranges met here): the integrator's parity is
// statistical, and every kernel that shades inlines the same code, so batch,
// single-scene and whole-path renders stay bit-identical to each other
// (Cornell 512^2: 2,188 -> 2,243 Msamples/s). Sampled directions take their
// angle through sincos_turn: 2,275.
// The square roots stay IEEE (x * rsqrtf(x) measured slower).

// schlick / dielectricReflectance (materials.ts:77-95)
__device__ __forceinline__ float schlick(float cos_t, float eta_i, float eta_t) {
  const float q = __fdividef(eta_i - eta_t, eta_i + eta_t);
  const float r0 = q * q;
  const float m = 1.0f - fmaxf(0.0f, fminf(1.0f, cos_t));
  const float m2 = m * m;
  return r0 + (1.0f - r0) * m2 * m2 * m;
}

__device__ __forceinline__ float dielectric_reflectance(float cos_i, float eta_i, float eta_t) {
  const float eta = __fdividef(eta_i, eta_t);
  const float sin2t = eta * eta * (1.0f - cos_i * cos_i);
  if (sin2t >= 1.0f) return 1.0f;
  if (eta_i > eta_t) return schlick(sqrtf(1.0f - sin2t), eta_i, eta_t);
  return schlick(cos_i, eta_i, eta_t);
}

// metalInto (materials.ts:102-124)
__device__ __forceinline__ V3f metal_dir(V3f d, V3f n, float rough, float u1, float u2, float u3) {
  const float k = 2.0f * dot3(d, n);
  V3f r = madd3(d, n, -k);
  if (rough > 0.0f) {
    const V3f u = unit_vector(u1, u2);
    const float rad = cbrtf(u3) * rough;
    r = madd3(r, u, rad);
  }
  return normalize3(r);
}

// dielectricInto (materials.ts:131-166)
__device__ __forceinline__ V3f dielectric_dir(V3f d, V3f n, float ior, bool front, float u) {
  const float eta_i = front ? 1.0f : ior, eta_t = front ? ior : 1.0f;
  const float eta = __fdividef(eta_i, eta_t);
  float cos_i = -dot3(d, n);
  if (cos_i > 1.0f) cos_i = 1.0f;
  const float refl = dielectric_reflectance(cos_i, eta_i, eta_t);
  const float sin2t = eta * eta * (1.0f - cos_i * cos_i);
  if (u < refl || sin2t > 1.0f) {
    const float k = 2.0f * dot3(d, n);
    return madd3(d, n, -k);
  }
  const float cos_t = sqrtf(1.0f - sin2t);
  const float s = eta * cos_i - cos_t;
  return normalize3(madd3(mk(d.x * eta, d.y * eta, d.z * eta), n, s));
}

// powerHeuristic (materials.ts:169-174)
__device__ __forceinline__ float power_heuristic(float a, float b) {
  const float a2 = a * a, denom = a2 + b * b;
  return denom > 0.0f ? __fdividef(a2, denom) : 0.0f;
}

// checkerPrimary (materials.ts:177-181)
__device__ __forceinline__ bool checker_primary(V3f p, float cells) {
  const int sum = (int)floorf(p.x * cells + 0.5f) + (int)floorf(p.y * cells + 0.5f) + (int)floorf(p.z * cells + 0.5f);
  return (sum & 1) == 0;
}

// ---- tracer.ts light sampling ---------------------------------------------------
// lightPdfScalar (tracer.ts:61-90)
__device__ __forceinline__ float light_pdf(const SceneDev& s, V3f p, V3f h, V3f hn, int32_t prim) {
  const float lc = (float)s.light_count;
  const float4* q = s.prims + (size_t)prim * 4;
  const V3f t = mk(h.x - p.x, h.y - p.y, h.z - p.z);
  const float dist2 = dot3(t, t);
  if (!(dist2 > 0.0f)) return 0.0f;
  const float inv = rsqrtf(dist2);
  const V3f w = mk(t.x * inv, t.y * inv, t.z * inv);
  const float4 a4 = __ldg(q);
  if (a4.w == 0.0f) {
    const float r = __ldg(q + 1).x;
    const V3f c = mk(a4.x - p.x, a4.y - p.y, a4.z - p.z);
    const float d2 = dot3(c, c);
    if (d2 > r * r) {
      const float cos_max = sqrtf(fmaxf(0.0f, 1.0f - (r * r) / d2));
      const float solid = 6.283185307179586f * (1.0f - cos_max);
      return solid > 0.0f ? 1.0f / (solid * lc) : 0.0f;
    }
  }
  const float cos_l = fabsf(dot3(hn, w));
  if (cos_l < 1e-6f) return 0.0f;
  return __fdividef(dist2, __ldg(q + 2).w * cos_l * lc);
}

struct LightSample {
  V3f dir;
  float dist, pdf;
  V3f emission;
};

// sampleLightInto (tracer.ts:93-180); consumes 1 + 2 random numbers.
__device__ __forceinline__ bool sample_light(const SceneDev& s, V3f p, uint32_t& rng, LightSample& out) {
  const int32_t prim = __ldg(s.lights + next_int(rng, s.light_count));
  const float lc = (float)s.light_count;
  const float4* q = s.prims + (size_t)prim * 4;
  const float4 m3 = __ldg(s.mats + (size_t)__ldg(s.prim_object + prim) * 4 + 3);
  out.emission = mk(m3.x, m3.y, m3.z);
  const float4 a4 = __ldg(q);
  if (a4.w == 0.0f) {
    const V3f c = mk(a4.x - p.x, a4.y - p.y, a4.z - p.z);
    const float r = __ldg(q + 1).x;
    const float d2 = dot3(c, c);
    if (d2 > r * r) {  // outside: cone of directions subtended by the sphere
      const float cos_max = sqrtf(fmaxf(0.0f, 1.0f - (r * r) / d2));
      const float u1 = next_f(rng);
      const float u2 = next_f(rng);
      const float cos_t = 1.0f - u1 * (1.0f - cos_max);
      const float sin_t = sqrtf(fmaxf(0.0f, 1.0f - cos_t * cos_t));
      float sp, cp;
      sincos_turn(u2, sp, cp);
      const float inv_d = rsqrtf(d2);
      const V3f ax = mk(c.x * inv_d, c.y * inv_d, c.z * inv_d);
      V3f t, b;
      basis(ax, t, b);
      const float sx = sin_t * cp, sy = sin_t * sp;
      const V3f w = normalize3(mk(t.x * sx + b.x * sy + ax.x * cos_t, t.y * sx + b.y * sy + ax.y * cos_t,
                                  t.z * sx + b.z * sy + ax.z * cos_t));
      const float half_b = -dot3(c, w);
      const float disc = half_b * half_b - (d2 - r * r);
      if (disc < 0.0f) return false;
      const float dist = -half_b - sqrtf(disc);
      if (dist <= 0.0f) return false;
      out.dir = w;
      out.dist = dist;
      out.pdf = 1.0f / (6.283185307179586f * (1.0f - cos_max) * lc);
      return true;
    }
    const float u1 = next_f(rng);
    const float u2 = next_f(rng);
    const V3f n = unit_vector(u1, u2);
    const V3f t = mk(c.x + n.x * r, c.y + n.y * r, c.z + n.z * r);
    const float dist2 = dot3(t, t);
    if (!(dist2 > 0.0f)) return false;
    const float dist = sqrtf(dist2);
    const float inv_dist = __fdividef(1.0f, dist);
    const V3f w = mk(t.x * inv_dist, t.y * inv_dist, t.z * inv_dist);
    const float cos_l = fabsf(dot3(n, w));
    if (cos_l < 1e-6f) return false;
    out.dir = w;
    out.dist = dist;
    out.pdf = __fdividef(dist2, __ldg(q + 2).w * cos_l * lc);
    return true;
  }
  float u1 = next_f(rng);
  float u2 = next_f(rng);
  if (u1 + u2 > 1.0f) {
    u1 = 1.0f - u1;
    u2 = 1.0f - u2;
  }
  const float4 b4 = __ldg(q + 1), c4 = __ldg(q + 2), n4 = __ldg(q + 3);
  const V3f qp = mk(a4.x + (b4.x - a4.x) * u1 + (c4.x - a4.x) * u2, a4.y + (b4.y - a4.y) * u1 + (c4.y - a4.y) * u2,
                    a4.z + (b4.z - a4.z) * u1 + (c4.z - a4.z) * u2);
  const V3f t = mk(qp.x - p.x, qp.y - p.y, qp.z - p.z);
  const float dist2 = dot3(t, t);
  if (!(dist2 > 0.0f)) return false;
  const float dist = sqrtf(dist2);
  const float inv_dist = __fdividef(1.0f, dist);
    const V3f w = mk(t.x * inv_dist, t.y * inv_dist, t.z * inv_dist);
  const float cos_l = fabsf(n4.x * w.x + n4.y * w.y + n4.z * w.z);
  if (cos_l < 1e-6f) return false;
  out.dir = w;
  out.dist = dist;
  out.pdf = __fdividef(dist2, c4.w * cos_l * lc);
  return true;
}

// ---- camera.ts ------------------------------------------------------------------
struct FrameF {
  float ox, oy, oz, rx, ry, rz, ux, uy, uz, fx, fy, fz;
  float tan_half_fov, aspect, lens_radius, focus_distance;
};

// generateRay (camera.ts:62-72)
__device__ __forceinline__ void camera_ray(const FrameF& f, float sx, float sy, float lx, float ly, V3f& o, V3f& d) {
  const float px = (2.0f * sx - 1.0f) * f.tan_half_fov * f.aspect;
  const float py = (2.0f * sy - 1.0f) * f.tan_half_fov;
  const V3f focus = mk(f.ox + ((f.rx * px + f.ux * py) + f.fx) * f.focus_distance,
                       f.oy + ((f.ry * px + f.uy * py) + f.fy) * f.focus_distance,
                       f.oz + ((f.rz * px + f.uz * py) + f.fz) * f.focus_distance);
  const float a = lx * f.lens_radius, b = ly * f.lens_radius;
  o = mk(f.ox + (f.rx * a + f.ux * b), f.oy + (f.ry * a + f.uy * b), f.oz + (f.rz * a + f.uz * b));
  d = normalize3(mk(focus.x - o.x, focus.y - o.y, focus.z - o.z));
}

}  // namespace ctk
