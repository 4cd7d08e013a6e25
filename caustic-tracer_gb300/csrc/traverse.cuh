// Device-side ray queries over the packed scene (sm_103a).
//
// Geometry tests follow intersect.ts of the reference: raySphere (:20-39),
// two-sided Moller-Trumbore rayTriangle (:52-85) and the slab test rayAabb
// (:92-123). The reference evaluates them in float64; here each primitive test
// runs in float32 together with a running error bound. Every accept/reject
// decision (|det| >= 1e-12, 0 <= u <= 1, v >= 0, u + v <= 1, tmin < t < tmax,
// disc >= 0) is taken in float32 only when the value is further from the
// threshold than twice its first-order error bound; otherwise the test is
// re-run in float64 with the reference's operation order and no FMA
// contraction, which reproduces the reference's decision exactly. The
// reported t then has a relative error below kTRel (else float64 too), so
// two candidates can only swap order when their distances tie within 8e-6.
//
// Box tests are float32 slab tests widened by 1+2*gamma(3) (Ize, "Robust BVH
// Ray Traversal", JCGT 2013), so no box the float64 test enters is skipped.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace ctk {

constexpr int kStackSize = 64;               // ordered-walk stack (the tree's need is computed on upload)
constexpr float kEps = 5.9604645e-8f;        // 2^-24
constexpr float kErrK = 16.0f * kEps;        // error-bound multiplier (2x the first-order bound)
// Max relative error of a reported float32 t, checked against the first-order
// bound (half of the kErrK bound): two hits swap order only within 8e-6.
constexpr float kTRel = 4e-6f;
constexpr float kBoxWiden = 1.0000005f;      // 1 + 2*gamma(3), rounded up

// Device view of a scene. `quads` holds the reference BVH collapsed to four
// children per record (64 bytes): the children's lo.x, hi.x, lo.y, hi.y,
// lo.z, hi.z as half floats rounded outwards (NaN for an empty slot), then
// the four child references (>= 0 record, < 0 ~leafword).
struct SceneDev {
  const float4* __restrict__ prims;  // 4 per primitive (pack.ts:6-10)
  const float4* __restrict__ nodes;  // 2 per reference node (bvh.ts:6-15)
  const uint4* __restrict__ quads;   // 4 per 4-wide record
  const float4* __restrict__ planes; // 3 per primitive: plane records of the float32 tests
  const float4* __restrict__ tris;   // 3 per primitive: the first 48 bytes of prims (exact tests)
  const float4* __restrict__ mats;   // 4 per material (pack.ts:12-16)
  const int32_t* __restrict__ lights;
  const uint32_t* __restrict__ prim_object;
  uint32_t prim_count;
  uint32_t node_count;
  uint32_t light_count;
  int32_t root_ref;
  float root_lo[3], root_hi[3];
};

// 16-byte aligned: where a ray sits in local memory (the exact walk's
// WalkFrame), its fields load as 16-byte vectors.
struct alignas(16) RayF {
  float ox, oy, oz, dx, dy, dz, tmin, tmax;
  float ix, iy, iz;  // safe inverse direction (intersect.ts:142)
};

__device__ __forceinline__ float safe_inv(float d) {
  // The reference maps d == 0 to 1/1e-20; |d| below 1e-20 is clamped the same
  // way so the float32 inverse stays finite.
  return fabsf(d) < 1e-20f ? (d < 0.0f ? -1e20f : 1e20f) : 1.0f / d;
}

__device__ __forceinline__ void finish_ray(RayF& r) {
  r.ix = safe_inv(r.dx);
  r.iy = safe_inv(r.dy);
  r.iz = safe_inv(r.dz);
}

// ---- float64 path in the reference's exact operation order ---------------
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// intersect.ts:52-85 in float64 (inputs are the float32 values, widened).
static __device__ __noinline__ bool tri_exact(const RayF& r, float4 a4, float4 b4, float4 c4,
                                       double tmin, double tmax, double* t_out, double* u_out,
                                       double* v_out) {
  const double ox = r.ox, oy = r.oy, oz = r.oz, dx = r.dx, dy = r.dy, dz = r.dz;
  const double ax = a4.x, ay = a4.y, az = a4.z;
  const double e1x = ds(b4.x, ax), e1y = ds(b4.y, ay), e1z = ds(b4.z, az);
  const double e2x = ds(c4.x, ax), e2y = ds(c4.y, ay), e2z = ds(c4.z, az);
  const double px = ds(dm(dy, e2z), dm(dz, e2y));
  const double py = ds(dm(dz, e2x), dm(dx, e2z));
  const double pz = ds(dm(dx, e2y), dm(dy, e2x));
  const double det = da(da(dm(e1x, px), dm(e1y, py)), dm(e1z, pz));
  if (det > -1e-12 && det < 1e-12) return false;
  const double inv_det = __drcp_rn(det);
  const double tx = ds(ox, ax), ty = ds(oy, ay), tz = ds(oz, az);
  const double u = dm(da(da(dm(tx, px), dm(ty, py)), dm(tz, pz)), inv_det);
  if (u < 0 || u > 1) return false;
  const double qx = ds(dm(ty, e1z), dm(tz, e1y));
  const double qy = ds(dm(tz, e1x), dm(tx, e1z));
  const double qz = ds(dm(tx, e1y), dm(ty, e1x));
  const double v = dm(da(da(dm(dx, qx), dm(dy, qy)), dm(dz, qz)), inv_det);
  if (v < 0 || da(u, v) > 1) return false;
  const double t = dm(da(da(dm(e2x, qx), dm(e2y, qy)), dm(e2z, qz)), inv_det);
  if (t <= tmin || t >= tmax) return false;
  *t_out = t;
  *u_out = u;
  *v_out = v;
  return true;
}

// intersect.ts:20-39 in float64. Returns t or -1.
static __device__ __noinline__ double sphere_exact(const RayF& r, float4 c4, float rad, double tmin,
                                            double tmax) {
  const double lx = ds(r.ox, c4.x), ly = ds(r.oy, c4.y), lz = ds(r.oz, c4.z);
  const double dx = r.dx, dy = r.dy, dz = r.dz, rr = rad;
  const double a = da(da(dm(dx, dx), dm(dy, dy)), dm(dz, dz));
  const double hb = da(da(dm(lx, dx), dm(ly, dy)), dm(lz, dz));
  const double c = ds(da(da(dm(lx, lx), dm(ly, ly)), dm(lz, lz)), dm(rr, rr));
  const double disc = ds(dm(hb, hb), dm(a, c));
  if (disc < 0) return -1;
  const double s = __dsqrt_rn(disc);
  double t = __ddiv_rn(ds(-hb, s), a);
  if (t <= tmin || t >= tmax) {
    t = __ddiv_rn(da(-hb, s), a);
    if (t <= tmin || t >= tmax) return -1;
  }
  return t;
}

// ---- float32 candidate tests with exact fallback ------------------------------
//
// A candidate is a primitive the ray hits inside its own (tmin, tmax). The
// tests below classify in float32 when every decision is certain and return
// t with a rigorous error bound `e`; otherwise they run the reference's
// float64 test and return its t (e = the float32 rounding of that t).
// Ordering candidates against the current closest hit happens in test_leaf.

struct Cand {
  float t, e, u, v;
};

__device__ __forceinline__ float rounding_err(float t) { return fabsf(t) * kEps; }

// intersect.ts:52-85. Returns true for a candidate.
__device__ __forceinline__ bool tri_candidate(const RayF& r, float4 a4, float4 b4, float4 c4, Cand& c,
                                              uint32_t& fallbacks) {
  const float e1x = b4.x - a4.x, e1y = b4.y - a4.y, e1z = b4.z - a4.z;
  const float e2x = c4.x - a4.x, e2y = c4.y - a4.y, e2z = c4.z - a4.z;
  const float px = r.dy * e2z - r.dz * e2y;
  const float py = r.dz * e2x - r.dx * e2z;
  const float pz = r.dx * e2y - r.dy * e2x;
  const float det = e1x * px + e1y * py + e1z * pz;
  const float tx = r.ox - a4.x, ty = r.oy - a4.y, tz = r.oz - a4.z;
  const float un = tx * px + ty * py + tz * pz;
  // Magnitude sums bounding the rounding error of p, det and un.
  const float pax = fabsf(r.dy * e2z) + fabsf(r.dz * e2y);
  const float pay = fabsf(r.dz * e2x) + fabsf(r.dx * e2z);
  const float paz = fabsf(r.dx * e2y) + fabsf(r.dy * e2x);
  const float ed = kErrK * (fabsf(e1x) * pax + fabsf(e1y) * pay + fabsf(e1z) * paz);
  const float eu = kErrK * (fabsf(tx) * pax + fabsf(ty) * pay + fabsf(tz) * paz);
  const float ad = fabsf(det);
  bool exact = false;
  if (ad - ed <= 1e-12f) {
    if (ad + ed < 1e-12f) return false;  // |det| < 1e-12 for certain
    exact = true;
  }
  if (!exact) {
    const float sg = det < 0.0f ? -1.0f : 1.0f;
    const float su = sg * un;
    if (su < -eu || su - ad > eu + ed) return false;  // u < 0 or u > 1 for certain
    if (fabsf(su) <= eu || fabsf(su - ad) <= eu + ed) {
      exact = true;
    } else {
      const float qx = ty * e1z - tz * e1y;
      const float qy = tz * e1x - tx * e1z;
      const float qz = tx * e1y - ty * e1x;
      const float qax = fabsf(ty * e1z) + fabsf(tz * e1y);
      const float qay = fabsf(tz * e1x) + fabsf(tx * e1z);
      const float qaz = fabsf(tx * e1y) + fabsf(ty * e1x);
      const float sv = sg * (r.dx * qx + r.dy * qy + r.dz * qz);
      const float ev = kErrK * (fabsf(r.dx) * qax + fabsf(r.dy) * qay + fabsf(r.dz) * qaz);
      const float euv = eu + ev + ed;
      if (sv < -ev || su + sv - ad > euv) return false;  // v < 0 or u + v > 1
      if (fabsf(sv) <= ev || fabsf(su + sv - ad) <= euv) {
        exact = true;
      } else {
        const float st = sg * (e2x * qx + e2y * qy + e2z * qz);
        const float et = kErrK * (fabsf(e2x) * qax + fabsf(e2y) * qay + fabsf(e2z) * qaz);
        const float mlo = et + r.tmin * ed;
        const float dlo = st - r.tmin * ad;  // (t - tmin) * |det|
        if (dlo < -mlo) return false;         // t <= tmin
        if (fabsf(dlo) <= mlo) exact = true;
        if (!exact && r.tmax < INFINITY) {
          const float mhi = et + r.tmax * ed;
          const float dhi = st - r.tmax * ad;  // (t - tmax) * |det|
          if (dhi > mhi) return false;          // t >= tmax
          if (fabsf(dhi) <= mhi) exact = true;
        }
        if (!exact) {
          c.t = st / ad;
          c.e = (et + c.t * ed) / ad + rounding_err(c.t);
          c.u = su / ad;
          c.v = sv / ad;
          return true;
        }
      }
    }
  }
  fallbacks++;
  double t, u, v;
  if (!tri_exact(r, a4, b4, c4, (double)r.tmin, (double)r.tmax, &t, &u, &v)) return false;
  c.t = (float)t;
  c.e = rounding_err(c.t);
  c.u = (float)u;
  c.v = (float)v;
  return true;
}

// intersect.ts:20-39: near root if inside (tmin, tmax), else the far root.
__device__ __forceinline__ bool sphere_candidate(const RayF& r, float4 c4, float rad, Cand& c,
                                                 uint32_t& fallbacks) {
  const float lx = r.ox - c4.x, ly = r.oy - c4.y, lz = r.oz - c4.z;
  const float a = r.dx * r.dx + r.dy * r.dy + r.dz * r.dz;
  const float hb = lx * r.dx + ly * r.dy + lz * r.dz;
  const float ll = lx * lx + ly * ly + lz * lz;
  const float disc = hb * hb - a * (ll - rad * rad);
  const float hba = fabsf(lx * r.dx) + fabsf(ly * r.dy) + fabsf(lz * r.dz);
  const float edisc = kErrK * (hba * hba + a * (ll + rad * rad));
  c.u = c.v = 0.0f;
  bool exact = false;
  if (disc < -edisc) return false;
  if (disc <= edisc) {
    exact = true;
  } else {
    const float s = sqrtf(disc);
    const float es = edisc / s + kEps * s;
    const float ehb = kErrK * hba;
    const float inva = 1.0f / a;
    for (int k = 0; k < 2; k++) {
      const float t = (k == 0 ? -hb - s : -hb + s) * inva;
      const float e = (ehb + es) * inva + kErrK * fabsf(t);
      if (t + e <= r.tmin || t - e >= r.tmax) continue;  // root rejected for certain
      if (t - e > r.tmin && t + e < r.tmax) {
        c.t = t;
        c.e = e + rounding_err(t);
        return true;
      }
      exact = true;
      break;
    }
    if (!exact) return false;
  }
  fallbacks++;
  const double t = sphere_exact(r, c4, rad, (double)r.tmin, (double)r.tmax);
  if (!(t > 0)) return false;
  c.t = (float)t;
  c.e = rounding_err(c.t);
  return true;
}

struct HitF {
  int32_t prim;
  float t, u, v;
  float err;  // bound on |t - reference t| for the current closest hit
};

// float64 distance of `prim` along the ray (the reference's value), or -1.
static __device__ __noinline__ double exact_t(const SceneDev& s, const RayF& r, int32_t prim) {
  const float4* q = s.tris + (size_t)prim * 3;
  const float4 a4 = __ldg(q), b4 = __ldg(q + 1);
  if (a4.w == 0.0f) return sphere_exact(r, a4, b4.x, (double)r.tmin, (double)r.tmax);
  double t, u, v;
  return tri_exact(r, a4, b4, __ldg(q + 2), (double)r.tmin, (double)r.tmax, &t, &u, &v) ? t : -1.0;
}

// The reference's distance to triangle `prim` without its barycentrics: the
// plane equation in float64 over the packed float32 vertices, equal to the
// reference's Moller-Trumbore t up to float64 rounding (~1e-15 relative), in
// about 25 float64 operations instead of about 60. Returns -1 for spheres.
static __device__ __noinline__ double plane_t64(const SceneDev& s, const RayF& r, int32_t prim) {
  const float4* q = s.tris + (size_t)prim * 3;
  const float4 a4 = __ldg(q);
  if (a4.w == 0.0f) return -1.0;
  const float4 b4 = __ldg(q + 1), c4 = __ldg(q + 2);
  const double e1x = (double)b4.x - a4.x, e1y = (double)b4.y - a4.y, e1z = (double)b4.z - a4.z;
  const double e2x = (double)c4.x - a4.x, e2y = (double)c4.y - a4.y, e2z = (double)c4.z - a4.z;
  const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  const double num = nx * ((double)a4.x - r.ox) + ny * ((double)a4.y - r.oy) + nz * ((double)a4.z - r.oz);
  const double den = nx * (double)r.dx + ny * (double)r.dy + nz * (double)r.dz;
  return num / den;
}

// Replaces a closest hit's float32 distance by the reference's float64 t
// (and barycentrics), once per ray after the walk.
static __device__ __noinline__ void refine_hit(const SceneDev& s, const RayF& r, HitF& h) {
  const float4* q = s.tris + (size_t)h.prim * 3;
  const float4 a4 = __ldg(q), b4 = __ldg(q + 1);
  if (a4.w == 0.0f) {
    const double t = sphere_exact(r, a4, b4.x, (double)r.tmin, (double)r.tmax);
    if (t > 0) h.t = (float)t;
  } else {
    double t, u, v;
    if (tri_exact(r, a4, b4, __ldg(q + 2), (double)r.tmin, (double)r.tmax, &t, &u, &v)) {
      h.t = (float)t;
      h.u = (float)u;
      h.v = (float)v;
    }
  }
  h.err = rounding_err(h.t);
}

// ---- double-float arithmetic (pairs hi + lo of floats, about 2^-44 per op) --
// Error-free transformations with explicit fused multiply-adds: two_sum (Knuth)
// and two_prod (fma), then renormalised sums and products.
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return F2{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ F2 quick_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return F2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 f2_add(F2 x, F2 y) {
  const F2 s = two_sum(x.hi, y.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ F2 f2_mul(F2 x, F2 y) {
  const float p = __fmul_rn(x.hi, y.hi);
  const float e = __fmaf_rn(x.hi, y.hi, -p);
  return quick_two_sum(p, __fadd_rn(e, __fadd_rn(__fmul_rn(x.hi, y.lo), __fmul_rn(x.lo, y.hi))));
}
__device__ __forceinline__ F2 f2_neg(F2 x) { return F2{-x.hi, -x.lo}; }
__device__ __forceinline__ F2 f2_div(F2 x, F2 y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  const F2 r = f2_add(x, f2_neg(f2_mul(F2{q1, 0.0f}, y)));
  return quick_two_sum(q1, __fdiv_rn(r.hi, y.hi));
}

// Distance to the plane of triangle `prim`, whose normal is computed here
// from the packed float32 vertices (the triangle the reference tests): with
// e1 = b - a, e2 = c - a, n = e1 x e2 and w = a - o, t = n.w / n.d. First
// in float32 with a first-order bound: the edges' and n's rounding (4 eps of
// each component's magnitude sum P), w's and the dot products' (4 and 3 eps
// of the terms' magnitudes) and the division's (eps), scaled by 1 + 1e-3 for
// the second-order terms (below 40 eps^2) and the bound's own rounding. When
// that bound exceeds `rel`, the same formula in double-float arithmetic,
// whose bound is the float32 one scaled by 2^-16 (a double-float operation
// rounds at 2^-40 or better) plus the final rounding to float32. Unlike the
// Moller-Trumbore quotient, whose error grows with distance / triangle size,
// these grow only with the angles, so they serve as the reported t of a
// closest hit whose walk bound is loose. Returns false for spheres or when
// neither bound is within `rel` (relative). It reads the compact triangle
// copy the walk has just tested, which is still in L1/L2 (1M-triangle soup:
// 1,094 against 1,086 Mrays/s reading the 64-byte records); so do the
// float64 re-checks below.
__device__ __forceinline__ bool plane_t(const SceneDev& s, const RayF& r, int32_t prim, float rel, float& t) {
  const float4* q = s.tris + (size_t)prim * 3;
  const float4 a4 = __ldg(q);
  if (a4.w == 0.0f) return false;
  const float4 b4 = __ldg(q + 1), c4 = __ldg(q + 2);
  const float e1x = b4.x - a4.x, e1y = b4.y - a4.y, e1z = b4.z - a4.z;
  const float e2x = c4.x - a4.x, e2y = c4.y - a4.y, e2z = c4.z - a4.z;
  const float nx = __fmaf_rn(e1y, e2z, -__fmul_rn(e1z, e2y));
  const float ny = __fmaf_rn(e1z, e2x, -__fmul_rn(e1x, e2z));
  const float nz = __fmaf_rn(e1x, e2y, -__fmul_rn(e1y, e2x));
  const float px = fabsf(e1y * e2z) + fabsf(e1z * e2y);
  const float py = fabsf(e1z * e2x) + fabsf(e1x * e2z);
  const float pz = fabsf(e1x * e2y) + fabsf(e1y * e2x);
  const float wx = a4.x - r.ox, wy = a4.y - r.oy, wz = a4.z - r.oz;
  const float num = __fmaf_rn(nx, wx, __fmaf_rn(ny, wy, __fmul_rn(nz, wz)));
  const float den = __fmaf_rn(nx, r.dx, __fmaf_rn(ny, r.dy, __fmul_rn(nz, r.dz)));
  const float en = 4.0f * kEps * (fabsf(wx) * px + fabsf(wy) * py + fabsf(wz) * pz) +
                   4.0f * kEps * (fabsf(nx * wx) + fabsf(ny * wy) + fabsf(nz * wz));
  const float ed = 4.0f * kEps * (fabsf(r.dx) * px + fabsf(r.dy) * py + fabsf(r.dz) * pz) +
                   3.0f * kEps * (fabsf(nx * r.dx) + fabsf(ny * r.dy) + fabsf(nz * r.dz));
  const float an = fabsf(num) - en, ad = fabsf(den) - ed;
  if (!(an > 0.0f && ad > 0.0f)) return false;
  const float bound = 1.001f * (en / an + ed / ad + kEps);
  if (bound <= rel) {
    t = num / den;
    return t > 0.0f;
  }
  if (!(bound * 0x1p-16f + 2.0f * kEps <= rel)) return false;
  // Double-float: the edge and w differences of floats are exact as pairs.
  const F2 E1x = two_sum(b4.x, -a4.x), E1y = two_sum(b4.y, -a4.y), E1z = two_sum(b4.z, -a4.z);
  const F2 E2x = two_sum(c4.x, -a4.x), E2y = two_sum(c4.y, -a4.y), E2z = two_sum(c4.z, -a4.z);
  const F2 Wx = two_sum(a4.x, -r.ox), Wy = two_sum(a4.y, -r.oy), Wz = two_sum(a4.z, -r.oz);
  const F2 Nx = f2_add(f2_mul(E1y, E2z), f2_neg(f2_mul(E1z, E2y)));
  const F2 Ny = f2_add(f2_mul(E1z, E2x), f2_neg(f2_mul(E1x, E2z)));
  const F2 Nz = f2_add(f2_mul(E1x, E2y), f2_neg(f2_mul(E1y, E2x)));
  const F2 Num = f2_add(f2_add(f2_mul(Nx, Wx), f2_mul(Ny, Wy)), f2_mul(Nz, Wz));
  const F2 Den = f2_add(f2_add(f2_mul(Nx, F2{r.dx, 0.0f}), f2_mul(Ny, F2{r.dy, 0.0f})), f2_mul(Nz, F2{r.dz, 0.0f}));
  const F2 T = f2_div(Num, Den);
  t = T.hi;
  return t > 0.0f;
}

// A reported float32 distance whose bound exceeds this (relative) is
// replaced by the reference's float64 value before it is returned; the bound
// is twice the first-order error, so a reported t is within kTRel of the
// reference's. (At 1e-6 nearly every hit took the float64 pass: 2.75 ms of a
// 19 ms launch on the 1M-triangle soup.)
constexpr float kReportRel = kTRel;

// Plain float32 tests for the path integrator, whose parity is statistical:
// the reference's decisions (|det| < 1e-12 rejected, u, v in [0, 1],
// u + v <= 1, t in (tmin, closest); near root then far root for spheres) in
// float32, triangles in the plane-record form below. Every fused multiply-add is
// written out (the library is compiled with -fmad=false), so each kernel
// that inlines these tests rounds them identically.
__device__ __forceinline__ float fm(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }

// Havel-Herout form on the plane records (p0 = n, n.a; p1 = n1, -n1.a;
// p2 = n2, -n2.a): det = d.n (the reference's det with the sign flipped,
// same magnitude for its |det| < 1e-12 rejection), t*det = n.(a - o), then
// u*det and v*det from the hit point scaled by det, all compared as
// numerators against |det|. The plane distance is tested first, before the
// barycentrics.
__device__ __forceinline__ bool tri_plane(const RayF& r, float4 p0, float4 p1, float4 p2, float closest, Cand& c) {
  const float det = fm(r.dx, p0.x, fm(r.dy, p0.y, mul(r.dz, p0.z)));
  if (det > -1e-12f && det < 1e-12f) return false;
  const float tn = p0.w - fm(r.ox, p0.x, fm(r.oy, p0.y, mul(r.oz, p0.z)));  // t * det
  const float ad = fabsf(det), sg = det < 0.0f ? -1.0f : 1.0f;
  const float st = sg * tn;  // t * |det|
  if (st <= r.tmin * ad || st >= closest * ad) return false;
  const float px = fm(r.ox, det, mul(r.dx, tn));  // det * (o + t d)
  const float py = fm(r.oy, det, mul(r.dy, tn));
  const float pz = fm(r.oz, det, mul(r.dz, tn));
  const float su = sg * fm(p1.x, px, fm(p1.y, py, fm(p1.z, pz, mul(det, p1.w))));  // u * |det|
  if (su < 0.0f || su > ad) return false;
  const float sv = sg * fm(p2.x, px, fm(p2.y, py, fm(p2.z, pz, mul(det, p2.w))));  // v * |det|
  if (sv < 0.0f || su + sv > ad) return false;
  const float inv = 1.0f / ad;
  const float t = st * inv;
  if (t <= r.tmin || t >= closest) return false;
  c.t = t;
  c.e = 0.0f;
  c.u = su * inv;
  c.v = sv * inv;
  return true;
}

__device__ __forceinline__ bool sphere_fast(const RayF& r, float4 c4, float rad, float closest, Cand& c) {
  const float lx = r.ox - c4.x, ly = r.oy - c4.y, lz = r.oz - c4.z;
  const float a = fm(r.dx, r.dx, fm(r.dy, r.dy, mul(r.dz, r.dz)));
  const float hb = fm(lx, r.dx, fm(ly, r.dy, mul(lz, r.dz)));
  const float cc = fm(lx, lx, fm(ly, ly, fm(lz, lz, -mul(rad, rad))));
  const float disc = fm(hb, hb, -mul(a, cc));
  if (disc < 0.0f) return false;
  const float s = sqrtf(disc);
  const float inva = 1.0f / a;
  float t = (-hb - s) * inva;
  if (t <= r.tmin || t >= closest) {
    t = (-hb + s) * inva;
    if (t <= r.tmin || t >= closest) return false;
  }
  c.t = t;
  c.e = 0.0f;
  c.u = c.v = 0.0f;
  return true;
}

// Tests one primitive of a leaf (intersect.ts:155-193).
// EXACT: a candidate replaces the closest hit when it is nearer by more than
// both error bounds; when the two distances overlap within their bounds and
// the bounds are small (a tie within 1e-5), the float32 order decides;
// otherwise both distances are recomputed in float64 and compared exactly
// like the reference. Otherwise: plain float32 tests and comparisons.
// any: returns true for any candidate (occlusion). UV: keep the closest
// hit's barycentrics (the exact walk skips them when the caller does not ask
// for them: two divisions per candidate and two stores to the walk frame).
template <bool EXACT, bool UV = true>
__device__ __forceinline__ bool test_prim(const SceneDev& s, const RayF& r, uint32_t p, HitF& h, bool any,
                                          uint32_t& fallbacks) {
  Cand c;
  if constexpr (!EXACT) {
    const float4* q = s.planes + (size_t)p * 3;
    const float4 p0 = __ldg(q);
    const float4 p1 = __ldg(q + 1);
    const bool hit = p1.x != p1.x ? sphere_fast(r, p0, p0.w, h.t, c) : tri_plane(r, p0, p1, __ldg(q + 2), h.t, c);
    if (!hit) return false;
    h.prim = (int32_t)p;
    h.t = c.t;
    h.u = c.u;
    h.v = c.v;
    return any;
  }
  // The compact copy (48 of each primitive's 64 bytes) keeps a quarter of
  // the primitives' bytes out of L2 (1M-triangle soup: 1,084 against 1,073
  // Mrays/s).
  const float4* q = s.tris + (size_t)p * 3;
  const float4 a4 = __ldg(q);
  const float4 b4 = __ldg(q + 1);
  const bool cand = a4.w == 0.0f ? sphere_candidate(r, a4, b4.x, c, fallbacks)
                                 : tri_candidate(r, a4, b4, __ldg(q + 2), c, fallbacks);
  if (!cand) return false;
  if (any) {
    h.prim = (int32_t)p;
    h.t = c.t;
    return true;
  }
  bool take;
  if (h.prim < 0 || c.t + c.e < h.t - h.err) {
    take = true;
  } else if (c.t - c.e > h.t + h.err) {
    take = false;
  } else if (c.e + h.err <= 5e-6f * fminf(c.t, h.t)) {
    take = c.t < h.t;  // a tie within 1e-5: either order is admissible
  } else {
    fallbacks += 2;
    const double tn = exact_t(s, r, (int32_t)p), tb = exact_t(s, r, h.prim);
    take = tn < tb;
    if (take) {
      c.t = (float)tn;
      c.e = rounding_err(c.t);
    } else {
      h.t = (float)tb;
      h.err = rounding_err(h.t);
    }
  }
  if (take) {
    h.prim = (int32_t)p;
    h.t = c.t;
    h.err = c.e;
    if constexpr (UV) {
      h.u = c.u;
      h.v = c.v;
    }
  }
  return false;
}

// All primitives of a leaf; returns true at the first candidate when `any`.
template <bool EXACT>
__device__ __forceinline__ bool test_leaf(const SceneDev& s, const RayF& r, uint32_t leafword, HitF& h, bool any,
                                          uint32_t& fallbacks) {
  const uint32_t count = leafword & 7u, start = leafword >> 3;
  for (uint32_t p = start; p < start + count; p++)
    if (test_prim<EXACT>(s, r, p, h, any, fallbacks)) return true;
  return false;
}

// Conservative slab test against [lo, hi]; returns the entry distance or +inf.
__device__ __forceinline__ float box_entry(const RayF& r, float lox, float hix, float loy,
                                           float hiy, float loz, float hiz, float bound) {
  const float tx0 = (lox - r.ox) * r.ix, tx1 = (hix - r.ox) * r.ix;
  const float ty0 = (loy - r.oy) * r.iy, ty1 = (hiy - r.oy) * r.iy;
  const float tz0 = (loz - r.oz) * r.iz, tz1 = (hiz - r.oz) * r.iz;
  const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1)) * kBoxWiden;
  return (tn <= tf && tf >= 0.0f && tn <= bound) ? tn : INFINITY;
}

// Upper bound of the reference's current closest distance (prunes boxes).
__device__ __forceinline__ float prune_bound(const HitF& h) { return h.t + h.err; }

// Ordered front-to-back walk over the 4-wide records (the reference's
// intersectClosest, intersect.ts:202-282, on the same boxes with two binary
// levels per step; with `any`, the any-hit query of occluded,
// intersect.ts:368-420), as a state machine advanced one step at a time: a
// step expands one record (four child boxes; the nearest child entered, the
// others pushed farthest first with their entry distances), tests one
// primitive of the current leaf, or pops the stack past entries beyond the
// closest hit. Equal-cost steps keep the lanes of a warp in step.
// The walk's counters. A step reads them once and writes them back once
// (one 16-byte access each where the walk lives in local memory).
struct alignas(16) WalkCtl {
  int32_t ref;  // >= 0 interior record, kWalkLeaf: testing [cur, end), kWalkPop, kWalkDone
  uint32_t cur, end;
  int32_t sp;
};

struct alignas(16) Walk {
  WalkCtl c;
  RayF r;
  HitF h;
  bool any, overflow;
};

// The walk stack: (child reference, entry distance bits), one 8-byte access
// per push or pop, in local memory. Beside it the lane's query number and
// fallback count: they change once per query (or never), and keeping them
// in local memory instead of registers spares the step's spill slots (exact
// walk: spill stores 72 -> 44 bytes, 1M soup 1,093 -> 1,109 Mrays/s;
// integrator: caustic scene 2,176 -> 2,194 Msamples/s, batched soups
// 1,450 -> 1,457).
struct WalkStack {
  int2 e[kStackSize];
  uint32_t idx, fallbacks;
};

// A walk's state and stack as one object. An array indexed at run time keeps
// its whole enclosing object in local memory, so in a WalkFrame the ray, hit
// and counters live in local memory beside the stack (read back from L1);
// a Walk declared apart from its WalkStack is kept in registers. Measured on
// GB300: the exact query walk (1M-triangle soup, 16.7 M rays, 40 registers)
// runs at 894 Mrays/s with a WalkFrame against 761 with the state apart
// (where the compiler spills it; 786 with only the hit in local memory, 748
// with only the ray), while the integrator's walk gains with its state
// apart (caustic scene 1,822 -> 1,914 Msamples/s, 100k soup 499 -> 526).
// With the ray and the frame 16-byte aligned (the counters first, then the
// ray's three 16-byte groups) the exact walk runs at 912 against 896; with
// the counters read and written once per step (WalkCtl) at 1,049 against
// 968 (and the integrator's walk, caustic scene, at 1,969 against 1,915).
struct WalkFrame {
  Walk w;
  WalkStack st;
};

constexpr int32_t kWalkPop = INT32_MAX, kWalkDone = INT32_MIN, kWalkLeaf = INT32_MIN + 1;

// Enters child `child` (interior record or ~leafword).
__device__ __forceinline__ void walk_enter(WalkCtl& c, int32_t child) {
  if (child >= 0) {
    c.ref = child;
  } else {
    const uint32_t word = (uint32_t)~child;
    c.cur = word >> 3;
    c.end = c.cur + (word & 7u);
    c.ref = c.cur < c.end ? kWalkLeaf : kWalkPop;
  }
}

// Starts a walk for w.r (tmin/tmax set, inverse direction computed).
__device__ __forceinline__ void walk_begin(const SceneDev& s, Walk& w, bool any) {
  w.h = HitF{-1, w.r.tmax, 0.0f, 0.0f, 0.0f};
  w.any = any;
  w.overflow = false;
  WalkCtl c{kWalkDone, 0u, 0u, 0};
  if (s.node_count != 0 && box_entry(w.r, s.root_lo[0], s.root_hi[0], s.root_lo[1], s.root_hi[1], s.root_lo[2],
                                     s.root_hi[2], w.r.tmax) != INFINITY) {
    walk_enter(c, s.root_ref);  // the root may be a leaf
    if (c.ref == kWalkPop) c.ref = kWalkDone;
  }
  w.c = c;
}

// One step; w.c.ref == kWalkDone when the query is answered. A step of the
// exact walk tests one primitive of a leaf; a step of the integrator's walk
// (plain float32 tests, a third of the instructions) tests the whole leaf,
// which pays one memory latency per leaf instead of one per primitive
// (caustic scene: 1,067 -> 1,214 Msamples/s, identical images; the exact
// walk with whole-leaf steps ran at 645 against 895 Mrays/s).
// ANYQ: the query kind when the kernel fixes it (0 closest, 1 any hit), so
// the step does not read it from the walk; -1 reads w.any (queries of both
// kinds in one launch).
template <bool EXACT, bool UV = true, int ANYQ = -1>
__device__ __forceinline__ void walk_step(const SceneDev& s, Walk& w, WalkStack& st, uint32_t& fallbacks) {
  const bool any = ANYQ < 0 ? w.any : ANYQ > 0;
  WalkCtl c = w.c;
  if (c.ref == kWalkLeaf) {
    if constexpr (EXACT) {
      if (test_prim<EXACT, UV>(s, w.r, c.cur, w.h, any, fallbacks))
        c.ref = kWalkDone;
      else if (++c.cur == c.end)
        c.ref = kWalkPop;
    } else {
      bool found = false;
      for (; c.cur < c.end && !found; c.cur++) found = test_prim<EXACT, UV>(s, w.r, c.cur, w.h, any, fallbacks);
      c.ref = found ? kWalkDone : kWalkPop;
    }
  } else if (c.ref >= 0 && c.ref != kWalkPop) {
    const uint4* q = s.quads + (size_t)c.ref * 4;
    const uint4 bx = __ldg(q), by = __ldg(q + 1), bz = __ldg(q + 2);
    const int4 c4 = __ldg(reinterpret_cast<const int4*>(q + 3));
    auto f2 = [](uint32_t h) { return __half22float2(*reinterpret_cast<const __half2*>(&h)); };
    const float2 xl01 = f2(bx.x), xl23 = f2(bx.y), xh01 = f2(bx.z), xh23 = f2(bx.w);
    const float2 yl01 = f2(by.x), yl23 = f2(by.y), yh01 = f2(by.z), yh23 = f2(by.w);
    const float2 zl01 = f2(bz.x), zl23 = f2(bz.y), zh01 = f2(bz.z), zh23 = f2(bz.w);
    const float bound = prune_bound(w.h);
    float t0 = box_entry(w.r, xl01.x, xh01.x, yl01.x, yh01.x, zl01.x, zh01.x, bound);
    float t1 = box_entry(w.r, xl01.y, xh01.y, yl01.y, yh01.y, zl01.y, zh01.y, bound);
    float t2 = box_entry(w.r, xl23.x, xh23.x, yl23.x, yh23.x, zl23.x, zh23.x, bound);
    float t3 = box_entry(w.r, xl23.y, xh23.y, yl23.y, yh23.y, zl23.y, zh23.y, bound);
    int32_t c0 = c4.x, c1 = c4.y, c2 = c4.z, c3 = c4.w;
    // Nearest first (misses, +inf, last): a five-exchange sorting network.
    auto order = [](float& ta, int32_t& ca, float& tb, int32_t& cb) {
      if (tb < ta) {
        const float t = ta;
        ta = tb, tb = t;
        const int32_t k = ca;
        ca = cb, cb = k;
      }
    };
    order(t0, c0, t1, c1);
    order(t2, c2, t3, c3);
    order(t0, c0, t2, c2);
    order(t1, c1, t3, c3);
    order(t1, c1, t2, c2);
    const int hits = (t0 != INFINITY) + (t1 != INFINITY) + (t2 != INFINITY) + (t3 != INFINITY);
    if (hits == 0) {
      c.ref = kWalkPop;
    } else if (c.sp + hits - 1 > kStackSize) {
      w.overflow = true;
      c.ref = kWalkDone;
    } else {
      if (hits > 3) st.e[c.sp++] = make_int2(c3, __float_as_int(t3));
      if (hits > 2) st.e[c.sp++] = make_int2(c2, __float_as_int(t2));
      if (hits > 1) st.e[c.sp++] = make_int2(c1, __float_as_int(t1));
      walk_enter(c, c0);
    }
  }
  if (c.ref == kWalkPop) {
    c.ref = kWalkDone;
    const float bound = prune_bound(w.h);
    while (c.sp > 0) {
      --c.sp;
      const int2 e = st.e[c.sp];
      if (__int_as_float(e.y) <= bound) {
        walk_enter(c, e.x);
        break;
      }
    }
  }
  w.c = c;
}

// Persistent warp loop over `total` queries numbered 0..total-1, handed out in
// warp-sized batches from *counter. begin(i, w) loads query i into w.r and
// calls walk_begin; finish(i, w) consumes the answer. Lanes whose queries are
// answered are refilled as soon as REFILL lanes of the warp are idle, so
// lanes keep stepping instead of waiting for the warp's slowest ray (5 suits
// the exact query walk: 1,072 Mrays/s against 1,065-1,069 at 3, 4 or 6 and
// 1,061 at 8; 6 the integrator's). Each round takes STEPS walk steps per
// lane: the exact walk two (one step per round ran 5 % slower on the
// 1M-triangle query walk, three 20 % slower), the integrator's walk, whose
// steps test whole leaves, 8 for one scene and 12 for a batch (the callers
// in wavefront.cuh give the measurements). With PHASED, the steps after the
// first move either the lanes testing primitives or those expanding records,
// whichever are more, so each branch runs with fuller warps; every lane
// still makes its own tests in the same order (the integrator's walk gains,
// the exact query walk loses 2-4 %). All 32 lanes of every warp must call
// this (the block size is a multiple of 32).
// `s` is the scene the lane walks: a fixed scene, or (queries of many scenes)
// a per-lane copy that begin() replaces with the new query's scene.
// Query numbers are below 2^32 - 1 (`total` is a uint32_t), so all ones marks
// a lane without a query (one register instead of a signed 64-bit index:
// exact 1M-soup walk 1,070 against 1,063 Mrays/s).
constexpr uint32_t kNoQuery = 0xffffffffu;

template <bool EXACT, int REFILL, bool PHASED, int STEPS, bool UV = true, int ANYQ = -1, class Scene, class Begin,
          class Finish>
__device__ __forceinline__ void walk_persistent(Scene& s, uint32_t* counter, uint32_t total, Begin begin,
                                                Finish finish, uint32_t& fallbacks) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  WalkFrame frame;             // the exact walk: state beside the stack
  Walk apart;                  // the integrator's walk: state in registers
  WalkStack apart_stack;
  Walk& w = EXACT ? frame.w : apart;
  WalkStack& st = EXACT ? frame.st : apart_stack;
  w.c.ref = kWalkDone;
  uint32_t& idx = st.idx;  // query held by this lane
  idx = kNoQuery;
  st.fallbacks = 0;
  uint32_t& fb = st.fallbacks;
  bool drained = false;
  for (;;) {
    const bool idle = w.c.ref == kWalkDone;
    if (idle && idx != kNoQuery) {
      finish(idx, w);
      idx = kNoQuery;
    }
    const uint32_t want = __ballot_sync(0xffffffffu, idle);
    if (!drained && (__popc(want) >= REFILL || want == 0xffffffffu)) {
      const uint32_t leader = __ffs(want) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(want));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + __popc(want) >= total) drained = true;
      if (idle) {
        const uint32_t k = base + __popc(want & lt_mask);
        if (k < total) {
          idx = k;
          begin(k, w);
        }
      }
    }
    if (__all_sync(0xffffffffu, idx == kNoQuery) && drained) {
      fallbacks += st.fallbacks;
      break;
    }
    // One copy of the step in the loop body (not unrolled): the integrator's
    // walk runs 1 % faster on the caustic scene, the exact walk unchanged
    // with half the spill slots.
#pragma unroll 1
    for (int k = 0; k < STEPS; k++) {
      bool go = w.c.ref != kWalkDone;
      if (PHASED && k > 0) {  // steps after the first move the majority kind
        const uint32_t leaf = __ballot_sync(0xffffffffu, w.c.ref == kWalkLeaf);
        const uint32_t inner = __ballot_sync(0xffffffffu, w.c.ref >= 0);
        go = go && (w.c.ref == kWalkLeaf) == (__popc(leaf) >= __popc(inner));
      }
      if (go) walk_step<EXACT, UV, ANYQ>(s, w, st, fb);
    }
  }
}

// Scenes of at most kBrutePrims primitives: every primitive tested in packed
// order, no boxes. The skip-link walk visits leaves in node-array order, and
// the leaves of that order cover the primitives contiguously in packed order,
// so this is the same sequence of primitive tests minus those the walk's
// (conservative) box tests would skip; every lane runs the same instructions.
constexpr uint32_t kBrutePrims = 32;

template <bool EXACT>
__device__ __forceinline__ void walk_all(const SceneDev& s, const RayF& r, HitF& h, bool any, uint32_t& fallbacks) {
  for (uint32_t p = 0; p < s.prim_count; p++)
    if (test_prim<EXACT>(s, r, p, h, any, fallbacks)) return;
}

// Stackless skip-link walk over the reference node array, the literal
// mirror of intersectClosestStackless (intersect.ts:290-365) and occluded
// (intersect.ts:368-420). Needs no stack; every lane visits nodes in the
// same increasing order, which keeps small trees in lockstep.
template <bool EXACT = true>
__device__ __forceinline__ void walk_stackless(const SceneDev& s, const RayF& r, HitF& h, bool any,
                                               uint32_t& fallbacks) {
  uint32_t node = 0;
  while (node < s.node_count) {
    const float4 lo = __ldg(s.nodes + (size_t)node * 2);
    const float4 hi = __ldg(s.nodes + (size_t)node * 2 + 1);
    if (box_entry(r, lo.x, hi.x, lo.y, hi.y, lo.z, hi.z, prune_bound(h)) == INFINITY) {
      node = (uint32_t)lo.w;
    } else if (hi.w >= 0.0f && test_leaf<EXACT>(s, r, (uint32_t)hi.w, h, any, fallbacks) && any) {
      node = s.node_count;
    } else {
      node++;
    }
  }
}

}  // namespace ctk
