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
// two candidates can only swap order when their distances tie within 4e-6.
//
// Box tests are float32 slab tests widened by 1+2*gamma(3) (Ize, "Robust BVH
// Ray Traversal", JCGT 2013), so no box the float64 test enters is skipped.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ctk {

constexpr int kStackSize = 64;               // ordered-walk stack (tree depth is checked on upload)
constexpr float kEps = 5.9604645e-8f;        // 2^-24
constexpr float kErrK = 16.0f * kEps;        // error-bound multiplier (2x the first-order bound)
constexpr float kTRel = 2e-6f;               // max relative error of a reported float32 t
constexpr float kBoxWiden = 1.0000005f;      // 1 + 2*gamma(3), rounded up

// Device view of a scene. `pairs` holds one 64-byte record per interior node
// of the reference BVH: the boxes of both children interleaved by axis and
// the two child references (>= 0 interior record, < 0 ~leafword).
struct SceneDev {
  const float4* __restrict__ prims;  // 4 per primitive (pack.ts:6-10)
  const float4* __restrict__ nodes;  // 2 per reference node (bvh.ts:6-15)
  const float4* __restrict__ pairs;  // 4 per interior node
  const float4* __restrict__ mats;   // 4 per material (pack.ts:12-16)
  const int32_t* __restrict__ lights;
  const uint32_t* __restrict__ prim_object;
  uint32_t node_count;
  uint32_t light_count;
  int32_t root_ref;
  float root_lo[3], root_hi[3];
};

struct RayF {
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

// ---- float32 tests with exact fallback -------------------------------------

// Result of a primitive test: 0 miss, 1 hit (t/u/v written).
__device__ __forceinline__ bool tri_test(const RayF& r, float4 a4, float4 b4, float4 c4,
                                         float closest, float& t_out, float& u_out, float& v_out,
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
  const float sg = det < 0.0f ? -1.0f : 1.0f;
  const float su = sg * un;
  float sv = 0.0f, st = 0.0f, ev = 0.0f, et = 0.0f;
  if (!exact) {
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
      sv = sg * (r.dx * qx + r.dy * qy + r.dz * qz);
      ev = kErrK * (fabsf(r.dx) * qax + fabsf(r.dy) * qay + fabsf(r.dz) * qaz);
      const float euv = eu + ev + ed;
      if (sv < -ev || su + sv - ad > euv) return false;  // v < 0 or u + v > 1
      if (fabsf(sv) <= ev || fabsf(su + sv - ad) <= euv) {
        exact = true;
      } else {
        st = sg * (e2x * qx + e2y * qy + e2z * qz);
        et = kErrK * (fabsf(e2x) * qax + fabsf(e2y) * qay + fabsf(e2z) * qaz);
        const float mlo = et + r.tmin * ed;
        const float dlo = st - r.tmin * ad;  // t - tmin, scaled by |det|
        if (dlo < -mlo) return false;         // t <= tmin
        if (fabsf(dlo) <= mlo) {
          exact = true;
        } else if (closest < INFINITY) {
          const float mhi = et + closest * ed;
          const float dhi = st - closest * ad;
          if (dhi > mhi) return false;  // t >= closest
          if (fabsf(dhi) <= mhi) exact = true;
        }
        if (!exact) {
          const float t = st / ad;
          if (et + t * ed > kTRel * t * ad) {
            exact = true;  // t not accurate enough for ordering
          } else {
            t_out = t;
            u_out = su / ad;
            v_out = sv / ad;
            return true;
          }
        }
      }
    }
  }
  fallbacks++;
  double t, u, v;
  if (!tri_exact(r, a4, b4, c4, (double)r.tmin, (double)closest, &t, &u, &v)) return false;
  t_out = (float)t;
  u_out = (float)u;
  v_out = (float)v;
  return true;
}

// Sphere test; returns true and sets t_out when hit in (tmin, closest).
__device__ __forceinline__ bool sphere_test(const RayF& r, float4 c4, float rad, float closest,
                                            float& t_out, uint32_t& fallbacks) {
  const float lx = r.ox - c4.x, ly = r.oy - c4.y, lz = r.oz - c4.z;
  const float a = r.dx * r.dx + r.dy * r.dy + r.dz * r.dz;
  const float hb = lx * r.dx + ly * r.dy + lz * r.dz;
  const float ll = lx * lx + ly * ly + lz * lz;
  const float c = ll - rad * rad;
  const float disc = hb * hb - a * c;
  const float hba = fabsf(lx * r.dx) + fabsf(ly * r.dy) + fabsf(lz * r.dz);
  const float edisc = kErrK * (hba * hba + a * (ll + rad * rad));
  bool exact = false;
  if (disc < -edisc) return false;
  if (disc <= edisc) {
    exact = true;
  } else {
    const float s = sqrtf(disc);
    const float es = edisc / s + kEps * s;
    const float ehb = kErrK * hba;
    const float inva = 1.0f / a;
    // candidate roots, near first (intersect.ts:33-37)
    for (int k = 0; k < 2 && !exact; k++) {
      const float num = k == 0 ? -hb - s : -hb + s;
      const float t = num * inva;
      const float e = (ehb + es) * inva + kErrK * fabsf(t);
      if (t + e <= r.tmin || t - e >= closest) continue;  // root rejected for certain
      if (t - e > r.tmin && t + e < closest) {
        if (e > kTRel * t) {
          exact = true;
          break;
        }
        t_out = t;
        return true;
      }
      exact = true;
    }
    if (!exact) return false;
  }
  fallbacks++;
  const double t = sphere_exact(r, c4, rad, (double)r.tmin, (double)closest);
  if (!(t > 0)) return false;
  t_out = (float)t;
  return true;
}

// Conservative slab test against [lo, hi]; returns the entry distance or +inf.
__device__ __forceinline__ float box_entry(const RayF& r, float lox, float hix, float loy,
                                           float hiy, float loz, float hiz, float closest) {
  const float tx0 = (lox - r.ox) * r.ix, tx1 = (hix - r.ox) * r.ix;
  const float ty0 = (loy - r.oy) * r.iy, ty1 = (hiy - r.oy) * r.iy;
  const float tz0 = (loz - r.oz) * r.iz, tz1 = (hiz - r.oz) * r.iz;
  const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1)) * kBoxWiden;
  return (tn <= tf && tf >= 0.0f && tn <= closest) ? tn : INFINITY;
}

struct HitF {
  int32_t prim;
  float t, u, v;
};

// Tests the primitives of a leaf (intersect.ts:155-193). ANY: stop at the first hit.
template <bool ANY>
__device__ __forceinline__ bool test_leaf(const SceneDev& s, const RayF& r, uint32_t leafword,
                                          HitF& h, uint32_t& fallbacks) {
  const uint32_t count = leafword & 7u, start = leafword >> 3;
  for (uint32_t p = start; p < start + count; p++) {
    const float4* q = s.prims + (size_t)p * 4;
    const float4 a4 = __ldg(q);
    const float4 b4 = __ldg(q + 1);
    float t, u = 0.0f, v = 0.0f;
    bool hit;
    if (a4.w == 0.0f) {
      hit = sphere_test(r, a4, b4.x, h.t, t, fallbacks);
    } else {
      const float4 c4 = __ldg(q + 2);
      hit = tri_test(r, a4, b4, c4, h.t, t, u, v, fallbacks);
    }
    if (hit) {
      h.t = t;
      h.prim = (int32_t)p;
      h.u = u;
      h.v = v;
      if (ANY) return true;
    }
  }
  return false;
}

// Ordered front-to-back walk over the interior pair records (the reference's
// intersectClosest, intersect.ts:202-282). ANY = any-hit for occlusion
// (intersect.ts:368-420). h.t must hold the ray's tmax on entry. Returns
// false if the stack would overflow (never for trees that passed the upload
// depth check); no out-of-bounds write happens in that case.
template <bool ANY>
__device__ __forceinline__ bool walk_ordered(const SceneDev& s, const RayF& r, HitF& h,
                                             uint32_t& fallbacks) {
  if (box_entry(r, s.root_lo[0], s.root_hi[0], s.root_lo[1], s.root_hi[1], s.root_lo[2],
                s.root_hi[2], h.t) == INFINITY)
    return true;
  int32_t stack_ref[kStackSize];
  float stack_t[kStackSize];
  int sp = 0;
  int32_t ref = s.root_ref;
  for (;;) {
    while (ref >= 0) {
      const float4* pr = s.pairs + (size_t)ref * 4;
      const float4 n0 = __ldg(pr), n1 = __ldg(pr + 1), n2 = __ldg(pr + 2), n3 = __ldg(pr + 3);
      const float tl = box_entry(r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, h.t);
      const float tr = box_entry(r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, h.t);
      const int32_t cl = __float_as_int(n3.x), cr = __float_as_int(n3.y);
      if (tl != INFINITY) {
        if (tr != INFINITY) {
          if (sp >= kStackSize) return false;
          if (tl <= tr) {
            stack_ref[sp] = cr;
            stack_t[sp++] = tr;
            ref = cl;
          } else {
            stack_ref[sp] = cl;
            stack_t[sp++] = tl;
            ref = cr;
          }
        } else {
          ref = cl;
        }
        continue;
      }
      if (tr != INFINITY) {
        ref = cr;
        continue;
      }
      ref = INT32_MAX;  // no child entered: pop
      break;
    }
    if (ref != INT32_MAX) {
      if (test_leaf<ANY>(s, r, (uint32_t)~ref, h, fallbacks)) return true;
    }
    // pop entries still closer than the current hit
    for (;;) {
      if (sp == 0) return true;
      --sp;
      if (stack_t[sp] < h.t) break;
    }
    ref = stack_ref[sp];
  }
}

// Stackless skip-link walk over the reference node array, the literal
// mirror of intersectClosestStackless (intersect.ts:290-365) and occluded
// (intersect.ts:368-420).
template <bool ANY>
__device__ __forceinline__ void walk_stackless(const SceneDev& s, const RayF& r, HitF& h,
                                               uint32_t& fallbacks) {
  uint32_t node = 0;
  while (node < s.node_count) {
    const float4 lo = __ldg(s.nodes + (size_t)node * 2);
    const float4 hi = __ldg(s.nodes + (size_t)node * 2 + 1);
    if (box_entry(r, lo.x, hi.x, lo.y, hi.y, lo.z, hi.z, h.t) == INFINITY) {
      node = (uint32_t)lo.w;
      continue;
    }
    if (hi.w >= 0.0f) {
      if (test_leaf<ANY>(s, r, (uint32_t)hi.w, h, fallbacks)) return;
    }
    node++;
  }
}

}  // namespace ctk
