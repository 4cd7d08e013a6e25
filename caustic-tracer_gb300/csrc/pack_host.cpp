// Host packer of libcaustic_gb300: ct_pack_scene.
//
// Produces the reference's PackedScene arrays (pack.ts:195-223) bit for bit:
// primitives enumerated in scene order (pack.ts:131-192), a binned-SAH BVH
// with 12 buckets and leaves of at most 4 primitives (bvh.ts:111-296) stored
// as the depth-first skip-link node array (bvh.ts:6-15), primitives reordered
// into leaf order, materials (pack.ts:75-119) and the emitter list.
//
// The build is iterative (explicit work stack) and bins all three axes in one
// sweep over a node's primitives; node numbering, the float64 arithmetic of
// the cost sweeps and the in-place partition follow the reference exactly so
// the resulting arrays are identical. Compile with -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include "common.hpp"

namespace ct {

namespace {
thread_local std::string g_last_error;
}

ct_status fail(ct_status status, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

void clear_error() { g_last_error.clear(); }

const char* last_error() { return g_last_error.c_str(); }

namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr int kBuckets = CT_SAH_BUCKETS;
constexpr double kPi = 3.14159265358979323846;

struct Bounds3 {
  double lo[3], hi[3];
};

// Scene-order primitive soup: float records plus float64 bounds/centroids.
struct Soup {
  std::vector<float> prims;        // 16 per primitive, scene order
  std::vector<uint32_t> object;    // scene object per primitive
  std::vector<double> lo, hi, mid; // 3 per primitive
};

inline void put_bounds(Soup& s, size_t i, double x0, double y0, double z0, double x1, double y1,
                       double z1) {
  double* lo = &s.lo[i * 3];
  double* hi = &s.hi[i * 3];
  double* mid = &s.mid[i * 3];
  lo[0] = x0, lo[1] = y0, lo[2] = z0;
  hi[0] = x1, hi[1] = y1, hi[2] = z1;
  mid[0] = 0.5 * (x0 + x1);
  mid[1] = 0.5 * (y0 + y1);
  mid[2] = 0.5 * (z0 + z1);
}

inline double min3(double a, double b, double c) { return std::min(std::min(a, b), c); }
inline double max3(double a, double b, double c) { return std::max(std::max(a, b), c); }

// One triangle record (pack.ts:158-189): vertices, unit normal, area, bounds.
void emit_triangle(Soup& s, size_t p, uint32_t obj, const double a[3], const double b[3],
                   const double c[3]) {
  float* r = &s.prims[p * CT_PRIM_STRIDE];
  const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                        e1[0] * e2[1] - e1[1] * e2[0]};
  // normalize (vec3.ts:29-32): scale by 1/len, zero vector when degenerate
  const double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
  double n[3] = {0, 0, 0};
  if (len > 0) {
    const double inv = 1 / len;
    n[0] = cr[0] * inv, n[1] = cr[1] * inv, n[2] = cr[2] * inv;
  }
  const double area = 0.5 * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
  for (int k = 0; k < 3; k++) {
    r[k] = (float)a[k];
    r[4 + k] = (float)b[k];
    r[8 + k] = (float)c[k];
    r[12 + k] = (float)n[k];
  }
  r[3] = CT_PRIM_TRIANGLE;
  r[7] = (float)obj;
  r[11] = (float)area;
  r[15] = 0;
  s.object[p] = obj;
  const double pad = 1e-6;
  put_bounds(s, p, min3(a[0], b[0], c[0]) - pad, min3(a[1], b[1], c[1]) - pad,
             min3(a[2], b[2], c[2]) - pad, max3(a[0], b[0], c[0]) + pad,
             max3(a[1], b[1], c[1]) + pad, max3(a[2], b[2], c[2]) + pad);
}

uint64_t primitive_count(const ct_shape& sh) {
  switch (sh.kind) {
    case 0:
    case 1:
      return 1;
    case 2:
      return 2;
    case 3:
      return sh.index_count / 3;
    default:
      return 0;
  }
}

ct_status enumerate(const ct_object* objs, uint32_t n, Soup& s, uint32_t* total_out) {
  uint64_t total = 0;
  for (uint32_t i = 0; i < n; i++) {
    const ct_shape& sh = objs[i].shape;
    if (sh.kind < 0 || sh.kind > 3) return fail(CT_ERR_INVALID_ARGUMENT, "object %u: unknown shape kind %d", i, sh.kind);
    if (sh.kind == 3) {
      if ((sh.index_count && !sh.indices) || (sh.vertex_count && !sh.vertices))
        return fail(CT_ERR_INVALID_ARGUMENT, "object %u: mesh arrays missing", i);
      for (uint32_t k = 0; k < sh.index_count - sh.index_count % 3; k++)
        if (sh.indices[k] >= sh.vertex_count)
          return fail(CT_ERR_INVALID_ARGUMENT, "object %u: mesh index %u out of range", i, sh.indices[k]);
    }
    total += primitive_count(sh);
  }
  // Leaf words store start*8+count in a float32 (bvh.ts:60-62): exact below 2^24.
  if (total * 8 + 8 > (1ull << 24))
    return fail(CT_ERR_UNSUPPORTED, "scene has %llu primitives; the packed float32 leaf encoding holds at most %u",
                (unsigned long long)total, (unsigned)((1u << 21) - 1));
  const size_t slots = std::max<uint64_t>(1, total);
  s.prims.assign(slots * CT_PRIM_STRIDE, 0.0f);
  s.object.assign(slots, 0);
  s.lo.resize(total * 3);
  s.hi.resize(total * 3);
  s.mid.resize(total * 3);
  size_t p = 0;
  for (uint32_t obj = 0; obj < n; obj++) {
    const ct_shape& sh = objs[obj].shape;
    const double* q = sh.p;
    switch (sh.kind) {
      case 0: {  // sphere (pack.ts:140-156)
        float* r = &s.prims[p * CT_PRIM_STRIDE];
        const double rad = q[3];
        r[0] = (float)q[0], r[1] = (float)q[1], r[2] = (float)q[2];
        r[3] = CT_PRIM_SPHERE;
        r[4] = (float)rad;
        r[7] = (float)obj;
        r[11] = (float)(4 * kPi * rad * rad);
        s.object[p] = obj;
        const double rp = rad + 1e-6 + std::fabs(rad) * 1e-6;
        put_bounds(s, p, q[0] - rp, q[1] - rp, q[2] - rp, q[0] + rp, q[1] + rp, q[2] + rp);
        p++;
        break;
      }
      case 1:
        emit_triangle(s, p++, obj, q, q + 3, q + 6);
        break;
      case 2: {  // quad (scene.ts:85-94)
        const double p0[3] = {q[0], q[1], q[2]};
        const double p1[3] = {q[0] + q[3], q[1] + q[4], q[2] + q[5]};
        const double p2[3] = {p1[0] + q[6], p1[1] + q[7], p1[2] + q[8]};
        const double p3[3] = {q[0] + q[6], q[1] + q[7], q[2] + q[8]};
        emit_triangle(s, p++, obj, p0, p1, p2);
        emit_triangle(s, p++, obj, p0, p2, p3);
        break;
      }
      case 3:  // mesh (scene.ts:96-105)
        for (uint32_t k = 0; k + 2 < sh.index_count; k += 3)
          emit_triangle(s, p++, obj, sh.vertices + 3 * (size_t)sh.indices[k],
                        sh.vertices + 3 * (size_t)sh.indices[k + 1],
                        sh.vertices + 3 * (size_t)sh.indices[k + 2]);
        break;
    }
  }
  *total_out = (uint32_t)total;
  return CT_OK;
}

inline double surface_area(double dx, double dy, double dz) { return 2 * (dx * dy + dy * dz + dz * dx); }

inline int bucket(double c, double origin, double scale) {
  double b = std::floor((c - origin) * scale);
  if (b >= kBuckets) b = kBuckets - 1;
  if (b < 0) b = 0;
  return (int)b;
}

struct Bin {
  int count;
  double lo[3], hi[3];
};

class BvhBuilder {
 public:
  BvhBuilder(const Soup& s, uint32_t count) : s_(s), count_(count) {
    order.resize(count);
    for (uint32_t i = 0; i < count; i++) order[i] = i;
  }

  std::vector<uint32_t> order;
  std::vector<float> nodes;
  uint32_t node_count = 0;

  void build() {
    if (count_ == 0) {  // bvh.ts:93-100: one empty leaf
      nodes.assign(CT_NODE_STRIDE, 0.0f);
      nodes[3] = 1;
      nodes[7] = 0;
      node_count = 1;
      return;
    }
    nodes.resize(((size_t)2 * count_ - 1) * CT_NODE_STRIDE);
    std::vector<std::pair<uint32_t, uint32_t>> work;  // pending [start, end) ranges, DFS order
    work.emplace_back(0, count_);
    while (!work.empty()) {
      auto [start, end] = work.back();
      work.pop_back();
      const uint32_t index = node_count++;
      float* node = &nodes[(size_t)index * CT_NODE_STRIDE];
      Bounds3 box, cbox;
      range_bounds(start, end, box, cbox);
      for (int k = 0; k < 3; k++) {  // bvh.ts:140-147 outward nudge
        node[k] = (float)(box.lo[k] - std::fabs(box.lo[k]) * 1.2e-7 - 1e-9);
        node[4 + k] = (float)(box.hi[k] + std::fabs(box.hi[k]) * 1.2e-7 + 1e-9);
      }
      if (end - start <= CT_MAX_LEAF_PRIMS) {
        node[7] = (float)((double)start * 8 + (end - start));
        continue;
      }
      int64_t mid = sah_partition(start, end, cbox);
      if (mid <= (int64_t)start || mid >= (int64_t)end) mid = median_partition(start, end, cbox);
      node[7] = -1.0f;
      // The left range is built next, the right range after the whole left subtree.
      work.emplace_back((uint32_t)mid, end);
      work.emplace_back(start, (uint32_t)mid);
    }
    nodes.resize((size_t)node_count * CT_NODE_STRIDE);
    // Skip links: a leaf skips to the next node; an interior node skips to where
    // its right child's subtree ends. Children have larger indices, so a
    // reverse sweep sees them first.
    for (int64_t i = (int64_t)node_count - 1; i >= 0; i--) {
      float* node = &nodes[(size_t)i * CT_NODE_STRIDE];
      if (node[7] >= 0) {
        node[3] = (float)(i + 1);
      } else {
        const uint32_t right = (uint32_t)nodes[(size_t)(i + 1) * CT_NODE_STRIDE + 3];
        node[3] = nodes[(size_t)right * CT_NODE_STRIDE + 3];
      }
    }
  }

 private:
  const Soup& s_;
  uint32_t count_;

  void range_bounds(uint32_t start, uint32_t end, Bounds3& box, Bounds3& cbox) const {
    for (int k = 0; k < 3; k++) {
      box.lo[k] = cbox.lo[k] = kInf;
      box.hi[k] = cbox.hi[k] = -kInf;
    }
    for (uint32_t i = start; i < end; i++) {
      const size_t o = (size_t)order[i] * 3;
      for (int k = 0; k < 3; k++) {
        if (s_.lo[o + k] < box.lo[k]) box.lo[k] = s_.lo[o + k];
        if (s_.hi[o + k] > box.hi[k]) box.hi[k] = s_.hi[o + k];
        if (s_.mid[o + k] < cbox.lo[k]) cbox.lo[k] = s_.mid[o + k];
        if (s_.mid[o + k] > cbox.hi[k]) cbox.hi[k] = s_.mid[o + k];
      }
    }
  }

  // Binned SAH (bvh.ts:168-281): returns the partition point or -1.
  int64_t sah_partition(uint32_t start, uint32_t end, const Bounds3& cbox) {
    Bin bins[3][kBuckets];
    bool live[3];
    double scale[3];
    for (int axis = 0; axis < 3; axis++) {
      const double extent = cbox.hi[axis] - cbox.lo[axis];
      live[axis] = extent > 1e-12;
      scale[axis] = live[axis] ? kBuckets / extent : 0;
      for (Bin& b : bins[axis]) {
        b.count = 0;
        for (int k = 0; k < 3; k++) b.lo[k] = kInf, b.hi[k] = -kInf;
      }
    }
    if (!live[0] && !live[1] && !live[2]) return -1;
    for (uint32_t i = start; i < end; i++) {
      const size_t o = (size_t)order[i] * 3;
      for (int axis = 0; axis < 3; axis++) {
        if (!live[axis]) continue;
        Bin& b = bins[axis][bucket(s_.mid[o + axis], cbox.lo[axis], scale[axis])];
        b.count++;
        for (int k = 0; k < 3; k++) {
          if (s_.lo[o + k] < b.lo[k]) b.lo[k] = s_.lo[o + k];
          if (s_.hi[o + k] > b.hi[k]) b.hi[k] = s_.hi[o + k];
        }
      }
    }
    double best_cost = kInf;
    int best_axis = -1, best_split = -1;
    for (int axis = 0; axis < 3; axis++) {
      if (!live[axis]) continue;
      const Bin* b = bins[axis];
      double right_area[kBuckets];
      int right_count[kBuckets];
      double r0[3] = {kInf, kInf, kInf}, r1[3] = {-kInf, -kInf, -kInf};
      int rc = 0;
      for (int s = kBuckets - 1; s >= 1; s--) {
        if (b[s].count > 0) {
          for (int k = 0; k < 3; k++) {
            if (b[s].lo[k] < r0[k]) r0[k] = b[s].lo[k];
            if (b[s].hi[k] > r1[k]) r1[k] = b[s].hi[k];
          }
          rc += b[s].count;
        }
        right_count[s - 1] = rc;
        right_area[s - 1] = rc > 0 ? surface_area(r1[0] - r0[0], r1[1] - r0[1], r1[2] - r0[2]) : 0;
      }
      double l0[3] = {kInf, kInf, kInf}, l1[3] = {-kInf, -kInf, -kInf};
      int lc = 0;
      for (int s = 0; s < kBuckets - 1; s++) {
        if (b[s].count > 0) {
          for (int k = 0; k < 3; k++) {
            if (b[s].lo[k] < l0[k]) l0[k] = b[s].lo[k];
            if (b[s].hi[k] > l1[k]) l1[k] = b[s].hi[k];
          }
          lc += b[s].count;
        }
        if (lc == 0 || right_count[s] == 0) continue;
        const double cost = lc * surface_area(l1[0] - l0[0], l1[1] - l0[1], l1[2] - l0[2]) +
                            right_count[s] * right_area[s];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = axis;
          best_split = s;
        }
      }
    }
    if (best_axis < 0) return -1;
    // bvh.ts:262-278: two-ended in-place partition; bucket <= split goes left.
    const double origin = cbox.lo[best_axis], sc = scale[best_axis];
    int64_t lo = start, hi = (int64_t)end - 1;
    while (lo <= hi) {
      if (bucket(s_.mid[(size_t)order[lo] * 3 + best_axis], origin, sc) <= best_split) {
        lo++;
      } else {
        std::swap(order[lo], order[hi]);
        hi--;
      }
    }
    if (lo == (int64_t)start || lo == (int64_t)end) return -1;
    return lo;
  }

  // bvh.ts:284-296: stable sort on the widest centroid axis, split in half.
  int64_t median_partition(uint32_t start, uint32_t end, const Bounds3& cbox) {
    const double ex = cbox.hi[0] - cbox.lo[0], ey = cbox.hi[1] - cbox.lo[1],
                 ez = cbox.hi[2] - cbox.lo[2];
    const int axis = ex >= ey && ex >= ez ? 0 : ey >= ez ? 1 : 2;
    const double* mid = s_.mid.data();
    std::stable_sort(order.begin() + start, order.begin() + end, [&](uint32_t a, uint32_t b) {
      return mid[(size_t)a * 3 + axis] < mid[(size_t)b * 3 + axis];
    });
    return (int64_t)((start + end) >> 1);
  }
};

// Material record (pack.ts:75-119) and its emission (scene.ts:176-185).
bool emission_of(const ct_material& m, double e[3]) {
  if (m.type == CT_MAT_EMISSIVE) {
    for (int k = 0; k < 3; k++) e[k] = m.color[k] * m.param;
    return true;
  }
  if (m.type == CT_MAT_LAMBERTIAN && m.has_emission &&
      (m.emission[0] > 0 || m.emission[1] > 0 || m.emission[2] > 0)) {
    for (int k = 0; k < 3; k++) e[k] = m.emission[k];
    return true;
  }
  return false;
}

void write_material(float* r, const ct_material& m) {
  std::memset(r, 0, sizeof(float) * CT_MAT_STRIDE);
  r[3] = (float)m.type;
  for (int k = 0; k < 3; k++) r[k] = (float)m.color[k];
  if (m.type == CT_MAT_LAMBERTIAN) {
    if (m.has_checker) {
      r[5] = (float)m.checker_scale;
      r[6] = 1;
      for (int k = 0; k < 3; k++) r[8 + k] = (float)m.checker_color2[k];
    }
  } else {
    r[4] = (float)m.param;
  }
  double e[3];
  if (emission_of(m, e))
    for (int k = 0; k < 3; k++) r[12 + k] = (float)e[k];
}

struct PackedOwner : ct_packed_scene {
  std::vector<float> prims, nodes, mats;
  std::vector<int32_t> lights;
  std::vector<uint32_t> prim_object, order_storage;
};

}  // namespace
}  // namespace ct

extern "C" {

int32_t ct_abi_version(void) { return CT_ABI_VERSION; }

const char* ct_last_error(void) { return ct::last_error(); }

ct_status ct_pack_scene(const ct_object* objects, uint32_t object_count, const ct_sky* sky,
                        ct_packed_scene** out) {
  using namespace ct;
  clear_error();
  CT_CHECK_ARG(out != nullptr, "ct_pack_scene: out is NULL");
  CT_CHECK_ARG(object_count == 0 || objects != nullptr, "ct_pack_scene: objects is NULL");
  *out = nullptr;
  for (uint32_t i = 0; i < object_count; i++)
    CT_CHECK_ARG(objects[i].material.type >= 0 && objects[i].material.type <= 3,
                 "object %u: unknown material type %d", i, objects[i].material.type);
  try {
    Soup soup;
    uint32_t total = 0;
    ct_status st = enumerate(objects, object_count, soup, &total);
    if (st != CT_OK) return st;
    BvhBuilder bvh(soup, total);
    bvh.build();
    auto* own = new PackedOwner();
    own->prims.assign((size_t)std::max<uint32_t>(1, total) * CT_PRIM_STRIDE, 0.0f);
    own->prim_object.assign(std::max<uint32_t>(1, total), 0);
    for (uint32_t i = 0; i < total; i++) {
      const uint32_t src = bvh.order[i];
      std::memcpy(&own->prims[(size_t)i * CT_PRIM_STRIDE], &soup.prims[(size_t)src * CT_PRIM_STRIDE],
                  sizeof(float) * CT_PRIM_STRIDE);
      own->prim_object[i] = soup.object[src];
    }
    own->mats.assign((size_t)std::max<uint32_t>(1, object_count) * CT_MAT_STRIDE, 0.0f);
    std::vector<uint8_t> emits(object_count, 0);
    for (uint32_t i = 0; i < object_count; i++) {
      write_material(&own->mats[(size_t)i * CT_MAT_STRIDE], objects[i].material);
      double e[3];
      emits[i] = emission_of(objects[i].material, e) ? 1 : 0;
    }
    for (uint32_t i = 0; i < total; i++)
      if (emits[own->prim_object[i]]) own->lights.push_back((int32_t)i);
    own->nodes = std::move(bvh.nodes);
    own->order_storage = std::move(bvh.order);
    ct_packed_scene_view& v = own->view;
    v.prims = own->prims.data();
    v.prim_count = total;
    v.nodes = own->nodes.data();
    v.node_count = bvh.node_count;
    v.mats = own->mats.data();
    v.mat_count = object_count;
    v.lights = own->lights.data();
    v.light_count = (uint32_t)own->lights.size();
    v.prim_object = own->prim_object.data();
    std::memset(&v.sky, 0, sizeof v.sky);
    if (sky) v.sky = *sky;
    own->order = own->order_storage.data();
    *out = own;
    return CT_OK;
  } catch (const std::bad_alloc&) {
    return fail(CT_ERR_OUT_OF_MEMORY, "ct_pack_scene: host allocation failed");
  }
}

void ct_packed_scene_free(ct_packed_scene* ps) {
  if (!ps) return;
  delete static_cast<ct::PackedOwner*>(ps);
}

// rng.ts mirror for host-side scene generators: n draws of Rng(seed).next()
// (kind 0), nextU32() (kind 1) or range(lo, hi) (kind 2); returns the state
// reached so a caller can continue the stream with ct_rng_continue.
uint32_t ct_rng_stream(uint32_t seed_or_state, int32_t is_state, uint64_t n, int32_t kind,
                       double lo, double hi, double* out) {
  auto pcg = [](uint32_t x) {
    uint32_t state = x * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28) + 4u)) ^ state) * 277803737u;
    return (word >> 22) ^ word;
  };
  uint32_t st;
  if (is_state) {
    st = seed_or_state;
  } else {
    st = pcg(seed_or_state);
    if (st == 0) st = 0x9e3779b9u;
  }
  for (uint64_t i = 0; i < n; i++) {
    st ^= st << 13;
    st ^= st >> 17;
    st ^= st << 5;
    const double u = (double)st / 4294967296.0;
    out[i] = kind == 1 ? (double)st : kind == 0 ? u : lo + (hi - lo) * u;
  }
  return st;
}

}  // extern "C"
