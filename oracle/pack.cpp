// Oracle (test infrastructure): scene packing and the binned-SAH BVH build.
// Restates src/tracer/pack.ts and src/tracer/bvh.ts of the reference.
#include <algorithm>
#include <cmath>
#include <limits>

#include "oracle.hpp"

namespace oracle {

namespace {

constexpr double INF = std::numeric_limits<double>::infinity();
constexpr int BUCKETS = CT_SAH_BUCKETS;

struct PrimBounds {  // bvh.ts:22-28
  uint32_t count = 0;
  std::vector<double> min, max, centroid;
};

// bvh.ts:46-58
void set_prim_bounds(PrimBounds& pb, uint32_t i, double x0, double y0, double z0, double x1,
                     double y1, double z1) {
  size_t o = (size_t)i * 3;
  pb.min[o] = x0;
  pb.min[o + 1] = y0;
  pb.min[o + 2] = z0;
  pb.max[o] = x1;
  pb.max[o + 1] = y1;
  pb.max[o + 2] = z1;
  pb.centroid[o] = 0.5 * (x0 + x1);
  pb.centroid[o + 1] = 0.5 * (y0 + y1);
  pb.centroid[o + 2] = 0.5 * (z0 + z1);
}

double encode_leaf(double start, double count) { return start * 8 + count; }  // bvh.ts:60-62

double surface_area(double dx, double dy, double dz) {  // bvh.ts:70
  return 2 * (dx * dy + dy * dz + dz * dx);
}

// bvh.ts:72-297
struct Builder {
  const PrimBounds& pb;
  std::vector<uint32_t> order;
  std::vector<float> nodes;
  uint32_t node_count = 0;
  int bucket_count[BUCKETS];
  double bucket_min[BUCKETS * 3], bucket_max[BUCKETS * 3];
  double right_area[BUCKETS];
  int right_count[BUCKETS];

  explicit Builder(const PrimBounds& b) : pb(b) {
    order.resize(pb.count);
    for (uint32_t i = 0; i < pb.count; i++) order[i] = i;
    size_t n = pb.count > 0 ? 2 * (size_t)pb.count - 1 : 1;
    nodes.assign(std::max<size_t>(1, n) * CT_NODE_STRIDE, 0.0f);
  }

  void build() {  // bvh.ts:92-109
    if (pb.count == 0) {
      float* n = nodes.data();
      n[0] = n[1] = n[2] = 0;
      n[3] = 1;
      n[4] = n[5] = n[6] = 0;
      n[7] = (float)encode_leaf(0, 0);
      node_count = 1;
    } else {
      build_node(0, pb.count);
    }
    nodes.resize((size_t)node_count * CT_NODE_STRIDE);
  }

  void build_node(uint32_t start, uint32_t end) {  // bvh.ts:111-165
    uint32_t node_index = node_count++;
    size_t base = (size_t)node_index * CT_NODE_STRIDE;
    double bminx = INF, bminy = INF, bminz = INF, bmaxx = -INF, bmaxy = -INF, bmaxz = -INF;
    double cminx = INF, cminy = INF, cminz = INF, cmaxx = -INF, cmaxy = -INF, cmaxz = -INF;
    for (uint32_t i = start; i < end; i++) {
      size_t o = (size_t)order[i] * 3;
      double x0 = pb.min[o], y0 = pb.min[o + 1], z0 = pb.min[o + 2];
      double x1 = pb.max[o], y1 = pb.max[o + 1], z1 = pb.max[o + 2];
      if (x0 < bminx) bminx = x0;
      if (y0 < bminy) bminy = y0;
      if (z0 < bminz) bminz = z0;
      if (x1 > bmaxx) bmaxx = x1;
      if (y1 > bmaxy) bmaxy = y1;
      if (z1 > bmaxz) bmaxz = z1;
      double cx = pb.centroid[o], cy = pb.centroid[o + 1], cz = pb.centroid[o + 2];
      if (cx < cminx) cminx = cx;
      if (cy < cminy) cminy = cy;
      if (cz < cminz) cminz = cz;
      if (cx > cmaxx) cmaxx = cx;
      if (cy > cmaxy) cmaxy = cy;
      if (cz > cmaxz) cmaxz = cz;
    }
    // bvh.ts:140-147: outward nudge before the Float32 store.
    nodes[base] = (float)(bminx - std::fabs(bminx) * 1.2e-7 - 1e-9);
    nodes[base + 1] = (float)(bminy - std::fabs(bminy) * 1.2e-7 - 1e-9);
    nodes[base + 2] = (float)(bminz - std::fabs(bminz) * 1.2e-7 - 1e-9);
    nodes[base + 4] = (float)(bmaxx + std::fabs(bmaxx) * 1.2e-7 + 1e-9);
    nodes[base + 5] = (float)(bmaxy + std::fabs(bmaxy) * 1.2e-7 + 1e-9);
    nodes[base + 6] = (float)(bmaxz + std::fabs(bmaxz) * 1.2e-7 + 1e-9);

    uint32_t count = end - start;
    if (count <= CT_MAX_LEAF_PRIMS) {
      nodes[base + 3] = (float)(node_index + 1);
      nodes[base + 7] = (float)encode_leaf(start, count);
      return;
    }
    int64_t mid = sah_split(start, end, cminx, cminy, cminz, cmaxx, cmaxy, cmaxz);
    if (mid <= (int64_t)start || mid >= (int64_t)end)
      mid = median_split(start, end, cminx, cminy, cminz, cmaxx, cmaxy, cmaxz);
    nodes[base + 7] = -1.0f;
    build_node(start, (uint32_t)mid);
    build_node((uint32_t)mid, end);
    nodes[base + 3] = (float)node_count;
  }

  int bucket_of(double c, double origin, double scale_) const {
    double b = std::floor((c - origin) * scale_);
    if (b >= BUCKETS) b = BUCKETS - 1;
    if (b < 0) b = 0;
    return (int)b;
  }

  // bvh.ts:168-281
  int64_t sah_split(uint32_t start, uint32_t end, double cminx, double cminy, double cminz,
                    double cmaxx, double cmaxy, double cmaxz) {
    double best_cost = INF;
    int best_axis = -1, best_split = -1;
    double best_origin = 0, best_scale = 0;
    for (int axis = 0; axis < 3; axis++) {
      double cmin = axis == 0 ? cminx : axis == 1 ? cminy : cminz;
      double cmax = axis == 0 ? cmaxx : axis == 1 ? cmaxy : cmaxz;
      double extent = cmax - cmin;
      if (!(extent > 1e-12)) continue;
      double to_bucket = BUCKETS / extent;
      for (int k = 0; k < BUCKETS; k++) bucket_count[k] = 0;
      for (int k = 0; k < BUCKETS * 3; k++) {
        bucket_min[k] = INF;
        bucket_max[k] = -INF;
      }
      for (uint32_t i = start; i < end; i++) {
        size_t o = (size_t)order[i] * 3;
        int b = bucket_of(pb.centroid[o + axis], cmin, to_bucket);
        bucket_count[b]++;
        int bo = b * 3;
        for (int k = 0; k < 3; k++) {
          if (pb.min[o + k] < bucket_min[bo + k]) bucket_min[bo + k] = pb.min[o + k];
          if (pb.max[o + k] > bucket_max[bo + k]) bucket_max[bo + k] = pb.max[o + k];
        }
      }
      // bvh.ts:213-230: suffix sweep over buckets s+1..end.
      double rx0 = INF, ry0 = INF, rz0 = INF, rx1 = -INF, ry1 = -INF, rz1 = -INF;
      int rc = 0;
      for (int s = BUCKETS - 1; s >= 1; s--) {
        int bo = s * 3;
        if (bucket_count[s] > 0) {
          if (bucket_min[bo] < rx0) rx0 = bucket_min[bo];
          if (bucket_min[bo + 1] < ry0) ry0 = bucket_min[bo + 1];
          if (bucket_min[bo + 2] < rz0) rz0 = bucket_min[bo + 2];
          if (bucket_max[bo] > rx1) rx1 = bucket_max[bo];
          if (bucket_max[bo + 1] > ry1) ry1 = bucket_max[bo + 1];
          if (bucket_max[bo + 2] > rz1) rz1 = bucket_max[bo + 2];
          rc += bucket_count[s];
        }
        right_count[s - 1] = rc;
        right_area[s - 1] = rc > 0 ? surface_area(rx1 - rx0, ry1 - ry0, rz1 - rz0) : 0;
      }
      // bvh.ts:232-257: prefix sweep, left side = buckets 0..s.
      double lx0 = INF, ly0 = INF, lz0 = INF, lx1 = -INF, ly1 = -INF, lz1 = -INF;
      int lc = 0;
      for (int s = 0; s < BUCKETS - 1; s++) {
        int bo = s * 3;
        if (bucket_count[s] > 0) {
          if (bucket_min[bo] < lx0) lx0 = bucket_min[bo];
          if (bucket_min[bo + 1] < ly0) ly0 = bucket_min[bo + 1];
          if (bucket_min[bo + 2] < lz0) lz0 = bucket_min[bo + 2];
          if (bucket_max[bo] > lx1) lx1 = bucket_max[bo];
          if (bucket_max[bo + 1] > ly1) ly1 = bucket_max[bo + 1];
          if (bucket_max[bo + 2] > lz1) lz1 = bucket_max[bo + 2];
          lc += bucket_count[s];
        }
        int rcs = right_count[s];
        if (lc == 0 || rcs == 0) continue;
        double cost = lc * surface_area(lx1 - lx0, ly1 - ly0, lz1 - lz0) + rcs * right_area[s];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = axis;
          best_split = s;
          best_origin = cmin;
          best_scale = to_bucket;
        }
      }
    }
    if (best_axis < 0) return -1;
    // bvh.ts:262-278: in-place partition, bucket <= best_split goes left.
    int64_t lo = start, hi = (int64_t)end - 1;
    while (lo <= hi) {
      size_t o = (size_t)order[lo] * 3;
      int b = bucket_of(pb.centroid[o + best_axis], best_origin, best_scale);
      if (b <= best_split) {
        lo++;
      } else {
        std::swap(order[lo], order[hi]);
        hi--;
      }
    }
    if (lo == (int64_t)start || lo == (int64_t)end) return -1;
    return lo;
  }

  // bvh.ts:284-296: stable sort along the widest centroid axis, split in half.
  int64_t median_split(uint32_t start, uint32_t end, double cminx, double cminy, double cminz,
                       double cmaxx, double cmaxy, double cmaxz) {
    double ex = cmaxx - cminx, ey = cmaxy - cminy, ez = cmaxz - cminz;
    int axis = ex >= ey && ex >= ez ? 0 : ey >= ez ? 1 : 2;
    const std::vector<double>& c = pb.centroid;
    std::stable_sort(order.begin() + start, order.begin() + end, [&](uint32_t a, uint32_t b) {
      return c[(size_t)a * 3 + axis] < c[(size_t)b * 3 + axis];
    });
    return (int64_t)((start + end) >> 1);
  }
};

// pack.ts:75-119
void write_material(std::vector<float>& out, size_t index, const Material& m) {
  size_t o = index * CT_MAT_STRIDE;
  for (int k = 0; k < CT_MAT_STRIDE; k++) out[o + k] = 0;
  out[o + 3] = (float)m.type;
  switch (m.type) {
    case CT_MAT_LAMBERTIAN:
      out[o] = (float)m.color.x;
      out[o + 1] = (float)m.color.y;
      out[o + 2] = (float)m.color.z;
      if (m.checker) {
        out[o + 5] = (float)m.checker_scale;
        out[o + 6] = 1;
        out[o + 8] = (float)m.color2.x;
        out[o + 9] = (float)m.color2.y;
        out[o + 10] = (float)m.color2.z;
      }
      break;
    default:  // metal (albedo, roughness), dielectric (tint, ior), emissive (colour, strength)
      out[o] = (float)m.color.x;
      out[o + 1] = (float)m.color.y;
      out[o + 2] = (float)m.color.z;
      out[o + 4] = (float)m.param;
      break;
  }
  V3 e;
  if (material_emission(m, &e)) {
    out[o + 12] = (float)e.x;
    out[o + 13] = (float)e.y;
    out[o + 14] = (float)e.z;
  }
}

}  // namespace

// pack.ts:131-223
Packed pack_scene(const Scene& scene) {
  const double PI = 3.14159265358979323846;
  uint32_t total = 0;
  for (const Shape& s : scene.shapes) total += primitive_count(s);
  std::vector<float> prims((size_t)std::max<uint32_t>(1, total) * CT_PRIM_STRIDE, 0.0f);
  std::vector<uint32_t> prim_object(std::max<uint32_t>(1, total), 0);
  PrimBounds pb;
  pb.count = total;
  pb.min.resize((size_t)total * 3);
  pb.max.resize((size_t)total * 3);
  pb.centroid.resize((size_t)total * 3);
  uint32_t p = 0;
  std::vector<Tri> tris;
  for (size_t obj = 0; obj < scene.shapes.size(); obj++) {
    const Shape& sh = scene.shapes[obj];
    if (sh.kind == SHAPE_SPHERE) {
      size_t o = (size_t)p * CT_PRIM_STRIDE;
      const V3& c = sh.a;
      double r = sh.radius;
      prims[o] = (float)c.x;
      prims[o + 1] = (float)c.y;
      prims[o + 2] = (float)c.z;
      prims[o + 3] = CT_PRIM_SPHERE;
      prims[o + 4] = (float)r;
      prims[o + 7] = (float)obj;
      prims[o + 11] = (float)(4 * PI * r * r);
      prim_object[p] = (uint32_t)obj;
      double rp = r + 1e-6 + std::fabs(r) * 1e-6;  // pack.ts:153
      set_prim_bounds(pb, p, c.x - rp, c.y - rp, c.z - rp, c.x + rp, c.y + rp, c.z + rp);
      p++;
      continue;
    }
    tris.clear();
    shape_triangles(sh, tris);
    for (const Tri& t : tris) {
      size_t o = (size_t)p * CT_PRIM_STRIDE;
      V3 n = triangle_normal(t);
      prims[o] = (float)t.a.x;
      prims[o + 1] = (float)t.a.y;
      prims[o + 2] = (float)t.a.z;
      prims[o + 3] = CT_PRIM_TRIANGLE;
      prims[o + 4] = (float)t.b.x;
      prims[o + 5] = (float)t.b.y;
      prims[o + 6] = (float)t.b.z;
      prims[o + 7] = (float)obj;
      prims[o + 8] = (float)t.c.x;
      prims[o + 9] = (float)t.c.y;
      prims[o + 10] = (float)t.c.z;
      prims[o + 11] = (float)triangle_area(t);
      prims[o + 12] = (float)n.x;
      prims[o + 13] = (float)n.y;
      prims[o + 14] = (float)n.z;
      prim_object[p] = (uint32_t)obj;
      const double pad = 1e-6;
      set_prim_bounds(pb, p, std::min(std::min(t.a.x, t.b.x), t.c.x) - pad,
                      std::min(std::min(t.a.y, t.b.y), t.c.y) - pad,
                      std::min(std::min(t.a.z, t.b.z), t.c.z) - pad,
                      std::max(std::max(t.a.x, t.b.x), t.c.x) + pad,
                      std::max(std::max(t.a.y, t.b.y), t.c.y) + pad,
                      std::max(std::max(t.a.z, t.b.z), t.c.z) + pad);
      p++;
    }
  }
  Builder builder(pb);
  builder.build();

  Packed out;
  out.prim_count = total;
  out.prims.assign((size_t)std::max<uint32_t>(1, total) * CT_PRIM_STRIDE, 0.0f);
  out.prim_object.assign(std::max<uint32_t>(1, total), 0);
  for (uint32_t i = 0; i < total; i++) {
    uint32_t src = builder.order[i];
    std::copy(prims.begin() + (size_t)src * CT_PRIM_STRIDE,
              prims.begin() + (size_t)(src + 1) * CT_PRIM_STRIDE,
              out.prims.begin() + (size_t)i * CT_PRIM_STRIDE);
    out.prim_object[i] = prim_object[src];
  }
  out.nodes = std::move(builder.nodes);
  out.node_count = builder.node_count;
  out.order = std::move(builder.order);
  size_t nobj = scene.materials.size();
  out.mats.assign(std::max<size_t>(1, nobj) * CT_MAT_STRIDE, 0.0f);
  for (size_t i = 0; i < nobj; i++) write_material(out.mats, i, scene.materials[i]);
  out.mat_count = (uint32_t)nobj;
  V3 e;
  for (uint32_t i = 0; i < total; i++)
    if (material_emission(scene.materials[out.prim_object[i]], &e)) out.lights.push_back((int32_t)i);
  out.sky = scene.sky;
  return out;
}

// bvh.ts:319-381
BvhReport validate_bvh(const float* n, uint32_t node_count, const uint32_t* order,
                       uint32_t order_len, uint32_t prim_count) {
  BvhReport r{true, 0, 0, 0, 0};
  std::vector<uint8_t> covered(prim_count, 0);
  // Iterative post-order walk mirroring the recursive `walk` closure.
  struct Frame {
    uint32_t index, depth, stage, after_left;
  };
  std::vector<Frame> st;
  uint32_t ret = 0;
  st.push_back({0, 1, 0, 0});
  while (!st.empty()) {
    Frame& f = st.back();
    if (f.stage == 0) {
      if (f.depth > r.depth) r.depth = f.depth;
      if (f.index >= node_count) {
        r.errors++;
        ret = f.index + 1;
        st.pop_back();
        continue;
      }
      size_t base = (size_t)f.index * CT_NODE_STRIDE;
      double skip = n[base + 3], leaf = n[base + 7];
      if (leaf >= 0) {
        uint32_t start = (uint32_t)std::floor(leaf / 8);
        uint32_t count = (uint32_t)(leaf - std::floor(leaf / 8) * 8);
        r.leaf_count++;
        if (count > r.max_leaf_size) r.max_leaf_size = count;
        if (count > CT_MAX_LEAF_PRIMS) r.errors++;
        for (uint32_t i = start; i < start + count; i++) {
          if (i >= order_len) {
            r.errors++;
            continue;
          }
          uint32_t orig = order[i];
          if (orig < prim_count) {
            if (covered[orig]) r.errors++;
            covered[orig] = 1;
          }
        }
        if (skip != (double)f.index + 1) r.errors++;
        ret = f.index + 1;
        st.pop_back();
        continue;
      }
      f.stage = 1;
      uint32_t child = f.index + 1, d = f.depth + 1;
      st.push_back({child, d, 0, 0});
      continue;
    }
    if (f.stage == 1) {
      f.after_left = ret;
      f.stage = 2;
      uint32_t child = ret, d = f.depth + 1;
      st.push_back({child, d, 0, 0});
      continue;
    }
    // stage 2: both children done
    uint32_t after_right = ret;
    size_t base = (size_t)f.index * CT_NODE_STRIDE;
    if ((double)n[base + 3] != (double)after_right) r.errors++;
    uint32_t kids[2] = {f.index + 1, f.after_left};
    for (uint32_t child : kids) {
      if (child >= node_count) continue;
      size_t cb = (size_t)child * CT_NODE_STRIDE;
      for (int k = 0; k < 3; k++) {
        if (n[cb + k] < n[base + k] - 1e-6 || n[cb + 4 + k] > n[base + 4 + k] + 1e-6) {
          r.errors++;
          break;
        }
      }
    }
    ret = after_right;
    st.pop_back();
  }
  if (ret != node_count) r.errors++;
  if (prim_count > 0)
    for (uint32_t i = 0; i < prim_count; i++)
      if (!covered[i]) {
        r.errors++;
        break;
      }
  r.ok = r.errors == 0;
  return r;
}

}  // namespace oracle
