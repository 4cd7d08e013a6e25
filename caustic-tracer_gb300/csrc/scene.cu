// ct_scene_create / ct_scene_destroy: upload of a PackedScene (pack.ts:46-59).
//
// The host validates every index the kernels will follow (skip links, leaf
// ranges, light and material indices) before anything reaches the device,
// so a malformed array is rejected with CT_ERR_INVALID_ARGUMENT instead of
// becoming an out-of-bounds read. It also derives the traversal layout the
// ordered walk uses: the binary tree collapsed into 4-wide records of 128
// bytes (four child boxes by axis plus four child references), so one step
// of the walk tests four boxes with one cache line of loads and a ray takes
// about half the dependent steps of the binary walk.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <thread>
#include <vector>

#include <cuda_fp16.h>

#include "scene.hpp"

namespace ct {

ct_status DeviceBuffer::reserve(size_t want, size_t* total_bytes, int device, cudaStream_t stream) {
  if (want <= bytes) return CT_OK;
  release(total_bytes, stream);
  size_t grow = want + want / 4;
  if (path_alloc(device, grow, stream, &ptr) != CT_OK) {
    grow = want;
    ct_status st = path_alloc(device, grow, stream, &ptr);
    if (st != CT_OK) return st;
  }
  bytes = grow;
  if (total_bytes) *total_bytes += grow;
  return CT_OK;
}

void DeviceBuffer::release(size_t* total_bytes, cudaStream_t stream) {
  if (ptr) {
    path_free(ptr, stream);
    if (total_bytes) *total_bytes -= bytes;
  }
  ptr = nullptr;
  bytes = 0;
}

namespace {
std::mutex g_pool_mu;
constexpr int kPoolDevices = 64;
cudaMemPool_t g_pool[kPoolDevices] = {};

// Idle scene streams and their timing events, kept per device so that scene
// create and destroy do not pay for stream and event creation each time.
struct StreamSet {
  cudaStream_t stream;
  cudaEvent_t ev0, ev1, ev2;
};
constexpr size_t kIdleStreams = 32;
std::vector<StreamSet> g_idle[kPoolDevices];
}  // namespace

ct_status path_pool(int device, cudaMemPool_t* out) {
  CT_CHECK_ARG(device >= 0 && device < kPoolDevices, "device %d outside [0, %d)", device, kPoolDevices);
  std::lock_guard<std::mutex> guard(g_pool_mu);
  if (!g_pool[device]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    CT_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = ~0ull;  // freed blocks stay in the pool for the next render
    cudaError_t err = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (err != cudaSuccess) {
      cudaMemPoolDestroy(pool);
      return fail(CT_ERR_CUDA, "cudaMemPoolSetAttribute: %s", cudaGetErrorString(err));
    }
    g_pool[device] = pool;
  }
  *out = g_pool[device];
  return CT_OK;
}

ct_status path_alloc(int device, size_t bytes, cudaStream_t s, void** out) {
  *out = nullptr;
  cudaMemPool_t pool = nullptr;
  ct_status st = path_pool(device, &pool);
  if (st != CT_OK) return st;
  const cudaError_t err = cudaMallocFromPoolAsync(out, bytes, pool, s);
  if (err != cudaSuccess) {
    *out = nullptr;
    (void)cudaGetLastError();
    return fail(CT_ERR_OUT_OF_MEMORY, "path state of %zu bytes: %s", bytes, cudaGetErrorString(err));
  }
  return CT_OK;
}

void path_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

namespace {

bool is_index(float f, uint32_t limit) {
  return f >= 0.0f && f < (float)limit && std::floor(f) == f;
}

// Structural check of the skip-link array (bvh.ts:319-381 invariants that the
// traversals rely on) plus the depth and the number of interior nodes.
ct_status check_tree(const ct_packed_scene_view& v, uint32_t* interior_count, uint32_t* depth_out) {
  const float* n = v.nodes;
  const uint32_t N = v.node_count;
  uint32_t interior = 0, depth = 0;
  // Explicit post-order walk: frame = (node, depth, stage, end of left subtree).
  struct F {
    uint32_t node, depth, stage, after_left;
  };
  std::vector<F> st;
  st.push_back({0, 1, 0, 0});
  uint32_t ret = 0;
  while (!st.empty()) {
    F& f = st.back();
    const float* r = n + (size_t)f.node * CT_NODE_STRIDE;
    if (f.stage == 0) {
      if (f.node >= N) return fail(CT_ERR_INVALID_ARGUMENT, "node index %u out of range", f.node);
      if (f.depth > depth) depth = f.depth;
      if (f.depth > N) return fail(CT_ERR_INVALID_ARGUMENT, "node links form a cycle");
      if (r[7] >= 0.0f) {
        if (!is_index(r[7], 1u << 24)) return fail(CT_ERR_INVALID_ARGUMENT, "node %u: bad leaf word", f.node);
        const uint32_t word = (uint32_t)r[7], start = word >> 3, count = word & 7u;
        if ((uint64_t)start + count > v.prim_count)
          return fail(CT_ERR_INVALID_ARGUMENT, "node %u: leaf [%u, %u) beyond %u primitives", f.node, start,
                      start + count, v.prim_count);
        if (r[3] != (float)(f.node + 1)) return fail(CT_ERR_INVALID_ARGUMENT, "leaf %u: skip link is not %u", f.node, f.node + 1);
        ret = f.node + 1;
        st.pop_back();
        continue;
      }
      interior++;
      f.stage = 1;
      const uint32_t child = f.node + 1, d = f.depth + 1;
      st.push_back({child, d, 0, 0});
      continue;
    }
    if (f.stage == 1) {
      f.after_left = ret;
      const float* left = n + (size_t)(f.node + 1) * CT_NODE_STRIDE;
      if (left[3] != (float)ret) return fail(CT_ERR_INVALID_ARGUMENT, "node %u: skip link does not end its subtree", f.node + 1);
      f.stage = 2;
      const uint32_t child = ret, d = f.depth + 1;
      st.push_back({child, d, 0, 0});
      continue;
    }
    if (r[3] != (float)ret) return fail(CT_ERR_INVALID_ARGUMENT, "node %u: skip link does not end its subtree", f.node);
    st.pop_back();
  }
  if (ret != N) return fail(CT_ERR_INVALID_ARGUMENT, "tree covers %u of %u nodes", ret, N);
  *interior_count = interior;
  *depth_out = depth;
  return CT_OK;
}

// Collapses the reference's binary tree (bvh.ts node array) into the 4-wide
// records the ordered walk traverses: a record starts from a binary interior
// node and opens its largest-area interior child until it holds four children
// or only leaves. Record layout, 8 float4 = 128 bytes (one cache line):
//   [0] lo.x  [1] hi.x  [2] lo.y  [3] hi.y  [4] lo.z  [5] hi.z   (children 0..3)
//   [6] child references: >= 0 record, < 0 ~leafword            [7] unused
// Empty slots hold NaN bounds, which no box test accepts. The child boxes are
// the reference's own node boxes, so every box the walk tests is one the
// reference tests. *stack_need is the deepest stack the ordered walk can
// build: along the worst root-to-leaf path, each record pushes all but one
// of its children.
void build_quads(const ct_packed_scene_view& v, std::vector<float4>& recs, int32_t* root_ref,
                 uint32_t* stack_need) {
  const float* n = v.nodes;
  auto node = [&](uint32_t i) { return n + (size_t)i * CT_NODE_STRIDE; };
  auto leaf = [&](uint32_t i) { return node(i)[7] >= 0.0f; };
  auto right = [&](uint32_t i) { return (uint32_t)node(i + 1)[3]; };  // the left child's skip link
  auto area = [&](uint32_t i) {
    const float* r = node(i);
    const double dx = (double)r[4] - r[0], dy = (double)r[5] - r[1], dz = (double)r[6] - r[2];
    return dx * dy + dy * dz + dz * dx;
  };
  recs.assign(8, make_float4(0, 0, 0, 0));
  *stack_need = 0;
  if (v.node_count == 0 || leaf(0)) {
    *root_ref = v.node_count ? ~(int32_t)(uint32_t)node(0)[7] : ~0;
    return;
  }
  *root_ref = 0;
  // A record takes at least one binary interior node (its own), so there are
  // at most as many records as interior nodes: reserving that much keeps the
  // arrays from being copied as they grow (caustic scene, measured on an
  // x86 host: 10.3 -> 7.6 ms).
  const size_t max_records = std::max<size_t>(1, ((size_t)v.node_count - 1) / 2);
  recs.reserve(max_records * 8);
  std::vector<uint8_t> count_of;       // per record: children
  count_of.reserve(max_records);
  count_of.assign(1, 0);
  std::vector<std::pair<uint32_t, uint32_t>> todo{{0u, 0u}};  // (binary interior node, record)
  while (!todo.empty()) {
    const auto [b, r] = todo.back();
    todo.pop_back();
    uint32_t kids[4] = {b + 1, right(b), 0, 0};
    int k = 2;
    while (k < 4) {
      int best = -1;
      double best_area = -1.0;
      for (int c = 0; c < k; c++)
        if (!leaf(kids[c]) && area(kids[c]) > best_area) best = c, best_area = area(kids[c]);
      if (best < 0) break;
      const uint32_t x = kids[best];
      kids[best] = x + 1;
      kids[k++] = right(x);
    }
    const float nan = std::numeric_limits<float>::quiet_NaN();
    float lo[3][4], hi[3][4];
    int32_t refs[4] = {0, 0, 0, 0};
    for (int c = 0; c < 4; c++) {
      for (int a = 0; a < 3; a++) lo[a][c] = hi[a][c] = nan;
      if (c >= k) continue;
      const float* cn = node(kids[c]);
      for (int a = 0; a < 3; a++) lo[a][c] = cn[a], hi[a][c] = cn[4 + a];
      if (leaf(kids[c])) {
        refs[c] = ~(int32_t)(uint32_t)cn[7];
      } else {
        const uint32_t child = (uint32_t)(recs.size() / 8);
        recs.resize(recs.size() + 8, make_float4(0, 0, 0, 0));
        count_of.push_back(0);
        refs[c] = (int32_t)child;
        todo.push_back({kids[c], child});
      }
    }
    float4* q = &recs[(size_t)r * 8];
    for (int a = 0; a < 3; a++) {
      q[2 * a] = make_float4(lo[a][0], lo[a][1], lo[a][2], lo[a][3]);
      q[2 * a + 1] = make_float4(hi[a][0], hi[a][1], hi[a][2], hi[a][3]);
    }
    std::memcpy(&q[6], refs, sizeof refs);
    count_of[r] = (uint8_t)k;
  }
  // Children are numbered after their parents: one backward sweep gives the
  // worst stack below each record.
  const size_t R = recs.size() / 8;
  std::vector<uint32_t> need(R, 0);
  for (size_t r = R; r-- > 0;) {
    int32_t refs[4];
    std::memcpy(refs, &recs[r * 8 + 6], sizeof refs);
    uint32_t below = 0;
    for (int c = 0; c < count_of[r]; c++)
      if (refs[c] >= 0) below = std::max(below, need[(size_t)refs[c]]);
    need[r] = (uint32_t)(count_of[r] - 1) + below;
  }
  *stack_need = need[0];
}

// The records as the walk reads them, 64 bytes each: the six bound arrays as
// IEEE half floats, lower bounds rounded down and upper bounds rounded up
// (each box only grows, so no box the reference enters is missed; empty slots
// stay NaN), then the four child references:
//   [0] lo.x[0..3] hi.x[0..3]  [1] lo.y hi.y  [2] lo.z hi.z  (half2 pairs)  [3] refs
std::vector<uint4> half_records(const std::vector<float4>& recs) {
  const size_t R = recs.size() / 8;
  std::vector<uint4> out(R * 4);
  auto pair = [](float a, float b, bool up) {
    const __half ha = up ? __float2half_ru(a) : __float2half_rd(a);
    const __half hb = up ? __float2half_ru(b) : __float2half_rd(b);
    return (uint32_t)__half_as_ushort(ha) | ((uint32_t)__half_as_ushort(hb) << 16);
  };
  auto range = [&](size_t r0, size_t r1) {
    for (size_t r = r0; r < r1; r++) {
      const float4* q = &recs[r * 8];
      for (int a = 0; a < 3; a++) {
        const float4 lo = q[2 * a], hi = q[2 * a + 1];
        out[r * 4 + a] = make_uint4(pair(lo.x, lo.y, false), pair(lo.z, lo.w, false), pair(hi.x, hi.y, true),
                                    pair(hi.z, hi.w, true));
      }
      std::memcpy(&out[r * 4 + 3], &q[6], sizeof(uint4));
    }
  };
  // Large trees: four threads, each a contiguous quarter of the records.
  constexpr size_t kThreadedRecords = 16384;
  std::thread parts[3];
  size_t done = 0;
  if (R >= kThreadedRecords) {
    const size_t q = R / 4;
    try {
      for (int i = 0; i < 3; i++) {
        parts[i] = std::thread(range, (size_t)i * q, (size_t)(i + 1) * q);
        done = (size_t)(i + 1) * q;
      }
    } catch (const std::exception&) {  // no more threads: this thread takes the rest
    }
  }
  range(done, R);
  for (std::thread& t : parts)
    if (t.joinable()) t.join();
  return out;
}

// The arrays are present and their counts within the encodings' limits.
ct_status validate_pointers(const ct_packed_scene_view& v) {
  CT_CHECK_ARG(v.node_count == 0 || v.nodes != nullptr, "nodes is NULL");
  CT_CHECK_ARG(v.prim_count == 0 || v.prims != nullptr, "prims is NULL");
  CT_CHECK_ARG(v.prim_count == 0 || v.prim_object != nullptr, "prim_object is NULL");
  CT_CHECK_ARG(v.light_count == 0 || v.lights != nullptr, "lights is NULL");
  CT_CHECK_ARG(v.mats != nullptr || v.prim_count == 0, "mats is NULL");
  CT_CHECK_ARG(v.prim_count < (1u << 21), "prim_count %u exceeds the float32 leaf encoding", v.prim_count);
  CT_CHECK_ARG(v.node_count < (1u << 24), "node_count %u exceeds the float32 skip encoding", v.node_count);
  return CT_OK;
}

// The values of the node, primitive, material and light arrays and the sky
// (the tree's links are checked by check_tree).
ct_status validate_view(const ct_packed_scene_view& v) {
  for (size_t i = 0; i < (size_t)v.node_count * CT_NODE_STRIDE; i++)
    if (!std::isfinite(v.nodes[i])) return fail(CT_ERR_INVALID_ARGUMENT, "nodes[%zu] is not finite", i);
  const uint32_t mat_records = v.mat_count > 0 ? v.mat_count : 1;
  for (uint32_t p = 0; p < v.prim_count; p++) {
    const float* q = v.prims + (size_t)p * CT_PRIM_STRIDE;
    for (int k = 0; k < CT_PRIM_STRIDE; k++)
      if (!std::isfinite(q[k])) return fail(CT_ERR_INVALID_ARGUMENT, "prims[%u] has a non-finite value", p);
    if (q[3] != CT_PRIM_SPHERE && q[3] != CT_PRIM_TRIANGLE)
      return fail(CT_ERR_INVALID_ARGUMENT, "prims[%u]: unknown type %g", p, (double)q[3]);
    if (v.prim_object[p] >= mat_records)
      return fail(CT_ERR_INVALID_ARGUMENT, "prim_object[%u] = %u beyond %u materials", p, v.prim_object[p], mat_records);
  }
  for (uint32_t m = 0; m < v.mat_count; m++) {
    const float* q = v.mats + (size_t)m * CT_MAT_STRIDE;
    for (int k = 0; k < CT_MAT_STRIDE; k++)
      if (!std::isfinite(q[k])) return fail(CT_ERR_INVALID_ARGUMENT, "mats[%u] has a non-finite value", m);
    if (!(q[3] == 0 || q[3] == 1 || q[3] == 2 || q[3] == 3))
      return fail(CT_ERR_INVALID_ARGUMENT, "mats[%u]: unknown type %g", m, (double)q[3]);
  }
  for (uint32_t l = 0; l < v.light_count; l++)
    if (v.lights[l] < 0 || (uint32_t)v.lights[l] >= v.prim_count)
      return fail(CT_ERR_INVALID_ARGUMENT, "lights[%u] = %d beyond %u primitives", l, v.lights[l], v.prim_count);
  CT_CHECK_ARG(v.sky.kind == 0 || v.sky.kind == 1, "sky.kind %d is not 0 or 1", v.sky.kind);
  return CT_OK;
}

// tris[3p + k] = prims[4p + k], k < 3: the vertices (or a sphere's centre and
// radius) of each primitive without its fourth record, for the exact tests.
__global__ void k_compact_prims(const float4* __restrict__ prims, uint32_t n, float4* __restrict__ tris) {
  const size_t total = (size_t)n * 3, stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += stride) {
    const size_t p = i / 3;
    tris[i] = __ldg(prims + p * 4 + (i - p * 3));
  }
}

// Plane records of the integrator's float32 triangle test, 48 bytes per
// primitive (Havel and Herout, "Yet Faster Ray-Triangle Intersection (Using
// SSE4)", IEEE TVCG 16(3), 2010). For a triangle (a, b, c) with
// n = (b-a) x (c-a): [n, n.a | n1, -n1.a | n2, -n2.a] with
// n1 = ((c-a) x n)/|n|^2 and n2 = (n x (b-a))/|n|^2, computed in float64
// with every operation rounded separately (no fused multiply-adds) and
// rounded once to float32; a sphere stores its centre and radius and a NaN
// marker; a degenerate triangle stores zeros. Built on the device from the
// uploaded primitives, one thread per primitive, so the host neither
// computes nor uploads them.
__global__ void k_plane_records(const float4* __restrict__ prims, uint32_t n, float4* __restrict__ planes) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += stride) {
    const float4 q0 = prims[p * 4], q1 = prims[p * 4 + 1], q2 = prims[p * 4 + 2];
    float4* o = planes + p * 3;
    if (q0.w == (float)CT_PRIM_SPHERE) {
      o[0] = make_float4(q0.x, q0.y, q0.z, q1.x);
      o[1] = make_float4(__int_as_float(0x7fc00000), 0.0f, 0.0f, 0.0f);
      o[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      continue;
    }
    auto sub = [](double x, double y) { return __dsub_rn(x, y); };
    auto mul = [](double x, double y) { return __dmul_rn(x, y); };
    auto add = [](double x, double y) { return __dadd_rn(x, y); };
    const double a[3] = {q0.x, q0.y, q0.z};
    const double e1[3] = {sub(q1.x, a[0]), sub(q1.y, a[1]), sub(q1.z, a[2])};
    const double e2[3] = {sub(q2.x, a[0]), sub(q2.y, a[1]), sub(q2.z, a[2])};
    auto cross = [&](const double* x, const double* y, double* z) {
      z[0] = sub(mul(x[1], y[2]), mul(x[2], y[1]));
      z[1] = sub(mul(x[2], y[0]), mul(x[0], y[2]));
      z[2] = sub(mul(x[0], y[1]), mul(x[1], y[0]));
    };
    auto dot = [&](const double* x, const double* y) {
      return add(add(mul(x[0], y[0]), mul(x[1], y[1])), mul(x[2], y[2]));
    };
    double nn[3], n1[3], n2[3];
    cross(e1, e2, nn);
    const double l2 = dot(nn, nn);
    if (!(l2 > 0.0) || !isfinite(l2)) {
      o[0] = o[1] = o[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      continue;
    }
    cross(e2, nn, n1);
    cross(nn, e1, n2);
    for (int k = 0; k < 3; k++) n1[k] = __ddiv_rn(n1[k], l2), n2[k] = __ddiv_rn(n2[k], l2);
    o[0] = make_float4((float)nn[0], (float)nn[1], (float)nn[2], (float)dot(nn, a));
    o[1] = make_float4((float)n1[0], (float)n1[1], (float)n1[2], (float)-dot(n1, a));
    o[2] = make_float4((float)n2[0], (float)n2[1], (float)n2[2], (float)-dot(n2, a));
  }
}

// The scene's arrays share one allocation from the per-device stream-ordered
// pool (scene create and destroy then cost no cudaMalloc / cudaFree, and the
// latter would wait for the whole device).
size_t arena_slot(size_t bytes) { return (bytes + 255) & ~size_t(255); }

template <class T>
ct_status upload(ct_scene* s, DeviceBuffer& b, char*& cursor, const T* src, size_t count, size_t min_count) {
  const size_t n = count > min_count ? count : min_count;
  b.ptr = cursor;
  b.bytes = n * sizeof(T);
  cursor += arena_slot(b.bytes);
  if (n > count)  // only the padding past the copied elements starts at zero
    CT_CUDA(cudaMemsetAsync(static_cast<char*>(b.ptr) + count * sizeof(T), 0, (n - count) * sizeof(T), s->stream));
  if (count) CT_CUDA(cudaMemcpyAsync(b.ptr, src, count * sizeof(T), cudaMemcpyHostToDevice, s->stream));
  return CT_OK;
}

// A slot of the arena that a kernel fills (no host copy).
ct_status carve(ct_scene*, DeviceBuffer& b, char*& cursor, size_t bytes) {
  b.ptr = cursor;
  b.bytes = bytes;
  cursor += arena_slot(bytes);
  return CT_OK;
}

void destroy(ct_scene* s) {
  if (!s) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (DeviceBuffer* b : {&s->prims, &s->nodes, &s->quads, &s->mats, &s->lights, &s->prim_object, &s->planes,
                          &s->tris, &s->counters})
    b->ptr = nullptr, b->bytes = 0;  // slices of the arena
  if (s->arena) path_free(s->arena, s->stream);
  s->io.release(&s->device_bytes, s->stream);
  for (cudaStream_t c : {s->copy_in, s->copy_out, s->compute2})
    if (c) cudaStreamSynchronize(c), cudaStreamDestroy(c);
  for (cudaStream_t c : s->render_side)
    if (c) cudaStreamSynchronize(c), cudaStreamDestroy(c);
  for (cudaEvent_t e : {s->ev_in, s->ev_done, s->render_fork})
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : s->render_join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : s->render_acc)
    if (e) cudaEventDestroy(e);
  bool kept = false;
  if (s->stream && s->ev0 && s->ev1 && s->ev2 && s->device >= 0 && s->device < kPoolDevices &&
      cudaStreamSynchronize(s->stream) == cudaSuccess) {
    std::lock_guard<std::mutex> guard(g_pool_mu);
    std::vector<StreamSet>& idle = g_idle[s->device];
    if (idle.size() < kIdleStreams) {
      try {
        idle.push_back({s->stream, s->ev0, s->ev1, s->ev2});
        kept = true;
      } catch (const std::bad_alloc&) {
      }
    }
  }
  if (!kept) {
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->ev2) cudaEventDestroy(s->ev2);
    if (s->stream) cudaStreamDestroy(s->stream);
  }
  cudaSetDevice(prev);
  delete s;
}

// Scenes of at least this many primitives run the value checks on a separate
// thread, beside the tree check and record build (caustic scene, 327,746
// primitives; below this size the thread costs more than it saves).
constexpr uint32_t kThreadedPrims = 50000;

ct_status create(const ct_packed_scene_view& v, ct_scene** out) {
  ct_status st = validate_pointers(v);
  if (st != CT_OK) return st;
  // The value checks read only the primitive, material and light arrays, so
  // they run beside the tree check, the record build and the half records
  // (which follow the check). The plane records and the compact triangles
  // are built on the device from the uploaded primitives.
  const bool threaded = v.prim_count >= kThreadedPrims;
  ct_status values = CT_OK;
  std::thread t_values;
  if (threaded) {
    try {
      t_values = std::thread([&] { values = validate_view(v); });
    } catch (const std::exception&) {  // no thread: the checks run on this thread below
    }
  }
  struct Joiner {  // every return below joins the worker thread first
    std::thread& a;
    ~Joiner() {
      if (a.joinable()) a.join();
    }
  } joiner{t_values};
  if (!t_values.joinable()) {
    st = validate_view(v);
    if (st != CT_OK) return st;
  }
  uint32_t interior = 0, depth = 0;
  if (v.node_count > 0) {
    st = check_tree(v, &interior, &depth);
    if (st != CT_OK) return st;
  }
  std::vector<float4> quads;
  int32_t root_ref = ~0;
  uint32_t stack_need = 0;
  std::vector<uint4> halves;
  try {
    build_quads(v, quads, &root_ref, &stack_need);
    halves = half_records(quads);
  } catch (const std::bad_alloc&) {
    return fail(CT_ERR_OUT_OF_MEMORY, "ct_scene_create: host allocation failed");
  }
  if (t_values.joinable()) {
    t_values.join();
    // the error message belongs to the calling thread: run the check again here
    if (values != CT_OK) return validate_view(v);
  }

  ct_scene* s = new (std::nothrow) ct_scene();
  if (!s) return fail(CT_ERR_OUT_OF_MEMORY, "ct_scene_create: host allocation failed");
  cudaGetDevice(&s->device);
  auto bail = [&](ct_status code) {
    destroy(s);
    return code;
  };
  if (s->device >= 0 && s->device < kPoolDevices) {
    std::lock_guard<std::mutex> guard(g_pool_mu);
    std::vector<StreamSet>& idle = g_idle[s->device];
    if (!idle.empty()) {
      const StreamSet set = idle.back();
      idle.pop_back();
      s->stream = set.stream, s->ev0 = set.ev0, s->ev1 = set.ev1, s->ev2 = set.ev2;
    }
  }
  if (!s->stream) {
    cudaError_t err = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (err != cudaSuccess) {
      s->stream = nullptr;
      return bail(fail(CT_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(err)));
    }
    if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess ||
        cudaEventCreate(&s->ev2) != cudaSuccess)
      return bail(fail(CT_ERR_CUDA, "cudaEventCreate failed"));
  }
  s->prim_count = v.prim_count;
  s->node_count = v.node_count;
  s->interior_count = interior;
  s->mat_count = v.mat_count;
  s->light_count = v.light_count;
  s->depth = depth;
  s->stack_need = stack_need;
  s->sky = v.sky;
  const size_t arena = arena_slot(std::max<size_t>(v.prim_count * 4, 4) * sizeof(float4)) +
                       arena_slot(std::max<size_t>(v.node_count * 2, 2) * sizeof(float4)) +
                       arena_slot(std::max<size_t>(halves.size(), 4) * sizeof(uint4)) +
                       arena_slot(std::max<size_t>(v.mat_count * 4, 4) * sizeof(float4)) +
                       arena_slot(std::max<size_t>(v.light_count, 1) * sizeof(int32_t)) +
                       arena_slot(std::max<size_t>(v.prim_count, 1) * sizeof(uint32_t)) +
                       arena_slot(std::max<size_t>((size_t)v.prim_count * 3, 3) * sizeof(float4)) +
                       arena_slot(std::max<size_t>((size_t)v.prim_count * 3, 3) * sizeof(float4)) +
                       arena_slot(kCounterWords * sizeof(uint32_t));
  if ((st = path_alloc(s->device, arena, s->stream, &s->arena)) != CT_OK) return bail(st);
  s->device_bytes += arena;
  char* cursor = static_cast<char*>(s->arena);
  if ((st = upload(s, s->prims, cursor, reinterpret_cast<const float4*>(v.prims), (size_t)v.prim_count * 4, 4)) != CT_OK ||
      (st = upload(s, s->nodes, cursor, reinterpret_cast<const float4*>(v.nodes), (size_t)v.node_count * 2, 2)) != CT_OK ||
      (st = upload(s, s->quads, cursor, halves.data(), halves.size(), 4)) != CT_OK ||
      (st = upload(s, s->mats, cursor, reinterpret_cast<const float4*>(v.mats), (size_t)v.mat_count * 4, 4)) != CT_OK ||
      (st = upload(s, s->lights, cursor, v.lights, v.light_count, 1)) != CT_OK ||
      (st = upload(s, s->prim_object, cursor, v.prim_object, v.prim_count, 1)) != CT_OK ||
      (st = carve(s, s->planes, cursor, std::max<size_t>((size_t)v.prim_count * 3, 3) * sizeof(float4))) != CT_OK ||
      (st = carve(s, s->tris, cursor, std::max<size_t>((size_t)v.prim_count * 3, 3) * sizeof(float4))) != CT_OK ||
      (st = upload(s, s->counters, cursor, (const uint32_t*)nullptr, 0, kCounterWords)) != CT_OK)
    return bail(st);
  if (v.prim_count) {
    const size_t total = (size_t)v.prim_count * 3;
    const unsigned blocks = (unsigned)std::min<size_t>((total + 255) / 256, 4096);
    k_compact_prims<<<blocks, 256, 0, s->stream>>>(s->prims.as<float4>(), v.prim_count, s->tris.as<float4>());
    const unsigned plane_blocks = (unsigned)std::min<size_t>(((size_t)v.prim_count + 127) / 128, 4096);
    k_plane_records<<<plane_blocks, 128, 0, s->stream>>>(s->prims.as<float4>(), v.prim_count,
                                                         s->planes.as<float4>());
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return bail(fail(CT_ERR_CUDA, "scene records: %s", cudaGetErrorString(err)));
  } else {
    cudaError_t err = cudaMemsetAsync(s->tris.ptr, 0, s->tris.bytes, s->stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(s->planes.ptr, 0, s->planes.bytes, s->stream);
    if (err != cudaSuccess) return bail(fail(CT_ERR_CUDA, "scene upload: %s", cudaGetErrorString(err)));
  }
  if (v.mat_count == 0 && v.mats != nullptr) {
    // The reference always allocates one material record (pack.ts:122).
    cudaError_t err = cudaMemcpyAsync(s->mats.ptr, v.mats, CT_MAT_STRIDE * sizeof(float), cudaMemcpyHostToDevice, s->stream);
    if (err != cudaSuccess) return bail(fail(CT_ERR_CUDA, "material upload: %s", cudaGetErrorString(err)));
  }
  {
    cudaError_t err = cudaMemsetAsync(s->counters.ptr, 0, kCounterWords * sizeof(uint32_t), s->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s->stream);
    if (err != cudaSuccess) return bail(fail(CT_ERR_CUDA, "scene upload: %s", cudaGetErrorString(err)));
  }
  ctk::SceneDev& d = s->dev;
  d.prims = s->prims.as<float4>();
  d.nodes = s->nodes.as<float4>();
  d.quads = s->quads.as<uint4>();
  d.planes = s->planes.as<float4>();
  d.tris = s->tris.as<float4>();
  d.mats = s->mats.as<float4>();
  d.lights = s->lights.as<int32_t>();
  d.prim_object = s->prim_object.as<uint32_t>();
  d.prim_count = v.prim_count;
  d.node_count = v.node_count;
  d.light_count = v.light_count;
  if (v.node_count > 0) {
    d.root_ref = root_ref;
    for (int k = 0; k < 3; k++) {
      d.root_lo[k] = v.nodes[k];
      d.root_hi[k] = v.nodes[4 + k];
    }
  } else {
    d.root_ref = ~0;  // an empty leaf; the kernels skip scenes without nodes
  }
  *out = s;
  return CT_OK;
}

}  // namespace
}  // namespace ct

extern "C" {

ct_status ct_scene_create(const ct_packed_scene_view* ps, ct_scene** out) {
  ct::clear_error();
  CT_CHECK_ARG(ps != nullptr && out != nullptr, "ct_scene_create: NULL argument");
  *out = nullptr;
  try {
    return ct::create(*ps, out);
  } catch (const std::bad_alloc&) {
    return ct::fail(CT_ERR_OUT_OF_MEMORY, "ct_scene_create: host allocation failed");
  }
}

void ct_scene_destroy(ct_scene* scene) { ct::destroy(scene); }

uint64_t ct_scene_device_bytes(const ct_scene* scene) { return scene ? scene->device_bytes : 0; }

ct_status ct_scene_set_option(ct_scene* scene, int32_t option, int64_t value) {
  ct::clear_error();
  CT_CHECK_ARG(scene != nullptr, "scene is NULL");
  std::lock_guard<std::mutex> guard(scene->lock);
  switch (option) {
    case CT_OPT_WALK:
      CT_CHECK_ARG(value >= -1 && value <= 2, "CT_OPT_WALK %lld outside [-1, 2]", (long long)value);
      if (value == 0 || value == 1)
        CT_CHECK_ARG(scene->stack_need <= ctk::kStackSize, "the ordered walk of this tree needs %u stack entries (%d)",
                     scene->stack_need, ctk::kStackSize);
      scene->opt_walk = (int32_t)value;
      return CT_OK;
    case CT_OPT_WAVE_PATHS:
      CT_CHECK_ARG(value >= 0 && value <= (1ll << 30), "CT_OPT_WAVE_PATHS %lld outside [0, 2^30]", (long long)value);
      scene->opt_wave_paths = value;
      return CT_OK;
    case CT_OPT_TRACE_BLOCKS:
      CT_CHECK_ARG(value >= 0 && value <= 64, "CT_OPT_TRACE_BLOCKS %lld outside [0, 64]", (long long)value);
      scene->opt_trace_blocks = (int32_t)value;
      return CT_OK;
    case CT_OPT_PATH_KERNEL:
      CT_CHECK_ARG(value == 0 || value == 1, "CT_OPT_PATH_KERNEL %lld is not 0 or 1", (long long)value);
      scene->opt_path_kernel = value != 0;
      return CT_OK;
    default:
      return ct::fail(CT_ERR_INVALID_ARGUMENT, "unknown scene option %d", option);
  }
}

}  // extern "C"
