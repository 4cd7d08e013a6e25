// Batched ray queries: intersectClosest (intersect.ts:202-282) and occluded
// (intersect.ts:368-420) over device-resident scenes.
//
// The ordered walk runs as persistent warps sized to the resident capacity of
// the 152 SMs; lanes take rays from a work counter as their walks finish, so
// uneven walk lengths do not idle the rest of the warp. A ray is two float4
// loads (32 B). Closest hits whose float32 distance bound is loose are
// flagged and recomputed in float64 by a separate, converged pass.
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "profile.hpp"
#include "scene.hpp"

namespace ct {

namespace {

// 0 ordered walk (persistent lanes), 1 stackless skip links, 2 ordered walk one query per thread
std::atomic<int32_t> g_variant{0};

// 12 blocks of 128 per SM (40 registers, some spilled): the walk is a chain
// of dependent loads and gains from warps in flight, while fewer threads keep
// its local memory (state, stack) closer to L1 (1M-triangle soup: 837 Mrays/s
// against 834 at 16 blocks).
// BARY: barycentrics are returned (u_out, v_out); otherwise the walk does
// not carry them, which keeps two registers free per lane.
template <int VARIANT, bool ANY, bool BARY>
__global__ void __launch_bounds__(128, 12) k_trace(ctk::SceneDev s, const float4* __restrict__ rays,
                                               uint32_t n, int32_t* __restrict__ prim,
                                               float* __restrict__ t_out, float* __restrict__ u_out,
                                               float* __restrict__ v_out,
                                               uint8_t* __restrict__ blocked,
                                               uint32_t* __restrict__ counters, uint32_t* __restrict__ queue) {
  uint32_t fallbacks = 0;
  bool overflow = false;
  auto load = [&](uint32_t i, ctk::RayF& r) {
    // rays and hits are touched once: streaming loads and stores keep them
    // from evicting the tree's records from L1 (+0.4 %)
    const float4 r0 = __ldcs(rays + 2 * (size_t)i), r1 = __ldcs(rays + 2 * (size_t)i + 1);
    r = ctk::RayF{r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, 0.0f, 0.0f, 0.0f};
    ctk::finish_ray(r);
  };
  // A hit whose float32 distance bound exceeds kReportRel is stored with a
  // negative t; k_refine replaces it with the reference's float64 value.
  auto store = [&](uint32_t i, const ctk::RayF& r, ctk::HitF& h) {
    if (ANY) {
      blocked[i] = h.prim >= 0 ? 1 : 0;
    } else {
      __stcs(&prim[i], h.prim);
      float t = h.t;
      bool loose = h.err > ctk::kReportRel * h.t;
      // Without barycentrics, a loose triangle hit first tries the plane
      // distance (float32, bounded); k_refine takes what is still loose.
      if (!BARY && loose && h.prim >= 0 && ctk::plane_t(s, r, h.prim, ctk::kReportRel, t)) loose = false;
      __stcs(&t_out[i], h.prim < 0 ? INFINITY : (loose ? -h.t : t));
      if (BARY && u_out) u_out[i] = h.prim >= 0 ? h.u : 0.0f;
      if (BARY && v_out) v_out[i] = h.prim >= 0 ? h.v : 0.0f;
    }
  };
  if (VARIANT == 0) {
    ctk::walk_persistent<true, 5, false, 2, BARY && !ANY, ANY ? 1 : 0>(
        s, queue, n,
        [&](uint32_t i, ctk::Walk& w) {
          load(i, w.r);
          ctk::walk_begin(s, w, ANY);
        },
        [&](uint32_t i, ctk::Walk& w) {
          overflow |= w.overflow;
          store(i, w.r, w.h);
        },
        fallbacks);
  } else if (VARIANT == 2) {  // the ordered walk, one query per thread
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
      ctk::WalkFrame f;
      ctk::Walk& w = f.w;
      load(i, w.r);
      ctk::walk_begin(s, w, ANY);
      while (w.c.ref != ctk::kWalkDone) ctk::walk_step<true, BARY && !ANY, ANY ? 1 : 0>(s, w, f.st, fallbacks);
      overflow |= w.overflow;
      store(i, w.r, w.h);
    }
  } else {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
      ctk::RayF r;
      load(i, r);
      ctk::HitF h{-1, r.tmax, 0.0f, 0.0f, 0.0f};
      ctk::walk_stackless(s, r, h, ANY, fallbacks);
      store(i, r, h);
    }
  }
  if (fallbacks) atomicAdd(&counters[kCountFallbacks], fallbacks);
  if (overflow) atomicOr(&counters[kCountError], 1u);
}

// Recomputes the flagged (negative) distances of closest hits in float64, in
// the reference's operation order, with every lane of a warp in step.
__global__ void __launch_bounds__(256) k_refine(ctk::SceneDev s, const float4* __restrict__ rays, uint32_t n,
                                                const int32_t* __restrict__ prim, float* __restrict__ t_out,
                                                float* __restrict__ u_out, float* __restrict__ v_out) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (!(t_out[i] < 0.0f)) continue;
    const float4 r0 = __ldg(rays + 2 * (size_t)i), r1 = __ldg(rays + 2 * (size_t)i + 1);
    ctk::RayF r{r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, 0.0f, 0.0f, 0.0f};
    if (!u_out && !v_out) {  // only t is wanted: the plane distance in float64
      const double tp = ctk::plane_t64(s, r, prim[i]);
      if (tp > 0) {
        t_out[i] = (float)tp;
        continue;
      }
    }
    ctk::HitF h{prim[i], -t_out[i], 0.0f, 0.0f, 1.0f};
    if (u_out) h.u = u_out[i];
    if (v_out) h.v = v_out[i];
    ctk::refine_hit(s, r, h);
    t_out[i] = h.t;
    if (u_out) u_out[i] = h.u;
    if (v_out) v_out[i] = h.v;
  }
}

template <int VARIANT, bool ANY, bool BARY>
int grid_for(uint32_t n) {
  static int per_sm = -1, sms = 0;
  if (per_sm < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<VARIANT, ANY, BARY>, 128, 0);
    if (per_sm < 1) per_sm = 1;
  }
  const uint64_t need = ((uint64_t)n + 127) / 128;
  const uint64_t full = (uint64_t)sms * (uint64_t)per_sm;
  return (int)(need < full ? (need > 0 ? need : 1) : full);
}

// `slot` picks the persistent walk's work counter (two launches may run at
// once on two streams, each with its own).
template <bool ANY>
ct_status launch(ct_scene* s, const float* rays, uint32_t n, int32_t* prim, float* t, float* u,
                 float* v, uint8_t* blocked, cudaStream_t stream, int slot = 0) {
  if (n == 0) return CT_OK;
  // A tree whose walk could outgrow the ordered walk's stack uses the stackless walk.
  const int chosen = g_variant.load();
  const int variant = (chosen == 1 || s->stack_need > ctk::kStackSize) ? 1 : chosen;
  const float4* r4 = reinterpret_cast<const float4*>(rays);
  uint32_t* cnt = s->counters.as<uint32_t>();
  uint32_t* queue = cnt + kCountQueue + slot;
  CT_CUDA(cudaMemsetAsync(queue, 0, sizeof(uint32_t), stream));  // persistent work counter
  {
    ProfScope ps(ANY ? "occluded" : "closest", stream);
    auto go = [&](auto variant_c, auto bary_c) {
      constexpr int V = decltype(variant_c)::value;
      constexpr bool B = decltype(bary_c)::value;
      k_trace<V, ANY, B><<<grid_for<V, ANY, B>(n), 128, 0, stream>>>(s->dev, r4, n, prim, t, u, v, blocked, cnt,
                                                                   queue);
    };
    using B0 = std::integral_constant<bool, false>;
    using B1 = std::integral_constant<bool, true>;
    const bool bary = !ANY && (u || v);
    if (variant == 0)
      bary ? go(std::integral_constant<int, 0>{}, B1{}) : go(std::integral_constant<int, 0>{}, B0{});
    else if (variant == 2)
      bary ? go(std::integral_constant<int, 2>{}, B1{}) : go(std::integral_constant<int, 2>{}, B0{});
    else
      bary ? go(std::integral_constant<int, 1>{}, B1{}) : go(std::integral_constant<int, 1>{}, B0{});
  }
  CT_CUDA(cudaGetLastError());
  if (!ANY) {
    static int refine_grid = 0;
    if (!refine_grid) {
      int dev = 0, sms = 0, per_sm = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_refine, 256, 0);
      refine_grid = sms * (per_sm > 0 ? per_sm : 1);
    }
    ProfScope ps("refine", stream);
    const uint64_t need = ((uint64_t)n + 255) / 256;
    k_refine<<<(int)(need < (uint64_t)refine_grid ? need : refine_grid), 256, 0, stream>>>(s->dev, r4, n, prim, t,
                                                                                           u, v);
    CT_CUDA(cudaGetLastError());
  }
  return CT_OK;
}

// Rays per chunk of a pipelined host-pointer query (batches of at least two
// chunks are pipelined).
constexpr uint32_t kHostChunk = 1u << 22;

// Host-pointer query: stage the rays, run, copy the results back.
template <bool ANY>
ct_status host_query(ct_scene* s, const float* rays, uint32_t n, int32_t* prim, float* t, float* u,
                     float* v, uint8_t* blocked, ct_stats* stats) {
  CT_CHECK_ARG(s != nullptr, "scene is NULL");
  CT_CHECK_ARG(n == 0 || rays != nullptr, "rays is NULL");
  CT_CHECK_ARG(n == 0 || (ANY ? blocked != nullptr : (prim != nullptr && t != nullptr)), "output is NULL");
  std::lock_guard<std::mutex> guard(s->lock);
  CT_CUDA(cudaSetDevice(s->device));
  if (stats) std::memset(stats, 0, sizeof *stats);
  if (n == 0) return CT_OK;
  const size_t ray_bytes = (size_t)n * CT_RAY_FLOATS * sizeof(float);
  const size_t out_words = ANY ? ((size_t)n + 3) / 4 : (size_t)n * (2 + (u ? 1 : 0) + (v ? 1 : 0));
  ct_status st = s->io.reserve(ray_bytes + out_words * 4, &s->device_bytes, s->device, s->stream);
  if (st != CT_OK) return st;
  char* base = s->io.as<char>();
  float* d_rays = reinterpret_cast<float*>(base);
  char* o = base + ray_bytes;
  int32_t* d_prim = nullptr;
  float *d_t = nullptr, *d_u = nullptr, *d_v = nullptr;
  uint8_t* d_blocked = nullptr;
  if (ANY) {
    d_blocked = reinterpret_cast<uint8_t*>(o);
  } else {
    d_prim = reinterpret_cast<int32_t*>(o);
    d_t = reinterpret_cast<float*>(o) + n;
    size_t next = 2;
    if (u) d_u = reinterpret_cast<float*>(o) + (next++) * (size_t)n;
    if (v) d_v = reinterpret_cast<float*>(o) + (next++) * (size_t)n;
  }
  cudaStream_t stream = s->stream;
  // Large batches run in chunks: chunk k+1's rays go in on copy_in and chunk
  // k-1's results come out on copy_out while chunk k is traced, so the
  // copies hide behind the kernels (events order each chunk's copy in,
  // trace and copy out). Consecutive chunks alternate between two compute
  // streams (each with its own work counter), so a chunk's blocks start on
  // the SMs its predecessor's draining warps leave. A small batch is one
  // chunk on the scene stream.
  const uint32_t chunks = n >= 2 * kHostChunk ? (n + kHostChunk - 1) / kHostChunk : 1;
  cudaStream_t in = stream, out = stream;
  if (chunks > 1) {
    if (!s->copy_in) {
      for (cudaStream_t* c : {&s->copy_in, &s->copy_out, &s->compute2})
        CT_CUDA(cudaStreamCreateWithFlags(c, cudaStreamNonBlocking));
      for (cudaEvent_t* e : {&s->ev_in, &s->ev_done})
        CT_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    in = s->copy_in;
    out = s->copy_out;
  }
  CT_CUDA(cudaMemsetAsync(s->counters.ptr, 0, 2 * sizeof(uint32_t), stream));
  CT_CUDA(cudaEventRecord(s->ev0, stream));
  if (chunks > 1) {
    CT_CUDA(cudaStreamWaitEvent(in, s->ev0, 0));
    CT_CUDA(cudaStreamWaitEvent(s->compute2, s->ev0, 0));
  }
  for (uint32_t k = 0; k < chunks; k++) {
    const size_t first = (size_t)k * kHostChunk;
    const uint32_t m = chunks == 1 ? n : (uint32_t)std::min<size_t>(kHostChunk, n - first);
    const size_t rf = first * CT_RAY_FLOATS;
    CT_CUDA(cudaMemcpyAsync(d_rays + rf, rays + rf, (size_t)m * CT_RAY_FLOATS * sizeof(float),
                            cudaMemcpyHostToDevice, in));
    cudaStream_t compute = (k & 1) ? s->compute2 : stream;
    if (chunks > 1) {
      CT_CUDA(cudaEventRecord(s->ev_in, in));
      CT_CUDA(cudaStreamWaitEvent(compute, s->ev_in, 0));
    }
    if (k == 0) CT_CUDA(cudaEventRecord(s->ev1, stream));
    st = launch<ANY>(s, d_rays + rf, m, ANY ? nullptr : d_prim + first, ANY ? nullptr : d_t + first,
                     d_u ? d_u + first : nullptr, d_v ? d_v + first : nullptr, ANY ? d_blocked + first : nullptr,
                     compute, (int)(k & 1));
    if (st != CT_OK) return st;
    if (chunks > 1) {
      CT_CUDA(cudaEventRecord(s->ev_done, compute));
      CT_CUDA(cudaStreamWaitEvent(out, s->ev_done, 0));
    }
    if (ANY) {
      CT_CUDA(cudaMemcpyAsync(blocked + first, d_blocked + first, m, cudaMemcpyDeviceToHost, out));
    } else {
      CT_CUDA(cudaMemcpyAsync(prim + first, d_prim + first, (size_t)m * 4, cudaMemcpyDeviceToHost, out));
      CT_CUDA(cudaMemcpyAsync(t + first, d_t + first, (size_t)m * 4, cudaMemcpyDeviceToHost, out));
      if (u) CT_CUDA(cudaMemcpyAsync(u + first, d_u + first, (size_t)m * 4, cudaMemcpyDeviceToHost, out));
      if (v) CT_CUDA(cudaMemcpyAsync(v + first, d_v + first, (size_t)m * 4, cudaMemcpyDeviceToHost, out));
    }
  }
  CT_CUDA(cudaEventRecord(s->ev2, out));  // after every chunk's trace (out has waited for each)
  uint32_t counters[2] = {0, 0};
  CT_CUDA(cudaMemcpyAsync(counters, s->counters.ptr, sizeof counters, cudaMemcpyDeviceToHost, out));
  CT_CUDA(cudaStreamSynchronize(out));
  if (chunks > 1) {
    CT_CUDA(cudaStreamSynchronize(stream));
    CT_CUDA(cudaStreamSynchronize(s->compute2));
  }
  if (counters[1]) return fail(CT_ERR_UNSUPPORTED, "traversal stack overflow (stack need %u)", s->stack_need);
  if (stats) {
    float k_ms = 0, all_ms = 0;
    cudaEventElapsedTime(&k_ms, s->ev1, s->ev2);
    cudaEventElapsedTime(&all_ms, s->ev0, s->ev2);
    stats->kernel_ms = k_ms;
    stats->total_ms = all_ms;
    stats->rays = n;
    stats->fp64_fallbacks = counters[0];
    stats->launches = chunks;
  }
  return CT_OK;
}

// Object index of each hit primitive (-1 on a miss).
__global__ void k_pick_objects(const uint32_t* __restrict__ prim_object, const int32_t* __restrict__ prim,
                               uint32_t n, int32_t* __restrict__ object) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) object[i] = prim[i] >= 0 ? (int32_t)prim_object[prim[i]] : -1;
}

// camera.ts:62-77 primaryRay (generateRay with a zero lens sample), float64
// in the reference's operation order.
void primary_ray(const ct_camera_frame& f, double sx, double sy, double o[3], double d[3]) {
  const double px = (2 * sx - 1) * f.tan_half_fov * f.aspect;
  const double py = (2 * sy - 1) * f.tan_half_fov;
  double focus[3], dir[3];
  for (int k = 0; k < 3; k++)
    focus[k] = f.origin[k] + ((f.right[k] * px + f.up[k] * py) + f.forward[k]) * f.focus_distance;
  for (int k = 0; k < 3; k++) {
    const double offset = f.right[k] * (0 * f.lens_radius) + f.up[k] * (0 * f.lens_radius);
    o[k] = f.origin[k] + offset;
    dir[k] = focus[k] - o[k];
  }
  const double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);  // vec3.ts:26-31
  for (int k = 0; k < 3; k++) d[k] = len > 0 ? dir[k] * (1 / len) : 0.0;
}

ct_status pick(ct_scene* s, const ct_camera_frame* frame, uint32_t n, const double* sx, const double* sy,
               int32_t* object, int32_t* prim, float* t, double* point) {
  CT_CHECK_ARG(s != nullptr && frame != nullptr, "NULL scene or frame");
  CT_CHECK_ARG(n == 0 || (sx && sy && object && prim && t), "NULL host pointer");
  if (n == 0) return CT_OK;
  std::vector<float> rays((size_t)n * CT_RAY_FLOATS);
  std::vector<double> ray64((size_t)n * 6);
  for (uint32_t i = 0; i < n; i++) {
    double* o = &ray64[(size_t)i * 6];
    primary_ray(*frame, sx[i], sy[i], o, o + 3);
    float* r = &rays[(size_t)i * CT_RAY_FLOATS];
    for (int k = 0; k < 6; k++) r[k] = (float)o[k];
    r[6] = (float)1e-4;  // T_MIN (intersect.ts:14)
    r[7] = INFINITY;
  }
  std::lock_guard<std::mutex> guard(s->lock);
  CT_CUDA(cudaSetDevice(s->device));
  const size_t ray_bytes = rays.size() * sizeof(float);
  ct_status st = s->io.reserve(ray_bytes + (size_t)n * 12, &s->device_bytes, s->device, s->stream);
  if (st != CT_OK) return st;
  char* base = s->io.as<char>();
  float* d_rays = reinterpret_cast<float*>(base);
  int32_t* d_prim = reinterpret_cast<int32_t*>(base + ray_bytes);
  float* d_t = reinterpret_cast<float*>(d_prim + n);
  int32_t* d_obj = reinterpret_cast<int32_t*>(d_t + n);
  cudaStream_t stream = s->stream;
  CT_CUDA(cudaMemsetAsync(s->counters.ptr, 0, 2 * sizeof(uint32_t), stream));
  CT_CUDA(cudaMemcpyAsync(d_rays, rays.data(), ray_bytes, cudaMemcpyHostToDevice, stream));
  st = launch<false>(s, d_rays, n, d_prim, d_t, nullptr, nullptr, nullptr, stream);
  if (st != CT_OK) return st;
  k_pick_objects<<<(n + 255) / 256, 256, 0, stream>>>(s->prim_object.as<uint32_t>(), d_prim, n, d_obj);
  CT_CUDA(cudaGetLastError());
  CT_CUDA(cudaMemcpyAsync(prim, d_prim, (size_t)n * 4, cudaMemcpyDeviceToHost, stream));
  CT_CUDA(cudaMemcpyAsync(t, d_t, (size_t)n * 4, cudaMemcpyDeviceToHost, stream));
  CT_CUDA(cudaMemcpyAsync(object, d_obj, (size_t)n * 4, cudaMemcpyDeviceToHost, stream));
  uint32_t counters[2] = {0, 0};
  CT_CUDA(cudaMemcpyAsync(counters, s->counters.ptr, sizeof counters, cudaMemcpyDeviceToHost, stream));
  CT_CUDA(cudaStreamSynchronize(stream));
  if (counters[1]) return fail(CT_ERR_UNSUPPORTED, "traversal stack overflow (stack need %u)", s->stack_need);
  if (point) {
    for (uint32_t i = 0; i < n; i++) {  // picking.ts:32: origin + dir * t
      const double* o = &ray64[(size_t)i * 6];
      for (int k = 0; k < 3; k++)
        point[(size_t)i * 3 + k] = prim[i] >= 0 ? o[k] + o[3 + k] * (double)t[i] : NAN;
    }
  }
  return CT_OK;
}

}  // namespace
}  // namespace ct

extern "C" {

ct_status ct_pick(ct_scene* scene, const ct_camera_frame* frame, uint32_t count, const double* sx, const double* sy,
                  int32_t* object, int32_t* prim, float* t, double* point) {
  ct::clear_error();
  try {
    return ct::pick(scene, frame, count, sx, sy, object, prim, t, point);
  } catch (const std::bad_alloc&) {
    return ct::fail(CT_ERR_OUT_OF_MEMORY, "ct_pick: host allocation failed");
  }
}

int32_t ct_set_traversal(int32_t variant) {
  return ct::g_variant.exchange(variant == 1 || variant == 2 ? variant : 0);
}

ct_status ct_trace_closest(ct_scene* scene, const float* rays, uint32_t count, int32_t* prim,
                           float* t, float* u, float* v, ct_stats* stats) {
  ct::clear_error();
  return ct::host_query<false>(scene, rays, count, prim, t, u, v, nullptr, stats);
}

ct_status ct_trace_occluded(ct_scene* scene, const float* rays, uint32_t count, uint8_t* blocked,
                            ct_stats* stats) {
  ct::clear_error();
  return ct::host_query<true>(scene, rays, count, nullptr, nullptr, nullptr, nullptr, blocked, stats);
}

ct_status ct_trace_closest_device(ct_scene* scene, const float* rays, uint32_t count,
                                  int32_t* prim, float* t, float* u, float* v, void* stream) {
  ct::clear_error();
  CT_CHECK_ARG(scene != nullptr, "scene is NULL");
  CT_CHECK_ARG(count == 0 || (rays && prim && t), "NULL device pointer");
  CT_CUDA(cudaSetDevice(scene->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : scene->stream;
  return ct::launch<false>(scene, rays, count, prim, t, u, v, nullptr, s);
}

ct_status ct_trace_occluded_device(ct_scene* scene, const float* rays, uint32_t count,
                                   uint8_t* blocked, void* stream) {
  ct::clear_error();
  CT_CHECK_ARG(scene != nullptr, "scene is NULL");
  CT_CHECK_ARG(count == 0 || (rays && blocked), "NULL device pointer");
  CT_CUDA(cudaSetDevice(scene->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : scene->stream;
  return ct::launch<true>(scene, rays, count, nullptr, nullptr, nullptr, nullptr, blocked, s);
}

}  // extern "C"
