// Device-resident scene of libcaustic_gb300 (the object behind ct_scene*).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "common.hpp"
#include "traverse.cuh"

namespace ct {

#define CT_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t err_ = (call);                                                        \
    if (err_ != cudaSuccess)                                                          \
      return ::ct::fail(err_ == cudaErrorMemoryAllocation ? CT_ERR_OUT_OF_MEMORY      \
                                                          : CT_ERR_CUDA,              \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(err_), __FILE__, __LINE__); \
  } while (0)

// Growable device allocation owned by a scene.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  // Grows to at least `want` bytes from the per-device pool (path_alloc), in
  // the order of `stream`; release returns it there.
  ct_status reserve(size_t want, size_t* total_bytes, int device, cudaStream_t stream);
  void release(size_t* total_bytes, cudaStream_t stream);
  template <class T>
  T* as() const {
    return static_cast<T*>(ptr);
  }
};

// Path state (wavefront queues and per-path arrays) comes from one
// stream-ordered memory pool per device: a render or batch allocates it on
// its stream and frees it there when its work is queued, and the pool keeps
// freed blocks for the next one, so renders neither hold memory between
// calls nor pay for cudaMalloc/cudaFree (which would wait for the device).
ct_status path_alloc(int device, size_t bytes, cudaStream_t s, void** out);
void path_free(void* p, cudaStream_t s);

// Trace walk the single-scene integrator uses for `s` (0 ordered per thread,
// 1 ordered persistent, 2 stackless skip-link); see integrator.cu.
int integrator_walk_form(const ct_scene* s);
// True when renders of this scene run whole paths per lane (k_paths).
bool integrator_whole_paths(const ct_scene* s);

}  // namespace ct

struct ct_scene {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex lock;

  // Device copies of the packed arrays plus the 4-wide walk records: slices
  // of one pool allocation (`arena`).
  void* arena = nullptr;
  ct::DeviceBuffer prims, nodes, quads, mats, lights, prim_object;
  ct::DeviceBuffer planes;  // 3 float4 plane records per primitive (integrator tests)
  ct::DeviceBuffer tris;    // 3 float4 per primitive: a, b, c of prims (exact tests), built on the device
  uint32_t prim_count = 0, node_count = 0, interior_count = 0, mat_count = 0, light_count = 0;
  uint32_t depth = 0;       // deepest root-to-leaf path, in nodes
  uint32_t stack_need = 0;  // deepest stack the ordered walk can build
  ct_sky sky{};
  ctk::SceneDev dev{};

  // Staging for host-pointer entry points and per-call counters.
  ct::DeviceBuffer io;
  ct::DeviceBuffer counters;  // uint32 fp64-fallback counter and error flag
  size_t device_bytes = 0;

  // Tuning options (ct_scene_set_option): integrator walk form (-1 = chosen
  // from the tree), paths per wave (0 = library default) and blocks per SM
  // of the trace launches.
  int32_t opt_walk = -1;
  int64_t opt_wave_paths = 0;
  int32_t opt_trace_blocks = 0;  // blocks per SM of trace launches (0 = occupancy)
  bool opt_path_kernel = true;   // whole-path kernel for scenes of <= 32 primitives

  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
  // Streams and events of chunked host-pointer queries (created on the first
  // such query): rays in on copy_in, results out on copy_out, while `stream`
  // and compute2 trace alternate chunks.
  cudaStream_t copy_in = nullptr, copy_out = nullptr, compute2 = nullptr;
  cudaEvent_t ev_in = nullptr, ev_done = nullptr;
  // Streams and events of renders of several waves (created on the first
  // one): consecutive waves run round robin on the caller's stream and these.
  static constexpr int kRenderSides = 3;
  cudaStream_t render_side[kRenderSides] = {};
  cudaEvent_t render_fork = nullptr, render_join[kRenderSides] = {}, render_acc[kRenderSides + 1] = {};
};

namespace ct {
// Counters block layout (uint32 words).
enum CounterWord : int { kCountFallbacks = 0, kCountError = 1, kCountQueue = 2, kCounterWords = 64 };
}  // namespace ct
