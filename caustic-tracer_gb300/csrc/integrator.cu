// Single-scene path integrator: accumulatePass / renderImage (tracer.ts:348-395)
// on the wavefront kernels of wavefront.cuh.
//
// A render of P passes runs in waves of whole passes (default_wave_paths); a wave
// holds whole passes (path id = pass * W*H + pixel) and its accumulate
// kernel adds each pixel's samples in pass order, so results do not depend
// on the wave size.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "profile.hpp"
#include "scene.hpp"
#include "wavefront.cuh"

namespace ct {

namespace {

// Paths per wave, and path-state sets of a render of several waves: wave k
// runs on set k % n, on the caller's stream or one of the scene's side
// streams, so a wave's last bounces overlap the next waves' first ones.
// Caustic scene, 1080p x 64 spp (Msamples/s): one set of 8 Mi 1,205; three
// of 8 Mi 1,651; three of 16 Mi 1,787; four of 16 Mi 1,819 (11 GB of path
// state); four of 24 Mi 1,807; six of 16 Mi 1,805. With the faster walk of
// today, four sets and waves of 16 / 24 / 32 / 48 / 64 Mi: 2,090 / 2,093 /
// 2,154 / 2,174 / 2,179 at 64 spp (8 / 6 / 4 / 3 / 2 waves), but at 16 spp
// (33 M paths) 2,002 with two waves of 16 Mi against 1,926 with one of 48 Mi,
// and at 32 spp 2,087 (16 Mi) / 2,107 (48 Mi, two waves) / 2,064 (64 Mi,
// one); at 128 spp 2,095 / 2,167 / 2,198. So a render is split into at least
// two waves, each of at least 16 Mi and at most 48 Mi paths (four sets of
// 48 Mi hold 34 GB of path state).
constexpr uint64_t kMinWavePaths = 16ull << 20;
constexpr uint64_t kMaxWavePaths = 48ull << 20;
constexpr int kRenderSets = 4;

// Paths per wave when the scene sets none: half the render, within
// [kMinWavePaths, kMaxWavePaths] (whole passes are then packed up to it).
uint64_t default_wave_paths(uint64_t total_paths) {
  return std::min(kMaxWavePaths, std::max(kMinWavePaths, (total_paths + 1) / 2));
}

// The scene's side streams and events for renders of several waves.
ct_status render_streams(ct_scene* s, int sets) {
  for (int i = 0; i < sets - 1; i++) {
    if (!s->render_side[i]) CT_CUDA(cudaStreamCreateWithFlags(&s->render_side[i], cudaStreamNonBlocking));
    if (!s->render_join[i]) CT_CUDA(cudaEventCreateWithFlags(&s->render_join[i], cudaEventDisableTiming));
  }
  for (int i = 0; i < sets; i++)
    if (!s->render_acc[i]) CT_CUDA(cudaEventCreateWithFlags(&s->render_acc[i], cudaEventDisableTiming));
  if (!s->render_fork) CT_CUDA(cudaEventCreateWithFlags(&s->render_fork, cudaEventDisableTiming));
  return CT_OK;
}
constexpr uint32_t kSkipMaxNodes = 31;         // trees this small use the stackless skip-link walk

// Walk form of a scene's trace launches: the scene's CT_OPT_WALK when set,
// else the stackless walk for small trees and for trees whose ordered walk
// could outgrow its stack, and the persistent ordered walk for the rest. (The
// per-thread ordered walk, kept for CT_OPT_WALK and the autotuner, was the
// default for trees of depth <= 16 until the persistent walk took two steps
// per refill round: on the batched workload the persistent walk everywhere
// runs 819 against 800 Msamples/s.)
int walk_form(const ct_scene* s) {
  if (s->opt_walk >= 0) return s->opt_walk;
  if (s->node_count <= kSkipMaxNodes || s->stack_need > ctk::kStackSize) return kWalkSkip;
  return kWalkPersistent;
}

// Scenes of at most kBrutePrims primitives run whole paths per lane
// (k_paths): same sums as the wavefront kernels, no path queues.
bool whole_paths(const ct_scene* s, int form) {
  return s->opt_path_kernel && form == kWalkSkip && s->prim_count <= ctk::kBrutePrims;
}

// Runs `passes` passes starting at frame index `first` and adds them to the
// device sums accum (and sumsq when non-NULL).
ct_status run_passes(ct_scene* s, const ct_camera_frame& frame, uint32_t width, uint32_t height, uint32_t first,
                     uint32_t passes, const ct_trace_options& o, float* accum, float* sumsq, cudaStream_t stream) {
  const uint64_t pixels = (uint64_t)width * height;
  const uint64_t wave_paths =
      s->opt_wave_paths > 0 ? (uint64_t)s->opt_wave_paths : default_wave_paths(pixels * (uint64_t)passes);
  const uint64_t per_wave = std::max<uint64_t>(1, std::min<uint64_t>(passes, wave_paths / pixels));
  const uint64_t cap = per_wave * pixels;
  const int32_t B = o.max_bounces;
  const int form = walk_form(s);
  const bool whole = whole_paths(s, form);
  const uint64_t waves = (passes + per_wave - 1) / per_wave;
  const int sets = whole ? 1 : (int)std::min<uint64_t>(kRenderSets, waves);
  ct_status st;
  if (sets > 1 && (st = render_streams(s, sets)) != CT_OK) return st;
  // Path buffer per set: 2 queues + shadow queue (3 float4 each per path),
  // radiance (float4), hit prim/t, counters; k_paths needs the radiance and
  // counters.
  const size_t q_bytes = cap * sizeof(float4);
  const size_t counter_words = wave_counter_words(B);
  const size_t set_bytes = (whole ? q_bytes : 10 * q_bytes + cap * 8) + counter_words * 4 + 16 * 256;
  void* buf = nullptr;
  st = path_alloc(s->device, set_bytes * (size_t)sets, stream, &buf);
  if (st != CT_OK) return st;
  struct Release {  // back to the pool, in stream order, on every return
    void* p;
    cudaStream_t s;
    ~Release() { path_free(p, s); }
  } release{buf, stream};
  // The side streams join `stream` before the buffer goes back (declared
  // after `release`, so it runs first), also on an early error return.
  struct Join {
    ct_scene* s;
    cudaStream_t stream;
    int sets;
    bool forked = false;
    ~Join() {
      if (!forked) return;
      for (int i = 0; i < sets - 1; i++) {
        cudaEventRecord(s->render_join[i], s->render_side[i]);
        cudaStreamWaitEvent(stream, s->render_join[i], 0);
      }
    }
  } join{s, stream, sets};
  char* base = static_cast<char*>(buf);
  auto take = [&](size_t n) {
    char* p = base;
    base += (n + 255) & ~size_t(255);
    return p;
  };
  WaveArgs set_args[kRenderSets];
  for (int set = 0; set < sets; set++) {
    WaveArgs& a = set_args[set];
    a = WaveArgs{};
    a.scene = s->dev;
    a.sky = to_sky(s->sky);
    a.frame = to_frame(frame);
    if (!whole) {
      a.cur = Queue{(float4*)take(q_bytes), (float4*)take(q_bytes), (float4*)take(q_bytes), nullptr};
      a.next = Queue{(float4*)take(q_bytes), (float4*)take(q_bytes), (float4*)take(q_bytes), nullptr};
      a.shadow = ShadowQueue{(float4*)take(q_bytes), (float4*)take(q_bytes), (float4*)take(q_bytes)};
      a.hit_prim = (int32_t*)take(cap * 4);
      a.hit_t = (float*)take(cap * 4);
    }
    a.radiance = (float4*)take(q_bytes);
    a.counts = (uint32_t*)take(counter_words * 4);
    a.width = width;
    a.height = height;
    a.pixels = (uint32_t)pixels;
    a.max_bounces = B;
    a.rr = o.russian_roulette;
    a.nee = o.nee;
  }
  WaveArgs& a = set_args[0];
  const Grids<false>& g = grids<false>();
  if (whole) {
    for (uint64_t done = 0; done < passes; done += per_wave) {
      const uint32_t p = (uint32_t)std::min<uint64_t>(per_wave, passes - done);
      a.paths = (uint32_t)(p * pixels);
      a.first_frame = first + (uint32_t)done;
      CT_CUDA(cudaMemsetAsync(a.counts, 0, counter_words * 4, stream));
      {
        ProfScope ps("paths", stream);
        k_paths<<<g.capped(g.paths, s->opt_trace_blocks), kBlock, 0, stream>>>(a);
      }
      {
        ProfScope ps("accumulate", stream);
        k_accumulate<<<g.acc, kBlock, 0, stream>>>(a.radiance, a.pixels, p, accum, sumsq);
      }
      CT_CUDA(cudaGetLastError());
    }
    return CT_OK;
  }
  if (sets > 1) {
    CT_CUDA(cudaEventRecord(s->render_fork, stream));
    for (int i = 0; i < sets - 1; i++) CT_CUDA(cudaStreamWaitEvent(s->render_side[i], s->render_fork, 0));
    join.forked = true;
  }
  uint64_t k = 0;
  for (uint64_t done = 0; done < passes; done += per_wave, k++) {
    const int set = (int)(k % (uint64_t)sets);
    const cudaStream_t st = set ? s->render_side[set - 1] : stream;
    WaveArgs& wa = set_args[set];
    const uint32_t p = (uint32_t)std::min<uint64_t>(per_wave, passes - done);
    wa.paths = (uint32_t)(p * pixels);
    wa.first_frame = first + (uint32_t)done;
    CT_CUDA(cudaMemsetAsync(wa.counts, 0, counter_words * 4, st));
    {
      ProfScope ps("generate", st);
      k_generate<false><<<g.gen, kBlock, 0, st>>>(wa);
    }
    WaveArgs w = wa;
    auto trace = [&](int32_t b) {
      ProfScope ps("trace", st);
      launch_trace<false>(form, w, b, st, s->opt_trace_blocks);
    };
    for (int32_t b = 0; b <= B; b++) {
      trace(b);
      {
        ProfScope ps("shade", st);
        k_shade<false><<<g.shade, kBlock, 0, st>>>(w, b);
      }
      std::swap(w.cur, w.next);
    }
    trace(B + 1);
    // pass order: this wave's samples are added after the previous wave's
    if (sets > 1 && k > 0) CT_CUDA(cudaStreamWaitEvent(st, s->render_acc[(k - 1) % (uint64_t)sets], 0));
    {
      ProfScope ps("accumulate", st);
      k_accumulate<<<g.acc, kBlock, 0, st>>>(wa.radiance, wa.pixels, p, accum, sumsq);
    }
    if (sets > 1) CT_CUDA(cudaEventRecord(s->render_acc[set], st));
    CT_CUDA(cudaGetLastError());
  }
  return CT_OK;
}

// renderImage (tracer.ts:348-355) into the device array `out`; caller holds the scene lock.
ct_status render_locked(ct_scene* scene, const ct_camera_frame* frame, const ct_render_options* o, float* out,
                        cudaStream_t s) {
  CT_CHECK_ARG(o->spp > 0, "spp %d must be positive", o->spp);
  ct_status st = check_options(frame, o->width, o->height, o->max_bounces);
  if (st != CT_OK) return st;
  const size_t n = (size_t)o->width * o->height * 3;
  CT_CUDA(cudaMemsetAsync(out, 0, n * sizeof(float), s));
  const ct_trace_options t{o->max_bounces, o->russian_roulette, o->nee};
  st = run_passes(scene, *frame, (uint32_t)o->width, (uint32_t)o->height, o->seed * 7919u, (uint32_t)o->spp, t, out,
                  nullptr, s);
  if (st != CT_OK) return st;
  {
    ProfScope ps("scale", s);
    k_scale<<<592, 256, 0, s>>>(out, n, (float)o->spp);
  }
  CT_CUDA(cudaGetLastError());
  return CT_OK;
}

}  // namespace

int integrator_walk_form(const ct_scene* s) { return walk_form(s); }
bool integrator_whole_paths(const ct_scene* s) { return whole_paths(s, walk_form(s)); }

}  // namespace ct

extern "C" {

int32_t ct_scene_walk(const ct_scene* scene) { return scene ? ct::walk_form(scene) : -1; }

ct_status ct_accumulate_passes_device(ct_scene* scene, const ct_camera_frame* frame, int32_t width, int32_t height,
                                      uint32_t first_frame_index, int32_t passes, const ct_trace_options* opts,
                                      float* accum, float* sumsq, void* stream) {
  ct::clear_error();
  CT_CHECK_ARG(scene != nullptr && opts != nullptr && accum != nullptr, "NULL argument");
  CT_CHECK_ARG(passes >= 0, "passes %d is negative", passes);
  ct_status st = ct::check_options(frame, width, height, opts->max_bounces);
  if (st != CT_OK) return st;
  std::lock_guard<std::mutex> guard(scene->lock);
  CT_CUDA(cudaSetDevice(scene->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : scene->stream;
  if (passes == 0) return CT_OK;
  return ct::run_passes(scene, *frame, (uint32_t)width, (uint32_t)height, first_frame_index, (uint32_t)passes, *opts,
                        accum, sumsq, s);
}

ct_status ct_render_image_device(ct_scene* scene, const ct_camera_frame* frame, const ct_render_options* o, float* out,
                                 void* stream) {
  ct::clear_error();
  CT_CHECK_ARG(scene != nullptr && o != nullptr && out != nullptr, "NULL argument");
  std::lock_guard<std::mutex> guard(scene->lock);
  CT_CUDA(cudaSetDevice(scene->device));
  return ct::render_locked(scene, frame, o, out, stream ? static_cast<cudaStream_t>(stream) : scene->stream);
}

ct_status ct_accumulate_pass(ct_scene* scene, const ct_camera_frame* frame, int32_t width, int32_t height,
                             uint32_t frame_index, const ct_trace_options* opts, float* accum, ct_stats* stats) {
  ct::clear_error();
  CT_CHECK_ARG(scene != nullptr && opts != nullptr && accum != nullptr, "NULL argument");
  ct_status st = ct::check_options(frame, width, height, opts->max_bounces);
  if (st != CT_OK) return st;
  std::lock_guard<std::mutex> guard(scene->lock);
  CT_CUDA(cudaSetDevice(scene->device));
  const size_t n = (size_t)width * height * 3;
  st = scene->io.reserve(n * sizeof(float), &scene->device_bytes, scene->device, scene->stream);
  if (st != CT_OK) return st;
  cudaStream_t s = scene->stream;
  float* d = scene->io.as<float>();
  CT_CUDA(cudaEventRecord(scene->ev0, s));
  CT_CUDA(cudaMemcpyAsync(d, accum, n * sizeof(float), cudaMemcpyHostToDevice, s));
  CT_CUDA(cudaEventRecord(scene->ev1, s));
  st = ct::run_passes(scene, *frame, (uint32_t)width, (uint32_t)height, frame_index, 1, *opts, d, nullptr, s);
  if (st != CT_OK) return st;
  CT_CUDA(cudaEventRecord(scene->ev2, s));
  CT_CUDA(cudaMemcpyAsync(accum, d, n * sizeof(float), cudaMemcpyDeviceToHost, s));
  CT_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    float k = 0, all = 0;
    cudaEventElapsedTime(&k, scene->ev1, scene->ev2);
    cudaEventElapsedTime(&all, scene->ev0, scene->ev2);
    std::memset(stats, 0, sizeof *stats);
    stats->kernel_ms = k;
    stats->total_ms = all;
  }
  return CT_OK;
}

ct_status ct_render_image(ct_scene* scene, const ct_camera_frame* frame, const ct_render_options* o, float* out,
                          ct_stats* stats) {
  ct::clear_error();
  CT_CHECK_ARG(scene != nullptr && o != nullptr && out != nullptr, "NULL argument");
  CT_CHECK_ARG(o->width > 0 && o->height > 0, "image size %dx%d is not positive", o->width, o->height);
  const size_t n = (size_t)o->width * o->height * 3;
  std::lock_guard<std::mutex> guard(scene->lock);
  CT_CUDA(cudaSetDevice(scene->device));
  ct_status st = scene->io.reserve(n * sizeof(float), &scene->device_bytes, scene->device, scene->stream);
  if (st != CT_OK) return st;
  float* d = scene->io.as<float>();
  CT_CUDA(cudaEventRecord(scene->ev0, scene->stream));
  st = ct::render_locked(scene, frame, o, d, scene->stream);
  if (st != CT_OK) return st;
  CT_CUDA(cudaEventRecord(scene->ev1, scene->stream));
  CT_CUDA(cudaMemcpyAsync(out, d, n * sizeof(float), cudaMemcpyDeviceToHost, scene->stream));
  CT_CUDA(cudaStreamSynchronize(scene->stream));
  if (stats) {
    float k = 0;
    cudaEventElapsedTime(&k, scene->ev0, scene->ev1);
    std::memset(stats, 0, sizeof *stats);
    stats->kernel_ms = k;
    stats->total_ms = k;
  }
  return CT_OK;
}

}  // extern "C"

// ---- accumulatePass without allocation ------------------------------------------
//
// Some callers cannot allocate device memory at the time they render:
// real-time loops that forbid allocation per frame (an allocation can wait on
// the device and miss the frame), plugin hosts that hand the library a fixed
// memory budget at load time and own every later allocation, and deployments
// that reserve all device memory up front. ct_accumulate_pass_noalloc serves
// them: its
// scratch (path queues, shadow queue, per-path radiance, hit records, queue
// counters) lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits. The scene (created earlier
// with ct_scene_create) and the accumulation buffer are the caller's.
namespace ct {
namespace {

constexpr size_t round256(size_t n) { return (n + 255) & ~size_t(255); }
constexpr uint32_t kNoAllocMaxPixels = CT_NOALLOC_MAX_PIXELS;
constexpr size_t kNoAllocCounterWords = 4096;
// Bytes the carve in ct_accumulate_pass_noalloc takes for `pixels` path
// slots and `words` queue counters: 10 float4 arrays (two path queues and
// the shadow queue of three float4 each, the radiance), the hit prims and
// distances, the counters, each start rounded up to 256 bytes. It grows with
// both arguments, so the array sized for the maxima holds every accepted call.
constexpr size_t noalloc_layout_bytes(size_t pixels, size_t words) {
  return 10 * round256(pixels * sizeof(float4)) + 2 * round256(pixels * 4) + round256(words * 4);
}
constexpr size_t kNoAllocScratchBytes = noalloc_layout_bytes(kNoAllocMaxPixels, kNoAllocCounterWords);
static_assert(kNoAllocScratchBytes <= (size_t)44 << 20, "the static scratch stays within 44 MiB");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// cuCtxGetCurrent through the runtime's driver entry points (no link against
// libcuda): the scratch address belongs to the context it was looked up in.
using CtxGetCurrent = int (*)(void**);
CtxGetCurrent ctx_get_current() {
  static const CtxGetCurrent fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrent>(p);
  }();
  return fn;
}

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
struct NoAllocSlot {
  void* ptr = nullptr;
  void* ctx = nullptr;
};
NoAllocSlot g_noalloc[kMaxDevices];

// Device address of the scratch array on the current device (the host
// symbol itself is only a stand-in for it). Looked up on the first call on a
// device, and again whenever that device's current context differs from the
// one the address was taken in (after a cudaDeviceReset the array has a new
// address in the new primary context).
ct_status noalloc_scratch(int device, void** out) {
  CT_CHECK_ARG(device >= 0 && device < kMaxDevices, "device %d beyond %d", device, kMaxDevices);
  void* ctx = nullptr;
  CtxGetCurrent get = ctx_get_current();
  if (get && get(&ctx) != 0) ctx = nullptr;
  std::lock_guard<std::mutex> guard(g_noalloc_mu);
  NoAllocSlot& slot = g_noalloc[device];
  if (!slot.ptr || !ctx || slot.ctx != ctx) {
    void* p = nullptr;
    CT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    slot.ptr = p;
    slot.ctx = ctx;
  }
  *out = slot.ptr;
  return CT_OK;
}

}  // namespace
}  // namespace ct

extern "C" {

ct_status ct_accumulate_pass_noalloc(ct_scene* scene, const ct_camera_frame* frame, int32_t width, int32_t height,
                                     uint32_t frame_index, const ct_trace_options* opts, float* accum, void* stream) {
  using namespace ct;
  clear_error();
  CT_CHECK_ARG(scene != nullptr && opts != nullptr && accum != nullptr, "NULL argument");
  ct_status st = check_options(frame, width, height, opts->max_bounces);
  if (st != CT_OK) return st;
  const uint64_t pixels = (uint64_t)width * (uint64_t)height;
  CT_CHECK_ARG(pixels <= kNoAllocMaxPixels,
               "ct_accumulate_pass_noalloc: %dx%d = %llu pixels exceeds the static scratch limit of %u pixels",
               width, height, (unsigned long long)pixels, kNoAllocMaxPixels);
  const int32_t B = opts->max_bounces;
  const size_t counter_words = wave_counter_words(B);
  CT_CHECK_ARG(counter_words <= kNoAllocCounterWords, "max_bounces %d needs more queue counters than the static scratch holds", B);
  std::lock_guard<std::mutex> guard(scene->lock);
  CT_CUDA(cudaSetDevice(scene->device));
  void* scratch = nullptr;
  st = noalloc_scratch(scene->device, &scratch);
  if (st != CT_OK) return st;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : scene->stream;

  // Carve the per-path arrays for exactly `pixels` slots (one pass).
  char* base = static_cast<char*>(scratch);
  auto take = [&](size_t n) {
    char* p = base;
    base += round256(n);
    return p;
  };
  const size_t q = pixels * sizeof(float4);
  WaveArgs a{};
  a.scene = scene->dev;
  a.sky = to_sky(scene->sky);
  a.frame = to_frame(*frame);
  a.cur = Queue{(float4*)take(q), (float4*)take(q), (float4*)take(q), nullptr};
  a.next = Queue{(float4*)take(q), (float4*)take(q), (float4*)take(q), nullptr};
  a.shadow = ShadowQueue{(float4*)take(q), (float4*)take(q), (float4*)take(q)};
  a.radiance = (float4*)take(q);
  a.hit_prim = (int32_t*)take(pixels * 4);
  a.hit_t = (float*)take(pixels * 4);
  a.counts = (uint32_t*)take(counter_words * 4);
  a.width = (uint32_t)width;
  a.height = (uint32_t)height;
  a.pixels = (uint32_t)pixels;
  a.paths = (uint32_t)pixels;
  a.first_frame = frame_index;
  a.max_bounces = B;
  a.rr = opts->russian_roulette;
  a.nee = opts->nee;

  // The array keeps the previous call's contents: the counters must start at zero.
  CT_CUDA(cudaMemsetAsync(a.counts, 0, counter_words * 4, s));
  const Grids<false>& g = grids<false>();
  if (integrator_whole_paths(scene)) {
    // the kernels ct_accumulate_pass runs for this scene: whole paths per lane
    k_paths<<<g.capped(g.paths, scene->opt_trace_blocks), kBlock, 0, s>>>(a);
  } else {
    const int form = integrator_walk_form(scene);
    k_generate<false><<<g.gen, kBlock, 0, s>>>(a);
    WaveArgs w = a;
    for (int32_t b = 0; b <= B + 1; b++) {
      launch_trace<false>(form, w, b, s, scene->opt_trace_blocks);
      if (b > B) break;
      k_shade<false><<<g.shade, kBlock, 0, s>>>(w, b);
      std::swap(w.cur, w.next);
    }
  }
  k_accumulate<<<g.acc, kBlock, 0, s>>>(a.radiance, a.pixels, 1, accum, nullptr);
  CT_CUDA(cudaGetLastError());
  return CT_OK;
}

}  // extern "C"
