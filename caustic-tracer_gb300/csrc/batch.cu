// Batched rendering: many scenes, cameras and image sizes in one graph.
//
// A batch is a list of jobs (scene, camera, size, frame indices, passes, sum
// buffer). Their paths are packed into waves of up to `wave_paths` paths. The
// planner takes the jobs grouped by trace walk and then by scene (a wave
// runs one walk's kernel; the paths in flight at any time touch few BVHs) and
// appends each job's passes as chunks: as many whole passes as fit in the
// open wave, laid out pass-major; a pass larger than a wave is split by pixel
// ranges over several waves. A wave holds at most one chunk of any job, so
// every pixel's samples are added in pass order by a single thread (the sum a
// single-scene render computes). All waves run on the shared wavefront
// kernels (BATCH = true), each path finding its scene, sky, camera and output
// through its job record. ct_batch_run captures the full launch sequence of
// all waves once into a CUDA graph and replays it; the frame indices live in
// a device table, so progressive passes reuse the same graph
// (ct_batch_set_first_frames). ct_batch_run_direct launches the same
// sequence without a graph, for batches run once.
//
// A batch of several waves keeps up to kWaveSets sets of path state and runs
// consecutive waves round robin on as many streams, so one wave's last
// bounces (few paths left, short launches) overlap the next wave's first
// ones. Each wave's accumulate kernel waits for the previous wave's, which
// keeps every pixel's passes added in pass order: the sums are those of the
// one-stream order (256-scene batch: 951 -> 1,076 Msamples/s with two sets).
#include <algorithm>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

#include "profile.hpp"
#include "scene.hpp"
#include "wavefront.cuh"

struct ct_batch {
  int device = 0;
  cudaStream_t stream = nullptr;  // used when ct_batch_run gets no stream
  ct_trace_options opts{};
  int walk = 0;
  std::vector<ct_batch_job> jobs;
  std::vector<ct::SegDev> segs;            // all waves, host copy
  std::vector<uint32_t> seg_pass;          // pass number of each segment
  struct Wave {
    uint32_t seg0, nsegs, paths, acc;
    int walk;
  };
  std::vector<Wave> waves;
  uint64_t max_paths = 0, total_paths = 0;
  void* d_paths = nullptr;  // job and chunk tables, then the path state (pool memory)
  ct::JobDev* d_jobs = nullptr;
  ct::SegDev* d_segs = nullptr;
  static constexpr int kMaxSets = 4;
  ct::WaveArgs sets[kMaxSets]{};  // path-state sets; wave k uses set k % nsets
  int nsets = 1;
  cudaStream_t side[kMaxSets] = {};  // streams of sets 1.. (set 0 runs on the caller's stream)
  cudaEvent_t fork = nullptr, join[kMaxSets] = {}, acc_done[kMaxSets] = {};
  cudaEvent_t sums_done = nullptr;  // after the last accumulate of a direct run
  size_t counter_words = 0;
  bool segs_dirty = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t graph_nodes = 0;
  cudaEvent_t done = nullptr;  // recorded after every run
};

namespace ct {
namespace {

// Paths per wave and path-state sets (streams) of a batch of several waves:
// on the 256-scene workload 8 Mi paths and one set 952 Msamples/s, two sets
// 1,075, four 1,137; 24 Mi paths and four sets 1,201 (six: 1,202); 32 Mi
// and four sets 1,207 (48 Mi: 1,216). With the faster walk of today: 24,
// 32, 40, 48, 64 Mi and four sets 1,428 / 1,436 / 1,439 / 1,449 / 1,446;
// 48 Mi and six sets 1,441. Four sets of 48 Mi paths hold 33 GB of path
// state; a batch takes only what its largest wave needs.
constexpr uint64_t kDefaultWavePaths = 48ull << 20;
constexpr int kWaveSets = 4;

// Trace walk of job j's waves: the batch's walk, or (kWalkPerJob) the one its
// scene uses alone.
int job_walk(const ct_batch* b, uint32_t j) {
  return b->walk != kWalkPerJob ? b->walk : integrator_walk_form(b->jobs[j].scene);
}

void plan(ct_batch* b, uint64_t cap) {
  const uint32_t n = (uint32_t)b->jobs.size();
  // Jobs grouped by walk, then by scene (groups in order of first
  // appearance); a wave holds jobs of one walk and runs its kernel. (The two
  // ordered walks give the same hits, but a wave of shallow and deep trees
  // together runs slower under either kernel than the two apart.)
  std::vector<uint32_t> order(n), group(n);
  std::vector<int> walk(n);
  std::unordered_map<const ct_scene*, uint32_t> first_job;
  for (uint32_t j = 0; j < n; j++) {
    group[j] = first_job.emplace(b->jobs[j].scene, j).first->second;
    walk[j] = job_walk(b, j);
    order[j] = j;
  }
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
    return walk[x] != walk[y] ? walk[x] < walk[y] : group[x] < group[y];
  });
  int cur_walk = n ? walk[order[0]] : kWalkThread;
  auto open = [&]() { b->waves.push_back({(uint32_t)b->segs.size(), 0, 0, 0, cur_walk}); };
  auto add = [&](uint32_t j, uint32_t q, uint32_t passes, uint32_t pixel0, uint32_t npix) {
    ct_batch::Wave& w = b->waves.back();
    b->segs.push_back(SegDev{j, b->jobs[j].first_frame_index + q, pixel0, w.paths, npix, passes, w.acc, 0});
    b->seg_pass.push_back(q);
    w.nsegs++;
    w.paths += passes * npix;
    w.acc += npix;
  };
  open();
  for (uint32_t j : order) {
    const ct_batch_job& job = b->jobs[j];
    if (walk[j] != cur_walk) {  // waves never mix walks
      cur_walk = walk[j];
      if (b->waves.back().nsegs) open();
      b->waves.back().walk = cur_walk;
    }
    const uint64_t pixels = (uint64_t)job.width * (uint64_t)job.height;
    const uint32_t P = (uint32_t)job.passes;
    uint32_t q = 0, done = 0;  // next pass; pixels of pass q already placed
    bool here = false;         // the open wave already holds a chunk of job j
    while (q < P) {
      if (here || b->waves.back().paths >= cap) {
        open();
        here = false;
      }
      const uint64_t room = cap - b->waves.back().paths;
      if (done == 0 && pixels <= room) {  // whole passes
        const uint32_t np = (uint32_t)std::min<uint64_t>(P - q, room / pixels);
        add(j, q, np, 0, (uint32_t)pixels);
        q += np;
      } else if (done == 0 && pixels <= cap) {  // a whole pass fits in a fresh wave
        open();
        continue;
      } else {  // a pass larger than a wave, split by pixel ranges
        const uint32_t take = (uint32_t)std::min<uint64_t>(pixels - done, room);
        add(j, q, 1, done, take);
        done += take;
        if (done == pixels) done = 0, q++;
      }
      here = true;
    }
  }
  if (b->waves.back().nsegs == 0) b->waves.pop_back();
  for (const auto& w : b->waves) {
    b->max_paths = std::max<uint64_t>(b->max_paths, w.paths);
    b->total_paths += w.paths;
  }
}

// Enqueues every wave of the batch on `s` (captured into the graph); with
// several path-state sets, wave k runs on the stream of set k % nsets (set 0
// on `s`, the others forked from and joined back into `s`). Direct runs
// (`direct`) record sums_done after the last accumulate, and with `after`
// their first accumulate waits for that batch's sums_done.
ct_status enqueue_all(ct_batch* b, cudaStream_t s, bool direct = false, const ct_batch* after = nullptr) {
  const Grids<true>& g = grids<true>();
  const int32_t B = b->opts.max_bounces;
  const int n = b->nsets;
  if (n > 1) {
    CT_CUDA(cudaEventRecord(b->fork, s));
    for (int i = 1; i < n; i++) CT_CUDA(cudaStreamWaitEvent(b->side[i], b->fork, 0));
  }
  for (size_t k = 0; k < b->waves.size(); k++) {
    const auto& wv = b->waves[k];
    const int set = (int)(k % (size_t)n);
    const cudaStream_t st = set ? b->side[set] : s;
    WaveArgs a = b->sets[set];
    a.segs = b->d_segs + wv.seg0;
    a.nsegs = wv.nsegs;
    a.paths = wv.paths;
    a.acc_items = wv.acc;
    CT_CUDA(cudaMemsetAsync(a.counts, 0, b->counter_words * 4, st));
    k_generate<true><<<g.gen, kBlock, 0, st>>>(a);
    WaveArgs w = a;
    for (int32_t bounce = 0; bounce <= B; bounce++) {
      launch_trace<true>(wv.walk, w, bounce, st);
      k_shade<true><<<g.shade, kBlock, 0, st>>>(w, bounce);
      std::swap(w.cur, w.next);
    }
    launch_trace<true>(wv.walk, w, B + 1, st);
    // pass order: wave k's sums are added after wave k-1's (and wave 0's after `after`'s)
    if (n > 1 && k > 0) CT_CUDA(cudaStreamWaitEvent(st, b->acc_done[(k - 1) % (size_t)n], 0));
    if (k == 0 && after && after->sums_done) CT_CUDA(cudaStreamWaitEvent(st, after->sums_done, 0));
    k_accumulate_batch<<<g.acc, kBlock, 0, st>>>(a);
    if (n > 1) CT_CUDA(cudaEventRecord(b->acc_done[set], st));
    if (direct && k + 1 == b->waves.size()) CT_CUDA(cudaEventRecord(b->sums_done, st));
  }
  for (int i = 1; i < n; i++) {
    CT_CUDA(cudaEventRecord(b->join[i], b->side[i]));
    CT_CUDA(cudaStreamWaitEvent(s, b->join[i], 0));
  }
  CT_CUDA(cudaGetLastError());
  return CT_OK;
}

void destroy(ct_batch* b) {
  if (!b) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (cudaStream_t x : b->side)
    if (x) cudaStreamSynchronize(x);
  if (b->done) cudaEventSynchronize(b->done);  // the last run, on whatever stream it used
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->d_paths) path_free(b->d_paths, b->stream);  // the runs are done: back to the pool at once
  if (b->done) cudaEventDestroy(b->done);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->sums_done) cudaEventDestroy(b->sums_done);
  for (int i = 0; i < ct_batch::kMaxSets; i++) {
    if (b->join[i]) cudaEventDestroy(b->join[i]);
    if (b->acc_done[i]) cudaEventDestroy(b->acc_done[i]);
    if (b->side[i]) cudaStreamDestroy(b->side[i]);
  }
  if (b->stream) cudaStreamDestroy(b->stream);
  cudaSetDevice(prev);
  delete b;
}

ct_status create(const ct_batch_job* jobs, uint32_t count, const ct_trace_options* o, int64_t wave_paths,
                 int32_t walk, ct_batch** out) {
  CT_CHECK_ARG(jobs != nullptr && count > 0 && o != nullptr && out != nullptr, "NULL argument or empty batch");
  CT_CHECK_ARG(walk >= -1 && walk <= 2, "batch walk %d must be -1 (per job), 0, 1 or 2", walk);
  CT_CHECK_ARG(wave_paths >= 0 && wave_paths <= (1ll << 30), "wave_paths %lld outside [0, 2^30]", (long long)wave_paths);
  const int device = jobs[0].scene ? jobs[0].scene->device : -1;
  for (uint32_t i = 0; i < count; i++) {
    const ct_batch_job& j = jobs[i];
    CT_CHECK_ARG(j.scene != nullptr && j.accum != nullptr, "job %u: NULL scene or accum", i);
    CT_CHECK_ARG(j.scene->device == device, "job %u: scene lives on device %d, job 0 on %d", i, j.scene->device, device);
    CT_CHECK_ARG(j.passes >= 0, "job %u: passes %d is negative", i, j.passes);
    if (walk == 0 || walk == 1)
      CT_CHECK_ARG(j.scene->stack_need <= ctk::kStackSize, "job %u: tree too deep for the ordered walk", i);
    ct_status st = check_options(&j.frame, j.width, j.height, o->max_bounces);
    if (st != CT_OK) return fail(st, "job %u: %s", i, last_error());
  }
  const uint64_t cap = wave_paths > 0 ? (uint64_t)wave_paths : kDefaultWavePaths;
  ct_batch* b = new (std::nothrow) ct_batch();
  if (!b) return fail(CT_ERR_OUT_OF_MEMORY, "ct_batch_create: host allocation failed");
  b->device = device;
  b->opts = *o;
  b->walk = walk >= 0 ? walk : kWalkPerJob;
  b->jobs.assign(jobs, jobs + count);
  auto bail = [&](ct_status code) {
    destroy(b);
    return code;
  };
  try {
    plan(b, cap);
  } catch (const std::bad_alloc&) {
    return bail(fail(CT_ERR_OUT_OF_MEMORY, "ct_batch_create: host allocation failed"));
  }
  {
    cudaError_t err = cudaSetDevice(device);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (err != cudaSuccess) {
      b->stream = nullptr;
      return bail(fail(CT_ERR_CUDA, "ct_batch_create: %s", cudaGetErrorString(err)));
    }
    err = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (err != cudaSuccess) {
      b->done = nullptr;
      return bail(fail(CT_ERR_CUDA, "ct_batch_create: %s", cudaGetErrorString(err)));
    }
    err = cudaEventCreateWithFlags(&b->sums_done, cudaEventDisableTiming);
    if (err != cudaSuccess) {
      b->sums_done = nullptr;
      return bail(fail(CT_ERR_CUDA, "ct_batch_create: %s", cudaGetErrorString(err)));
    }
    b->nsets = (int)std::min<size_t>(std::min(kWaveSets, ct_batch::kMaxSets), std::max<size_t>(1, b->waves.size()));
    if (b->nsets > 1) {
      auto event = [&](cudaEvent_t* e) {
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(e, cudaEventDisableTiming);
        if (err != cudaSuccess) *e = nullptr;
      };
      event(&b->fork);
      for (int i = 0; i < b->nsets; i++) {
        event(&b->acc_done[i]);
        if (i == 0) continue;
        event(&b->join[i]);
        if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&b->side[i], cudaStreamNonBlocking);
        if (err != cudaSuccess) b->side[i] = nullptr;
      }
      if (err != cudaSuccess) return bail(fail(CT_ERR_CUDA, "ct_batch_create: %s", cudaGetErrorString(err)));
    }
  }
  std::vector<JobDev> host_jobs(count);
  for (uint32_t i = 0; i < count; i++) {
    const ct_batch_job& j = jobs[i];
    host_jobs[i].scene = j.scene->dev;
    host_jobs[i].sky = to_sky(j.scene->sky);
    host_jobs[i].frame = to_frame(j.frame);
    host_jobs[i].width = (uint32_t)j.width;
    host_jobs[i].height = (uint32_t)j.height;
    host_jobs[i].accum = j.accum;
  }
  const uint64_t cap_paths = std::max<uint64_t>(1, b->max_paths);
  const size_t q = cap_paths * sizeof(float4), w4 = cap_paths * 4;
  b->counter_words = wave_counter_words(o->max_bounces);
  const size_t jobs_bytes = host_jobs.size() * sizeof(JobDev), segs_bytes = b->segs.size() * sizeof(SegDev);
  const size_t set_bytes = 10 * q + 4 * w4 + b->counter_words * 4 + 16 * 256;
  const size_t bytes = jobs_bytes + segs_bytes + (size_t)b->nsets * set_bytes + 5 * 256;
  ct_status st;
  if ((st = path_alloc(device, bytes, b->stream, &b->d_paths)) != CT_OK) return bail(st);
  char* base = static_cast<char*>(b->d_paths);
  auto take = [&](size_t n) {
    char* p = base;
    base += (n + 255) & ~size_t(255);
    return p;
  };
  b->d_jobs = (JobDev*)take(jobs_bytes);
  b->d_segs = (SegDev*)take(segs_bytes);
  {  // both tables before the first run (a later ct_batch_set_first_frames re-uploads the chunks in stream order)
    cudaError_t err = cudaMemcpyAsync(b->d_jobs, host_jobs.data(), jobs_bytes, cudaMemcpyHostToDevice, b->stream);
    if (err == cudaSuccess && segs_bytes)
      err = cudaMemcpyAsync(b->d_segs, b->segs.data(), segs_bytes, cudaMemcpyHostToDevice, b->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(b->stream);
    if (err != cudaSuccess) return bail(fail(CT_ERR_CUDA, "batch upload: %s", cudaGetErrorString(err)));
    b->segs_dirty = false;
  }
  for (int set = 0; set < b->nsets; set++) {
    WaveArgs& a = b->sets[set];
    a.cur = Queue{(float4*)take(q), (float4*)take(q), (float4*)take(q), (uint32_t*)take(w4)};
    a.next = Queue{(float4*)take(q), (float4*)take(q), (float4*)take(q), (uint32_t*)take(w4)};
    a.shadow = ShadowQueue{(float4*)take(q), (float4*)take(q), (float4*)take(q)};
    a.radiance = (float4*)take(q);
    a.hit_prim = (int32_t*)take(w4);
    a.hit_t = (float*)take(w4);
    a.counts = (uint32_t*)take(b->counter_words * 4);
    a.jobs = b->d_jobs;
    a.max_bounces = o->max_bounces;
    a.rr = o->russian_roulette;
    a.nee = o->nee;
  }
  *out = b;
  return CT_OK;
}

ct_status run(ct_batch* b, cudaStream_t s, bool direct, const ct_batch* after = nullptr) {
  CT_CUDA(cudaSetDevice(b->device));
  if (b->segs_dirty && !b->segs.empty()) {
    CT_CUDA(cudaMemcpyAsync(b->d_segs, b->segs.data(), b->segs.size() * sizeof(SegDev), cudaMemcpyHostToDevice, s));
    b->segs_dirty = false;
  }
  if (b->waves.empty()) return CT_OK;
  if (direct) {  // launches straight onto s (no capture): for one-shot batches
    ProfScope ps("batch_direct", s);
    ct_status st = enqueue_all(b, s, true, after);
    if (st != CT_OK) return st;
    CT_CUDA(cudaEventRecord(b->done, s));
    return CT_OK;
  }
  if (!b->exec) {
    (void)grids<true>();  // occupancy queries before capture
    cudaStream_t cap = b->stream;
    CT_CUDA(cudaStreamSynchronize(s));  // the segment upload above precedes the capture
    CT_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    ct_status st = enqueue_all(b, cap);
    cudaGraph_t graph = nullptr;
    cudaError_t err = cudaStreamEndCapture(cap, &graph);
    if (st != CT_OK) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    if (err != cudaSuccess) return fail(CT_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(err));
    b->graph = graph;
    CT_CUDA(cudaGraphGetNodes(graph, nullptr, &b->graph_nodes));
    CT_CUDA(cudaGraphInstantiate(&b->exec, graph, 0));
  }
  {
    ProfScope ps("batch_graph", s);
    CT_CUDA(cudaGraphLaunch(b->exec, s));
  }
  CT_CUDA(cudaEventRecord(b->done, s));
  return CT_OK;
}

}  // namespace
}  // namespace ct

extern "C" {

ct_status ct_batch_create(const ct_batch_job* jobs, uint32_t count, const ct_trace_options* opts, int64_t wave_paths,
                          int32_t walk, ct_batch** out) {
  ct::clear_error();
  if (out) *out = nullptr;
  try {
    return ct::create(jobs, count, opts, wave_paths, walk, out);
  } catch (const std::bad_alloc&) {
    return ct::fail(CT_ERR_OUT_OF_MEMORY, "ct_batch_create: host allocation failed");
  }
}

ct_status ct_batch_set_first_frames(ct_batch* batch, const uint32_t* first_frame_index) {
  ct::clear_error();
  CT_CHECK_ARG(batch != nullptr && first_frame_index != nullptr, "NULL argument");
  for (size_t i = 0; i < batch->segs.size(); i++)
    batch->segs[i].frame_index = first_frame_index[batch->segs[i].job] + batch->seg_pass[i];
  batch->segs_dirty = true;
  return CT_OK;
}

ct_status ct_batch_run(ct_batch* batch, void* stream) {
  ct::clear_error();
  CT_CHECK_ARG(batch != nullptr, "batch is NULL");
  return ct::run(batch, stream ? static_cast<cudaStream_t>(stream) : batch->stream, false);
}

ct_status ct_batch_run_direct(ct_batch* batch, void* stream) {
  ct::clear_error();
  CT_CHECK_ARG(batch != nullptr, "batch is NULL");
  return ct::run(batch, stream ? static_cast<cudaStream_t>(stream) : batch->stream, true);
}

ct_status ct_batch_run_direct_after(ct_batch* batch, void* stream, const ct_batch* after) {
  ct::clear_error();
  CT_CHECK_ARG(batch != nullptr, "batch is NULL");
  CT_CHECK_ARG(after == nullptr || after->device == batch->device, "batches live on different devices");
  return ct::run(batch, stream ? static_cast<cudaStream_t>(stream) : batch->stream, true, after);
}

ct_status ct_batch_info(const ct_batch* batch, uint32_t* waves, uint64_t* paths, uint64_t* graph_nodes,
                        int32_t* walk) {
  ct::clear_error();
  CT_CHECK_ARG(batch != nullptr, "batch is NULL");
  if (waves) *waves = (uint32_t)batch->waves.size();
  if (paths) *paths = batch->total_paths;
  if (graph_nodes) *graph_nodes = batch->graph_nodes;
  if (walk) *walk = batch->walk;
  return CT_OK;
}

void ct_batch_destroy(ct_batch* batch) { ct::destroy(batch); }

}  // extern "C"
