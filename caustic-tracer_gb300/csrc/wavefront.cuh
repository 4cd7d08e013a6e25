// Wavefront kernels of the path integrator (tracer.ts:191-395), shared by the
// single-scene renderer (integrator.cu) and the multi-scene batch renderer
// (batch.cu).
//
// A wave holds a set of paths, one per (job, pass, pixel), and runs bounce by
// bounce:
//   k_generate   camera rays (Rng.fromPixel, jitter, thin lens) -> path queue 0
//   k_trace      closest hit for the path queue of bounce b, fused with the
//                any-hit shadow rays queued by bounce b-1 (adds their
//                contribution when unoccluded)
//   k_shade      emission x MIS weight, Lambertian+NEE / metal / dielectric
//                scattering, Russian roulette; compacts the surviving paths
//                into the next queue and the NEE rays into the shadow queue
//   k_trace      the last bounce's shadow rays
//   k_accumulate adds each pixel's samples, in pass order, to its sum buffer
//                (non-finite samples dropped, tracer.ts:388)
// Queues are compacted with warp ballots, an intra-block prefix sum over the
// warp counts and one atomicAdd per block, so each block appends a
// contiguous, ordered run and the next kernel reads the path state coalesced.
// Queue lengths live in device memory: kernels run on persistent grids and
// read their own trip counts, so a wave needs no host synchronisation and a
// whole render can be captured in a CUDA graph.
//
// BATCH = false: every path belongs to one scene (WaveArgs::scene); path ids
// are pass * pixels + pixel. BATCH = true: paths of many jobs share the wave;
// segments map path ranges to (job, pass, pixel range) and each queue slot
// carries its job, whose record holds the scene, sky, camera and output.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "integrator.cuh"

namespace ct {
namespace {

constexpr int kBlock = 128;
constexpr int kWarps = kBlock / 32;

// Path state of one queue slot (3 x 16 bytes, read and written coalesced):
//   a = origin.xyz, rng state      b = dir.xyz, pdf (< 0: last bounce specular)
//   c = throughput.rgb, path id
struct Queue {
  float4* a;
  float4* b;
  float4* c;
  uint32_t* job;  // BATCH: job of each slot
};

// One NEE shadow ray: a = origin.xyz, tmax; b = dir.xyz, path id;
// c = contribution.rgb, job (BATCH).
struct ShadowQueue {
  float4* a;
  float4* b;
  float4* c;
};

struct SkyF {
  float zenith[3], horizon[3], strength;
  int32_t kind;
};

// One render job of a batch: scene, sky, camera, image size and sum buffer.
struct JobDev {
  ctk::SceneDev scene;
  SkyF sky;
  ctk::FrameF frame;
  uint32_t width, height;
  float* accum;
};

// One chunk of a wave: `passes` consecutive passes (frame indices
// frame_index, frame_index+1, ...) over pixels [pixel0, pixel0+npix) of `job`,
// laid out pass-major at paths [path0, path0 + passes*npix). Its pixels are
// accumulation items [acc0, acc0 + npix) of the wave. A wave holds at most
// one chunk of any job, so no two chunks add to the same pixel.
struct SegDev {
  uint32_t job, frame_index, pixel0, path0, npix, passes, acc0, pad;
};

struct WaveArgs {
  ctk::SceneDev scene;   // !BATCH
  SkyF sky;              // !BATCH
  ctk::FrameF frame;     // !BATCH
  Queue cur, next;
  ShadowQueue shadow;
  int32_t* hit_prim;
  float* hit_t;
  float4* radiance;      // per path id: accumulated L (w unused)
  uint32_t* counts;      // queue sizes and counters, layout in wave_counter_words
  uint32_t width, height, pixels, paths, first_frame;  // !BATCH (paths: both)
  int32_t max_bounces, rr, nee;
  // BATCH
  const JobDev* jobs;
  const SegDev* segs;
  uint32_t nsegs;
  uint32_t acc_items;    // pixels of all chunks of the wave
};

// Counter words of a wave: [0, B+2) path queue sizes, [B+2, 2B+4) shadow
// queue sizes, 2B+6 float64 fallbacks, [2B+8, 3B+10) persistent-walk work
// counters.
inline size_t wave_counter_words(int32_t max_bounces) { return 3 * (size_t)max_bounces + 12; }

// Block-wide stream compaction of two predicates at once: warp ballots, an
// intra-block prefix sum over the warp counts and one atomicAdd per counter
// per block, so the block's survivors of each predicate land contiguously.
// Returns slot_a in *counter_a (valid when pa) and slot_b in *counter_b
// (valid when pb). s_warp holds 2*kWarps words, s_base two.
__device__ __forceinline__ void block_append2(bool pa, bool pb, uint32_t* counter_a, uint32_t* counter_b,
                                              uint32_t* s_warp, uint32_t* s_base, uint32_t& slot_a,
                                              uint32_t& slot_b) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t ma = __ballot_sync(0xffffffffu, pa), mb = __ballot_sync(0xffffffffu, pb);
  if (lane == 0) {
    s_warp[warp] = __popc(ma);
    s_warp[kWarps + warp] = __popc(mb);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t ta = 0, tb = 0;
    for (int w = 0; w < kWarps; w++) {
      const uint32_t ca = s_warp[w], cb = s_warp[kWarps + w];
      s_warp[w] = ta;
      s_warp[kWarps + w] = tb;
      ta += ca;
      tb += cb;
    }
    s_base[0] = ta ? atomicAdd(counter_a, ta) : 0u;
    s_base[1] = tb ? atomicAdd(counter_b, tb) : 0u;
  }
  __syncthreads();
  slot_a = s_base[0] + s_warp[warp] + __popc(ma & lt);
  slot_b = s_base[1] + s_warp[kWarps + warp] + __popc(mb & lt);
  __syncthreads();
}

// Chunk holding path p (KEY = path0) or accumulation item p (KEY = acc0);
// chunks are sorted by both, the first at 0.
template <uint32_t SegDev::*KEY>
__device__ __forceinline__ uint32_t find_segment(const SegDev* segs, uint32_t nsegs, uint32_t p) {
  uint32_t lo = 0, hi = nsegs;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&(segs[mid].*KEY)) <= p) lo = mid;
    else hi = mid;
  }
  return lo;
}

// The camera ray of one path (accumulatePass per pixel, tracer.ts:361-395):
// jitter, optional lens sample and camera_ray, from Rng.fromPixel(pixel,
// frame_index); the path's queue state (a, b, c) with unit throughput.
__device__ __forceinline__ void generate_path(const ctk::FrameF& frame, uint32_t width, uint32_t height,
                                              uint32_t pixel, uint32_t frame_index, uint32_t pid, float4& qa,
                                              float4& qb, float4& qc) {
  const uint32_t y = pixel / width, x = pixel - y * width;
  uint32_t rng = ctk::seed_for(pixel, frame_index);
  const float jx = ctk::next_f(rng);
  const float jy = ctk::next_f(rng);
  const float sx = ((float)x + jx) / (float)width;
  const float sy = 1.0f - ((float)y + jy) / (float)height;
  float lx = 0.0f, ly = 0.0f;
  if (frame.lens_radius > 0.0f) {
    const float r = sqrtf(ctk::next_f(rng));
    float sp, cp;
    sincospif(2.0f * ctk::next_f(rng), &sp, &cp);
    lx = r * cp;
    ly = r * sp;
  }
  ctk::V3f o, d;
  ctk::camera_ray(frame, sx, sy, lx, ly, o, d);
  qa = make_float4(o.x, o.y, o.z, __uint_as_float(rng));
  qb = make_float4(d.x, d.y, d.z, -1.0f);
  qc = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(pid));
}


template <bool BATCH>
__global__ void __launch_bounds__(kBlock) k_generate(WaveArgs a) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.paths; p += stride) {
    uint32_t pixel, frame_index, width, height, job = 0;
    const ctk::FrameF* frame;
    if constexpr (BATCH) {
      const SegDev& sg = a.segs[find_segment<&SegDev::path0>(a.segs, a.nsegs, p)];
      job = sg.job;
      const uint32_t off = p - sg.path0, k = off / sg.npix;
      pixel = sg.pixel0 + (off - k * sg.npix);
      frame_index = sg.frame_index + k;
      const JobDev& j = a.jobs[job];
      width = j.width;
      height = j.height;
      frame = &j.frame;
      a.cur.job[p] = job;
    } else {
      const uint32_t pass = p / a.pixels;
      pixel = p - pass * a.pixels;
      frame_index = a.first_frame + pass;
      width = a.width;
      height = a.height;
      frame = &a.frame;
    }
    float4 qa, qb, qc;
    generate_path(*frame, width, height, pixel, frame_index, p, qa, qb, qc);
    a.cur.a[p] = qa;
    a.cur.b[p] = qb;
    a.cur.c[p] = qc;
    a.radiance[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.counts[0] = a.paths;
}

// Walk forms of the trace kernel (chosen per scene by the host):
//   kWalkThread     ordered walk, one per thread in a grid-stride loop;
//   kWalkPersistent ordered walk, lanes refill from a work counter as their
//                   walks finish (the default above 31 nodes);
//   kWalkSkip       the reference's stackless skip-link walk (no stack; all
//                   lanes visit nodes in the same order; for small trees;
//                   scenes of <= 32 primitives test every primitive in the
//                   order the walk would, without boxes);
//   kWalkPerJob     BATCH only, a planning mode: each job walks as its scene
//                   does alone; a wave holds jobs of one walk and runs its
//                   kernel.
enum WalkForm : int { kWalkThread = 0, kWalkPersistent = 1, kWalkSkip = 2, kWalkPerJob = 3 };

// Closest hits of the bounce-b path queue plus the shadow rays of bounce b-1.
// Blocks of 128 per SM, measured per walk form: the ordered walk per thread
// at 16 (32 registers), the persistent ordered walk of one scene at 10 (48
// registers, no spills: caustic scene 2,020 against 1,986 Msamples/s at 12
// blocks and 1,894 at 16, the 100k soup 567 against 544) and of a batch at
// 12 (40 registers; batched soups 1,335 against 1,320 at 10), the skip-link
// walk at 8 (it keeps its registers).
template <int FORM, bool BATCH>
constexpr int trace_min_blocks() { return FORM == 2 ? 8 : FORM == 1 ? (BATCH ? 12 : 10) : 16; }

template <int FORM, bool BATCH>
__global__ void __launch_bounds__(kBlock, trace_min_blocks<FORM, BATCH>()) k_trace(WaveArgs a, int32_t bounce) {
  const uint32_t n_ext = bounce <= a.max_bounces ? a.counts[bounce] : 0u;
  const uint32_t n_sh = bounce > 0 ? a.counts[a.max_bounces + 2 + bounce - 1] : 0u;
  uint32_t fallbacks = 0;
  // Query i < n_ext: closest hit of path slot i; otherwise shadow ray i - n_ext.
  auto load = [&](uint32_t i, ctk::RayF& r) {
    if (i < n_ext) {
      const float4 ra = __ldcs(&a.cur.a[i]), rb = __ldcs(&a.cur.b[i]);  // streamed: touched once
      r = ctk::RayF{ra.x, ra.y, ra.z, rb.x, rb.y, rb.z, ctk::kTMin, INFINITY, 0.0f, 0.0f, 0.0f};
    } else {
      const uint32_t j = i - n_ext;
      const float4 sa = __ldcs(&a.shadow.a[j]), sb = __ldcs(&a.shadow.b[j]);
      r = ctk::RayF{sa.x, sa.y, sa.z, sb.x, sb.y, sb.z, ctk::kTMin, sa.w, 0.0f, 0.0f, 0.0f};
    }
    ctk::finish_ray(r);
  };
  auto job_of = [&](uint32_t i) -> const JobDev& {
    return a.jobs[i < n_ext ? a.cur.job[i] : __float_as_uint(a.shadow.c[i - n_ext].w)];
  };
  auto finish = [&](uint32_t i, ctk::Walk& w) {
    if (i < n_ext) {
      __stcs(&a.hit_prim[i], w.h.prim);
      __stcs(&a.hit_t[i], w.h.t);
    } else if (w.h.prim < 0) {  // unoccluded: add the NEE contribution
      const uint32_t j = i - n_ext;
      const float4 c = a.shadow.c[j];
      float4* L = a.radiance + __float_as_uint(a.shadow.b[j].w);
      float4 l = *L;
      l.x += c.x;
      l.y += c.y;
      l.z += c.z;
      *L = l;
    }
  };
  // A batch query copies its job's scene record into registers once, so the
  // walk reads the base pointers as often as the single-scene kernel reads
  // its kernel parameters.
  // Walk steps per refill round (measured): one scene 8 (caustic scene 2,082
  // Msamples/s against 2,021 at 3, 2,085 at 6 and 2,020 at 12; 100k soup 591
  // against 567 at 3 and 595 at 12), a batch of soups 12 (1,406 against 1,334
  // at 3 and 1,398 at 8; 1,425 at 16). Refill at 6 idle lanes: caustic
  // 2,092, soup 603, batched 1,436 against 2,092 / 599 / 1,428 at 8, 2,079 /
  // 591 / 1,404 at 12 and 2,059 / 577 / 1,370 at 16 (4 as 6 within 0.3 %).
  if constexpr (FORM == kWalkPersistent && !BATCH) {
    ctk::walk_persistent<false, 6, true, 8>(
        a.scene, a.counts + 2 * a.max_bounces + 8 + bounce, n_ext + n_sh,
        [&](uint32_t i, ctk::Walk& w) {
          load(i, w.r);
          ctk::walk_begin(a.scene, w, i >= n_ext);
        },
        finish, fallbacks);
  } else if constexpr (FORM == kWalkPersistent) {
    ctk::SceneDev lane_scene = a.jobs[0].scene;
    ctk::walk_persistent<false, 6, true, 12>(
        lane_scene, a.counts + 2 * a.max_bounces + 8 + bounce, n_ext + n_sh,
        [&](uint32_t i, ctk::Walk& w) {
          load(i, w.r);
          lane_scene = job_of(i).scene;
          ctk::walk_begin(lane_scene, w, i >= n_ext);
        },
        finish, fallbacks);
  } else {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_ext + n_sh; i += stride) {
      ctk::Walk w;
      ctk::WalkStack st;
      load(i, w.r);
      const ctk::SceneDev sc = BATCH ? job_of(i).scene : a.scene;
      if constexpr (FORM == kWalkSkip) {
        w.h = ctk::HitF{-1, w.r.tmax, 0.0f, 0.0f, 0.0f};
        if (sc.prim_count <= ctk::kBrutePrims)
          ctk::walk_all<false>(sc, w.r, w.h, i >= n_ext, fallbacks);
        else
          ctk::walk_stackless<false>(sc, w.r, w.h, i >= n_ext, fallbacks);
      } else {
        ctk::walk_begin(sc, w, i >= n_ext);
        while (w.c.ref != ctk::kWalkDone) ctk::walk_step<false>(sc, w, st, fallbacks);
      }
      finish(i, w);
    }
  }
  if (fallbacks) atomicAdd(a.counts + 2 * a.max_bounces + 6, fallbacks);
}

// Result of shading one path-bounce: the continuing path's state (cont),
// the NEE shadow ray and its contribution (shadow), and the radiance
// (emission or sky) to add to the path now.
struct ShadeOut {
  bool cont, shadow;
  float4 na, nb, nc, sa, sb, scol;
  float lr, lg, lb;
};

// One bounce of radianceInto (tracer.ts:191-328) for a path whose closest
// hit is (prim, t) (prim < 0: miss): emission with its MIS weight, the
// material's scatter (Lambertian with NEE, metal, dielectric), Russian
// roulette. k_shade and the brute-force path kernel both run it, so the two
// take the same float operations in the same order.
__device__ __forceinline__ void shade_path(const ctk::SceneDev& sc, const SkyF& sky, uint32_t job, float4 qa,
                                           float4 qb, float4 qc, int32_t prim, float t, int32_t bounce,
                                           int32_t max_bounces, int32_t rr, int32_t nee, ShadeOut& out) {
  out.cont = out.shadow = false;
  out.na = out.nb = out.nc = out.sa = out.sb = out.scol = make_float4(0, 0, 0, 0);
  out.lr = out.lg = out.lb = 0.0f;
  const bool use_nee = nee != 0 && sc.light_count > 0;
  uint32_t rng = __float_as_uint(qa.w);
  const uint32_t pid = __float_as_uint(qc.w);
  const ctk::V3f o = ctk::mk(qa.x, qa.y, qa.z), d = ctk::mk(qb.x, qb.y, qb.z);
  float pdf = qb.w;
  float tr = qc.x, tg = qc.y, tb = qc.z;
  if (prim < 0) {
    if (sky.kind == 1) {  // tracer.ts:210-218
      const float f = 0.5f * (d.y + 1.0f);
      out.lr = tr * (sky.horizon[0] + (sky.zenith[0] - sky.horizon[0]) * f) * sky.strength;
      out.lg = tg * (sky.horizon[1] + (sky.zenith[1] - sky.horizon[1]) * f) * sky.strength;
      out.lb = tb * (sky.horizon[2] + (sky.zenith[2] - sky.horizon[2]) * f) * sky.strength;
    }
  } else {
    const float4* q = sc.prims + (size_t)prim * 4;
    const float4 q0 = __ldg(q);
    const ctk::V3f p = ctk::madd3(o, d, t);
    ctk::V3f nrm;
    if (q0.w == 0.0f) {
      const float inv_r = 1.0f / __ldg(q + 1).x;
      nrm = ctk::mk((p.x - q0.x) * inv_r, (p.y - q0.y) * inv_r, (p.z - q0.z) * inv_r);
    } else {
      const float4 q3 = __ldg(q + 3);
      nrm = ctk::mk(q3.x, q3.y, q3.z);
    }
    const bool front = ctk::dot3(d, nrm) < 0.0f;
    const ctk::V3f s = front ? nrm : ctk::mk(-nrm.x, -nrm.y, -nrm.z);
    const float4* m = sc.mats + (size_t)__ldg(sc.prim_object + prim) * 4;
    const float4 m0 = __ldg(m), m3 = __ldg(m + 3);
    if (m3.x > 0.0f || m3.y > 0.0f || m3.z > 0.0f) {  // tracer.ts:243-252
      float w = 1.0f;
      if (use_nee && pdf >= 0.0f) w = ctk::power_heuristic(pdf, ctk::light_pdf(sc, o, p, nrm, prim));
      out.lr = tr * m3.x * w;
      out.lg = tg * m3.y * w;
      out.lb = tb * m3.z * w;
    }
    const int type = (int)m0.w;
    ctk::V3f nd = d;
    if (type == CT_MAT_LAMBERTIAN) {
      const float4 m1 = __ldg(m + 1);
      float ar = m0.x, ag = m0.y, ab = m0.z;
      if (m1.z > 0.5f && !ctk::checker_primary(p, m1.y)) {
        const float4 m2 = __ldg(m + 2);
        ar = m2.x, ag = m2.y, ab = m2.z;
      }
      ctk::LightSample ls;
      if (use_nee && ctk::sample_light(sc, p, rng, ls)) {  // tracer.ts:263-274
        const float cos_s = ctk::dot3(s, ls.dir);
        if (cos_s > 0.0f && ls.pdf > 0.0f) {
          const float pdf_b = cos_s * ctk::kInvPi;
          const float k = __fdividef(cos_s * ctk::kInvPi * ctk::power_heuristic(ls.pdf, pdf_b), ls.pdf);
          out.shadow = true;
          out.sa = make_float4(p.x, p.y, p.z, ls.dist * ctk::kShadowShorten);
          out.sb = make_float4(ls.dir.x, ls.dir.y, ls.dir.z, __uint_as_float(pid));
          out.scol = make_float4(tr * ar * ls.emission.x * k, tg * ag * ls.emission.y * k,
                                 tb * ab * ls.emission.z * k, __uint_as_float(job));
        }
      }
      const float u1 = ctk::next_f(rng);
      const float u2 = ctk::next_f(rng);
      nd = ctk::cosine_hemisphere(s, u1, u2);
      pdf = fmaxf(0.0f, ctk::dot3(s, nd)) * ctk::kInvPi;
      tr *= ar, tg *= ag, tb *= ab;
      out.cont = true;
    } else if (type == CT_MAT_METAL) {
      const float u1 = ctk::next_f(rng);
      const float u2 = ctk::next_f(rng);
      const float u3 = ctk::next_f(rng);
      nd = ctk::metal_dir(d, s, __ldg(m + 1).x, u1, u2, u3);
      if (ctk::dot3(nd, s) > 0.0f) {
        tr *= m0.x, tg *= m0.y, tb *= m0.z;
        pdf = -1.0f;
        out.cont = true;
      }
    } else if (type == CT_MAT_DIELECTRIC) {
      const float u = ctk::next_f(rng);
      nd = ctk::dielectric_dir(d, s, __ldg(m + 1).x, front, u);
      tr *= m0.x, tg *= m0.y, tb *= m0.z;
      pdf = -1.0f;
      out.cont = true;
    }
    if (out.cont && rr && bounce >= 3) {  // tracer.ts:305-312
      const float max_b = fmaxf(tr, fmaxf(tg, tb));
      const float ps = max_b > 1.0f ? 1.0f : (max_b < 0.05f ? 0.05f : max_b);
      if (ctk::next_f(rng) > ps) {
        out.cont = false;
      } else {
        tr /= ps, tg /= ps, tb /= ps;
      }
    }
    if (bounce >= max_bounces) out.cont = false;
    out.na = make_float4(p.x, p.y, p.z, __uint_as_float(rng));
    out.nb = make_float4(nd.x, nd.y, nd.z, pdf);
    out.nc = make_float4(tr, tg, tb, __uint_as_float(pid));
  }
}

// 10 blocks of 128 per SM (48 registers, ~50 bytes spilled): 3 % faster on
// the Cornell box than 8 blocks at 64 registers.
template <bool BATCH>
__global__ void __launch_bounds__(kBlock, 10) k_shade(WaveArgs a, int32_t bounce) {
  __shared__ uint32_t s_warp[2 * kWarps], s_base[2];
  const uint32_t n = a.counts[bounce];
  uint32_t* next_count = a.counts + bounce + 1;
  uint32_t* shadow_count = a.counts + a.max_bounces + 2 + bounce;
  for (uint32_t base = blockIdx.x * kBlock; base < n; base += gridDim.x * kBlock) {
    const uint32_t i = base + threadIdx.x;
    bool cont = false, shadow = false;
    uint32_t job = 0;
    float4 na = make_float4(0, 0, 0, 0), nb = na, nc = na, sa = na, sb = na, scol = na;
    if (i < n) {
      const SkyF* sky = &a.sky;
      if constexpr (BATCH) {
        job = a.cur.job[i];
        sky = &a.jobs[job].sky;
      }
      const ctk::SceneDev sc = BATCH ? a.jobs[job].scene : a.scene;  // registers, loaded up front
      const float4 qa = a.cur.a[i], qb = a.cur.b[i], qc = a.cur.c[i];
      const int32_t prim = a.hit_prim[i];
      const float t = prim >= 0 ? a.hit_t[i] : 0.0f;
      ShadeOut so;
      shade_path(sc, *sky, job, qa, qb, qc, prim, t, bounce, a.max_bounces, a.rr, a.nee, so);
      cont = so.cont, shadow = so.shadow;
      na = so.na, nb = so.nb, nc = so.nc, sa = so.sa, sb = so.sb, scol = so.scol;
      const float lr = so.lr, lg = so.lg, lb = so.lb;
      const uint32_t pid = __float_as_uint(qc.w);
      if (lr != 0.0f || lg != 0.0f || lb != 0.0f) {
        float4* L = a.radiance + pid;
        float4 l = *L;
        l.x += lr;
        l.y += lg;
        l.z += lb;
        *L = l;
      }
    }
    uint32_t slot, sslot;
    block_append2(cont, shadow, next_count, shadow_count, s_warp, s_base, slot, sslot);
    if (cont) {
      a.next.a[slot] = na;
      a.next.b[slot] = nb;
      a.next.c[slot] = nc;
      if constexpr (BATCH) a.next.job[slot] = job;
    }
    if (shadow) {
      a.shadow.a[sslot] = sa;
      a.shadow.b[sslot] = sb;
      a.shadow.c[sslot] = scol;
    }
  }
}

// Whole paths of a single scene of at most kBrutePrims primitives, one lane
// per path: generate_path, then per bounce the closest hit (walk_all),
// shade_path, and at once the NEE shadow ray (walk_all, any hit). The path's
// radiance receives the same additions in the same order as through the
// wavefront kernels (bounce b's emission, then its shadow contribution, then
// bounce b+1's emission), so the sums are bit for bit those of
// k_generate/k_trace/k_shade, and the path's total goes to radiance[p] for
// k_accumulate. The scene is read from L1; no path state leaves the SM.
// Lanes whose paths end take new ones from a work counter (a.counts[0])
// once kPathRefill lanes of the warp are idle. 9 blocks of 128 per SM (56
// registers) and refill at 4 idle lanes (Cornell box, measured): 8 blocks
// (64 registers) 2,142 Msamples/s at 8 lanes; 10 blocks (48 registers,
// spilling) 2,297 at 4 lanes, 9 blocks 2,318; 11 or 12 blocks 2,090;
// refill at 16 lanes 1,994, at 1 or 2 lanes 2,256-2,260.
constexpr uint32_t kPathRefill = 4;

__global__ void __launch_bounds__(kBlock, 9) k_paths(WaveArgs a) {
  const uint32_t lane = threadIdx.x & 31u, lt_mask = (1u << lane) - 1u;
  const ctk::SceneDev& sc = a.scene;
  uint32_t fallbacks = 0;
  float4 qa = make_float4(0, 0, 0, 0), qb = qa, qc = qa;
  float lr = 0.0f, lg = 0.0f, lb = 0.0f;
  int32_t bounce = -1;  // < 0: no path
  uint32_t p = 0;
  bool drained = false;
  for (;;) {
    const bool idle = bounce < 0;
    const uint32_t want = __ballot_sync(0xffffffffu, idle);
    if (!drained && (__popc(want) >= kPathRefill || want == 0xffffffffu)) {
      const uint32_t leader = __ffs(want) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(a.counts, (uint32_t)__popc(want));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + __popc(want) >= a.paths) drained = true;
      if (idle) {
        const uint32_t k = base + __popc(want & lt_mask);
        if (k < a.paths) {
          p = k;
          const uint32_t pass = p / a.pixels;
          generate_path(a.frame, a.width, a.height, p - pass * a.pixels, a.first_frame + pass, p, qa, qb, qc);
          lr = lg = lb = 0.0f;
          bounce = 0;
        }
      }
    }
    if (drained && __all_sync(0xffffffffu, bounce < 0)) break;
    if (bounce < 0) continue;
    // walk_all tests primitives only: the inverse direction is not needed
    ctk::RayF r{qa.x, qa.y, qa.z, qb.x, qb.y, qb.z, ctk::kTMin, INFINITY, 0.0f, 0.0f, 0.0f};
    ctk::HitF h{-1, r.tmax, 0.0f, 0.0f, 0.0f};
    ctk::walk_all<false>(sc, r, h, false, fallbacks);
    ShadeOut so;
    shade_path(sc, a.sky, 0, qa, qb, qc, h.prim, h.t, bounce, a.max_bounces, a.rr, a.nee, so);
    if (so.lr != 0.0f || so.lg != 0.0f || so.lb != 0.0f) lr += so.lr, lg += so.lg, lb += so.lb;
    if (so.shadow) {
      ctk::RayF sr{so.sa.x, so.sa.y, so.sa.z, so.sb.x, so.sb.y, so.sb.z, ctk::kTMin, so.sa.w, 0.0f, 0.0f, 0.0f};
      ctk::HitF sh{-1, sr.tmax, 0.0f, 0.0f, 0.0f};
      ctk::walk_all<false>(sc, sr, sh, true, fallbacks);
      if (sh.prim < 0) lr += so.scol.x, lg += so.scol.y, lb += so.scol.z;
    }
    if (so.cont) {
      qa = so.na, qb = so.nb, qc = so.nc;
      bounce++;
    } else {
      a.radiance[p] = make_float4(lr, lg, lb, 0.0f);
      bounce = -1;
    }
  }
}

// Single scene: adds the wave's `passes` samples of each pixel, in pass order.
__global__ void __launch_bounds__(kBlock) k_accumulate(const float4* __restrict__ radiance, uint32_t pixels,
                                                       uint32_t passes, float* __restrict__ accum,
                                                       float* __restrict__ sumsq) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t px = blockIdx.x * blockDim.x + threadIdx.x; px < pixels; px += stride) {
    float r = accum[3 * (size_t)px], g = accum[3 * (size_t)px + 1], b = accum[3 * (size_t)px + 2];
    float qr = 0, qg = 0, qb = 0;
    if (sumsq) qr = sumsq[3 * (size_t)px], qg = sumsq[3 * (size_t)px + 1], qb = sumsq[3 * (size_t)px + 2];
    for (uint32_t s = 0; s < passes; s++) {
      const float4 l = radiance[(size_t)s * pixels + px];
      if (isfinite(l.x) && isfinite(l.y) && isfinite(l.z)) {
        r += l.x, g += l.y, b += l.z;
        qr += l.x * l.x, qg += l.y * l.y, qb += l.z * l.z;
      }
    }
    accum[3 * (size_t)px] = r, accum[3 * (size_t)px + 1] = g, accum[3 * (size_t)px + 2] = b;
    if (sumsq) sumsq[3 * (size_t)px] = qr, sumsq[3 * (size_t)px + 1] = qg, sumsq[3 * (size_t)px + 2] = qb;
  }
}

// Batch: each pixel of each chunk adds its chunk's samples, in pass order,
// to its job's sum (the same sequence of float additions as k_accumulate).
__global__ void __launch_bounds__(kBlock) k_accumulate_batch(WaveArgs a) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.acc_items; i += stride) {
    const SegDev& sg = a.segs[find_segment<&SegDev::acc0>(a.segs, a.nsegs, i)];
    const uint32_t local = i - sg.acc0;
    float* acc = a.jobs[sg.job].accum + 3 * (size_t)(sg.pixel0 + local);
    float r = acc[0], g = acc[1], b = acc[2];
    const float4* l = a.radiance + sg.path0 + local;
    for (uint32_t k = 0; k < sg.passes; k++, l += sg.npix) {
      const float4 v = *l;
      if (isfinite(v.x) && isfinite(v.y) && isfinite(v.z)) r += v.x, g += v.y, b += v.z;
    }
    acc[0] = r;
    acc[1] = g;
    acc[2] = b;
  }
}

__global__ void k_scale(float* __restrict__ v, size_t n, float div) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) v[i] = v[i] / div;
}

template <class K>
int persistent_grid(K kernel) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0);
  return sms * std::max(1, per_sm);
}

template <bool BATCH>
struct Grids {
  int gen = 0, trace[4] = {0, 0, 0, 0}, shade = 0, acc = 0, paths = 0, sms = 1;
  // `full` (the kernel's SMs x occupancy) capped at `blocks` per SM (0: uncapped).
  int capped(int full, int blocks) const { return blocks > 0 ? std::min(full, sms * blocks) : full; }
};

template <bool BATCH>
const Grids<BATCH>& grids() {
  static Grids<BATCH> g = [] {
    Grids<BATCH> r;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&r.sms, cudaDevAttrMultiProcessorCount, dev);
    r.sms = std::max(1, r.sms);
    r.gen = persistent_grid(k_generate<BATCH>);
    r.trace[kWalkThread] = persistent_grid(k_trace<kWalkThread, BATCH>);
    r.trace[kWalkPersistent] = persistent_grid(k_trace<kWalkPersistent, BATCH>);
    r.trace[kWalkSkip] = persistent_grid(k_trace<kWalkSkip, BATCH>);
    r.shade = persistent_grid(k_shade<BATCH>);
    r.acc = BATCH ? persistent_grid(k_accumulate_batch) : persistent_grid(k_accumulate);
    if (!BATCH) r.paths = persistent_grid(k_paths);
    return r;
  }();
  return g;
}

template <bool BATCH>
void launch_trace(int form, const WaveArgs& w, int32_t bounce, cudaStream_t stream, int blocks_per_sm = 0) {
  const Grids<BATCH>& g = grids<BATCH>();
  switch (form) {
    case kWalkPersistent:
      k_trace<kWalkPersistent, BATCH><<<g.capped(g.trace[kWalkPersistent], blocks_per_sm), kBlock, 0, stream>>>(
          w, bounce);
      break;
    default:
      k_trace<kWalkThread, BATCH><<<g.capped(g.trace[kWalkThread], blocks_per_sm), kBlock, 0, stream>>>(w, bounce);
      break;
    case kWalkSkip:
      k_trace<kWalkSkip, BATCH><<<g.capped(g.trace[kWalkSkip], blocks_per_sm), kBlock, 0, stream>>>(w, bounce);
      break;
  }
}

inline ctk::FrameF to_frame(const ct_camera_frame& f) {
  ctk::FrameF r;
  r.ox = (float)f.origin[0], r.oy = (float)f.origin[1], r.oz = (float)f.origin[2];
  r.rx = (float)f.right[0], r.ry = (float)f.right[1], r.rz = (float)f.right[2];
  r.ux = (float)f.up[0], r.uy = (float)f.up[1], r.uz = (float)f.up[2];
  r.fx = (float)f.forward[0], r.fy = (float)f.forward[1], r.fz = (float)f.forward[2];
  r.tan_half_fov = (float)f.tan_half_fov;
  r.aspect = (float)f.aspect;
  r.lens_radius = (float)f.lens_radius;
  r.focus_distance = (float)f.focus_distance;
  return r;
}

inline SkyF to_sky(const ct_sky& s) {
  SkyF r;
  r.kind = s.kind;
  for (int k = 0; k < 3; k++) {
    r.zenith[k] = (float)s.zenith[k];
    r.horizon[k] = (float)s.horizon[k];
  }
  r.strength = (float)s.strength;
  return r;
}

inline ct_status check_options(const ct_camera_frame* frame, int32_t width, int32_t height, int32_t max_bounces) {
  CT_CHECK_ARG(frame != nullptr, "frame is NULL");
  CT_CHECK_ARG(width > 0 && height > 0, "image size %dx%d is not positive", width, height);
  CT_CHECK_ARG((uint64_t)width * (uint64_t)height <= (1ull << 30), "image of %dx%d pixels is too large", width, height);
  CT_CHECK_ARG(max_bounces >= 0 && max_bounces <= 1024, "max_bounces %d outside [0, 1024]", max_bounces);
  const double* v = frame->origin;
  for (int k = 0; k < 16; k++)
    CT_CHECK_ARG(std::isfinite(v[k]), "camera frame has a non-finite value");
  return CT_OK;
}

}  // namespace
}  // namespace ct
