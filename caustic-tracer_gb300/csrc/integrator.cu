// Wavefront path integrator: accumulatePass / renderImage (tracer.ts:191-395).
//
// A wave holds P passes of one sample per pixel (path id = pass * W*H + pixel)
// and runs bounce by bounce:
//   k_generate  camera rays (Rng.fromPixel, jitter, thin lens) -> path queue 0
//   k_trace     closest hit for the path queue of bounce b, fused with the
//               any-hit shadow rays queued by bounce b-1 (adds their
//               contribution when unoccluded)
//   k_shade     emission x MIS weight, Lambertian+NEE / metal / dielectric
//               scattering, Russian roulette; compacts the surviving paths
//               into the next queue and the NEE rays into the shadow queue
//   k_trace     the last bounce's shadow rays
//   k_accumulate adds the P samples of each pixel in pass order (non-finite
//               samples dropped, tracer.ts:388) into the float32 sum buffer
// Queues are compacted with warp ballots, an intra-block prefix sum over the
// warp counts and one atomicAdd per block, so each block appends a contiguous,
// ordered run and the next kernel reads the path state coalesced. Queue
// lengths live in device memory: kernels are launched with persistent grids
// and read their own trip count, so a wave needs no host synchronisation.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "integrator.cuh"
#include "profile.hpp"
#include "scene.hpp"


namespace ct {

namespace {

constexpr int kBlock = 128;
constexpr int kWarps = kBlock / 32;
constexpr uint64_t kMaxWavePaths = 8ull << 20;  // paths in flight per wave
constexpr uint32_t kPersistentDepth = 16;      // tree depth above which traces refill lanes
constexpr uint32_t kSkipMaxNodes = 31;         // trees this small use the stackless skip-link walk

// Path state of one queue slot (3 x 16 bytes, read and written coalesced):
//   a = origin.xyz, rng state      b = dir.xyz, pdf (< 0: last bounce specular)
//   c = throughput.rgb, path id
struct Queue {
  float4* a;
  float4* b;
  float4* c;
};

// One NEE shadow ray: a = origin.xyz, tmax; b = dir.xyz, path id; c = contribution.rgb.
struct ShadowQueue {
  float4* a;
  float4* b;
  float4* c;
};

struct WaveArgs {
  ctk::SceneDev scene;
  ctk::FrameF frame;
  Queue cur, next;
  ShadowQueue shadow;
  int32_t* hit_prim;
  float* hit_t;
  float4* radiance;      // per path id: accumulated L (w unused)
  uint32_t* counts;      // queue sizes and counters, layout in run_passes
  uint32_t width, height, pixels, paths, first_frame;
  int32_t max_bounces, rr, nee;
  float sky_zenith[3], sky_horizon[3], sky_strength;
  int32_t sky_kind;
};

// Block-wide stream compaction: returns the output slot of this thread (valid
// when pred) and appends the block's survivors contiguously with one atomic.
__device__ __forceinline__ uint32_t block_append(bool pred, uint32_t* counter, uint32_t* s_warp, uint32_t* s_base) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t mask = __ballot_sync(0xffffffffu, pred);
  const uint32_t rank = __popc(mask & ((1u << lane) - 1u));
  if (lane == 0) s_warp[warp] = __popc(mask);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t total = 0;
    for (int w = 0; w < kWarps; w++) {
      const uint32_t c = s_warp[w];
      s_warp[w] = total;
      total += c;
    }
    *s_base = total ? atomicAdd(counter, total) : 0u;
  }
  __syncthreads();
  const uint32_t slot = *s_base + s_warp[warp] + rank;
  __syncthreads();
  return slot;
}

__global__ void __launch_bounds__(kBlock) k_generate(WaveArgs a) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.paths; p += stride) {
    const uint32_t pass = p / a.pixels, pixel = p - pass * a.pixels;
    const uint32_t y = pixel / a.width, x = pixel - y * a.width;
    uint32_t rng = ctk::seed_for(pixel, a.first_frame + pass);
    const float jx = ctk::next_f(rng);
    const float jy = ctk::next_f(rng);
    const float sx = ((float)x + jx) / (float)a.width;
    const float sy = 1.0f - ((float)y + jy) / (float)a.height;
    float lx = 0.0f, ly = 0.0f;
    if (a.frame.lens_radius > 0.0f) {
      const float r = sqrtf(ctk::next_f(rng));
      float sp, cp;
      sincospif(2.0f * ctk::next_f(rng), &sp, &cp);
      lx = r * cp;
      ly = r * sp;
    }
    ctk::V3f o, d;
    ctk::camera_ray(a.frame, sx, sy, lx, ly, o, d);
    a.cur.a[p] = make_float4(o.x, o.y, o.z, __uint_as_float(rng));
    a.cur.b[p] = make_float4(d.x, d.y, d.z, -1.0f);
    a.cur.c[p] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(p));
    a.radiance[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.counts[0] = a.paths;
}

// Closest hits of the bounce-b path queue plus the shadow rays of bounce b-1.
// Walk forms (chosen per scene by the host):
//   kWalkThread     ordered walk, one per thread in a grid-stride loop;
//   kWalkPersistent ordered walk, lanes refill from a work counter as their
//                   walks finish (pays off for deep trees);
//   kWalkSkip       the reference's stackless skip-link walk (no stack; all
//                   lanes visit nodes in the same order; for small trees).
enum WalkForm : int { kWalkThread = 0, kWalkPersistent = 1, kWalkSkip = 2 };

template <int FORM>
__global__ void __launch_bounds__(kBlock, 8) k_trace(WaveArgs a, int32_t bounce) {
  const uint32_t n_ext = bounce <= a.max_bounces ? a.counts[bounce] : 0u;
  const uint32_t n_sh = bounce > 0 ? a.counts[a.max_bounces + 2 + bounce - 1] : 0u;
  uint32_t fallbacks = 0;
  // Query i < n_ext: closest hit of path slot i; otherwise shadow ray i - n_ext.
  auto load = [&](uint32_t i, ctk::RayF& r) {
    if (i < n_ext) {
      const float4 ra = a.cur.a[i], rb = a.cur.b[i];
      r = ctk::RayF{ra.x, ra.y, ra.z, rb.x, rb.y, rb.z, ctk::kTMin, INFINITY, 0.0f, 0.0f, 0.0f};
    } else {
      const uint32_t j = i - n_ext;
      const float4 sa = a.shadow.a[j], sb = a.shadow.b[j];
      r = ctk::RayF{sa.x, sa.y, sa.z, sb.x, sb.y, sb.z, ctk::kTMin, sa.w, 0.0f, 0.0f, 0.0f};
    }
    ctk::finish_ray(r);
  };
  auto begin = [&](uint32_t i, ctk::Walk& w) {
    load(i, w.r);
    ctk::walk_begin(a.scene, w, i >= n_ext);
  };
  auto finish = [&](uint32_t i, ctk::Walk& w) {
    if (i < n_ext) {
      a.hit_prim[i] = w.h.prim;
      a.hit_t[i] = w.h.t;
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
  if constexpr (FORM == kWalkPersistent) {
    ctk::walk_persistent<false>(a.scene, a.counts + 2 * a.max_bounces + 8 + bounce, n_ext + n_sh, begin, finish,
                                fallbacks);
  } else {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_ext + n_sh; i += stride) {
      ctk::Walk w;
      if constexpr (FORM == kWalkSkip) {
        load(i, w.r);
        w.h = ctk::HitF{-1, w.r.tmax, 0.0f, 0.0f, 0.0f};
        ctk::walk_stackless<false>(a.scene, w.r, w.h, i >= n_ext, fallbacks);
      } else {
        begin(i, w);
        while (w.ref != ctk::kWalkDone) ctk::walk_step<false>(a.scene, w, fallbacks);
      }
      finish(i, w);
    }
  }
  if (fallbacks) atomicAdd(a.counts + 2 * a.max_bounces + 6, fallbacks);
}

__global__ void __launch_bounds__(kBlock) k_shade(WaveArgs a, int32_t bounce) {
  __shared__ uint32_t s_warp[kWarps], s_base;
  const ctk::SceneDev& sc = a.scene;
  const uint32_t n = a.counts[bounce];
  const bool use_nee = a.nee != 0 && sc.light_count > 0;
  uint32_t* next_count = a.counts + bounce + 1;
  uint32_t* shadow_count = a.counts + a.max_bounces + 2 + bounce;
  for (uint32_t base = blockIdx.x * kBlock; base < n; base += gridDim.x * kBlock) {
    const uint32_t i = base + threadIdx.x;
    bool cont = false, shadow = false;
    float4 na = make_float4(0, 0, 0, 0), nb = na, nc = na, sa = na, sb = na, scol = na;
    if (i < n) {
      const float4 qa = a.cur.a[i], qb = a.cur.b[i], qc = a.cur.c[i];
      uint32_t rng = __float_as_uint(qa.w);
      const uint32_t pid = __float_as_uint(qc.w);
      const ctk::V3f o = ctk::mk(qa.x, qa.y, qa.z), d = ctk::mk(qb.x, qb.y, qb.z);
      float pdf = qb.w;
      float tr = qc.x, tg = qc.y, tb = qc.z;
      float lr = 0.0f, lg = 0.0f, lb = 0.0f;
      const int32_t prim = a.hit_prim[i];
      if (prim < 0) {
        if (a.sky_kind == 1) {  // tracer.ts:210-218
          const float t = 0.5f * (d.y + 1.0f);
          lr = tr * (a.sky_horizon[0] + (a.sky_zenith[0] - a.sky_horizon[0]) * t) * a.sky_strength;
          lg = tg * (a.sky_horizon[1] + (a.sky_zenith[1] - a.sky_horizon[1]) * t) * a.sky_strength;
          lb = tb * (a.sky_horizon[2] + (a.sky_zenith[2] - a.sky_horizon[2]) * t) * a.sky_strength;
        }
      } else {
        const float t = a.hit_t[i];
        const float4* q = sc.prims + (size_t)prim * 4;
        const float4 q0 = __ldg(q);
        const ctk::V3f p = ctk::mk(o.x + d.x * t, o.y + d.y * t, o.z + d.z * t);
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
          lr = tr * m3.x * w;
          lg = tg * m3.y * w;
          lb = tb * m3.z * w;
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
              const float k = (cos_s * ctk::kInvPi * ctk::power_heuristic(ls.pdf, pdf_b)) / ls.pdf;
              shadow = true;
              sa = make_float4(p.x, p.y, p.z, ls.dist * ctk::kShadowShorten);
              sb = make_float4(ls.dir.x, ls.dir.y, ls.dir.z, __uint_as_float(pid));
              scol = make_float4(tr * ar * ls.emission.x * k, tg * ag * ls.emission.y * k,
                                 tb * ab * ls.emission.z * k, 0.0f);
            }
          }
          const float u1 = ctk::next_f(rng);
          const float u2 = ctk::next_f(rng);
          nd = ctk::cosine_hemisphere(s, u1, u2);
          pdf = fmaxf(0.0f, ctk::dot3(s, nd)) * ctk::kInvPi;
          tr *= ar, tg *= ag, tb *= ab;
          cont = true;
        } else if (type == CT_MAT_METAL) {
          const float u1 = ctk::next_f(rng);
          const float u2 = ctk::next_f(rng);
          const float u3 = ctk::next_f(rng);
          nd = ctk::metal_dir(d, s, __ldg(m + 1).x, u1, u2, u3);
          if (ctk::dot3(nd, s) > 0.0f) {
            tr *= m0.x, tg *= m0.y, tb *= m0.z;
            pdf = -1.0f;
            cont = true;
          }
        } else if (type == CT_MAT_DIELECTRIC) {
          const float u = ctk::next_f(rng);
          nd = ctk::dielectric_dir(d, s, __ldg(m + 1).x, front, u);
          tr *= m0.x, tg *= m0.y, tb *= m0.z;
          pdf = -1.0f;
          cont = true;
        }
        if (cont && a.rr && bounce >= 3) {  // tracer.ts:305-312
          const float max_b = fmaxf(tr, fmaxf(tg, tb));
          const float ps = max_b > 1.0f ? 1.0f : (max_b < 0.05f ? 0.05f : max_b);
          if (ctk::next_f(rng) > ps) {
            cont = false;
          } else {
            tr /= ps, tg /= ps, tb /= ps;
          }
        }
        if (bounce >= a.max_bounces) cont = false;
        na = make_float4(p.x, p.y, p.z, __uint_as_float(rng));
        nb = make_float4(nd.x, nd.y, nd.z, pdf);
        nc = make_float4(tr, tg, tb, __uint_as_float(pid));
      }
      if (lr != 0.0f || lg != 0.0f || lb != 0.0f) {
        float4* L = a.radiance + pid;
        float4 l = *L;
        l.x += lr;
        l.y += lg;
        l.z += lb;
        *L = l;
      }
    }
    const uint32_t slot = block_append(cont, next_count, s_warp, &s_base);
    const uint32_t sslot = block_append(shadow, shadow_count, s_warp, &s_base);
    if (cont) {
      a.next.a[slot] = na;
      a.next.b[slot] = nb;
      a.next.c[slot] = nc;
    }
    if (shadow) {
      a.shadow.a[sslot] = sa;
      a.shadow.b[sslot] = sb;
      a.shadow.c[sslot] = scol;
    }
  }
}

// Adds the wave's samples to the per-pixel sums in pass order.
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

struct Grids {
  int gen = 0, trace[3] = {0, 0, 0}, shade = 0, acc = 0;
};

const Grids& grids() {
  static Grids g = [] {
    Grids r;
    r.gen = persistent_grid(k_generate);
    r.trace[kWalkThread] = persistent_grid(k_trace<kWalkThread>);
    r.trace[kWalkPersistent] = persistent_grid(k_trace<kWalkPersistent>);
    r.trace[kWalkSkip] = persistent_grid(k_trace<kWalkSkip>);
    r.shade = persistent_grid(k_shade);
    r.acc = persistent_grid(k_accumulate);
    return r;
  }();
  return g;
}

// Walk form of a scene's trace launches: the scene's CT_OPT_WALK when set,
// else by tree size and depth.
int walk_form(const ct_scene* s) {
  if (s->opt_walk >= 0) return s->opt_walk;
  if (s->node_count <= kSkipMaxNodes) return kWalkSkip;
  return s->depth > kPersistentDepth ? kWalkPersistent : kWalkThread;
}

void launch_trace(int form, const WaveArgs& w, int32_t bounce, cudaStream_t stream) {
  const Grids& g = grids();
  switch (form) {
    case kWalkPersistent:
      k_trace<kWalkPersistent><<<g.trace[kWalkPersistent], kBlock, 0, stream>>>(w, bounce);
      break;
    case kWalkSkip:
      k_trace<kWalkSkip><<<g.trace[kWalkSkip], kBlock, 0, stream>>>(w, bounce);
      break;
    default:
      k_trace<kWalkThread><<<g.trace[kWalkThread], kBlock, 0, stream>>>(w, bounce);
      break;
  }
}

ctk::FrameF to_frame(const ct_camera_frame& f) {
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

ct_status check_options(const ct_camera_frame* frame, int32_t width, int32_t height, int32_t max_bounces) {
  CT_CHECK_ARG(frame != nullptr, "frame is NULL");
  CT_CHECK_ARG(width > 0 && height > 0, "image size %dx%d is not positive", width, height);
  CT_CHECK_ARG((uint64_t)width * (uint64_t)height <= (1ull << 30), "image of %dx%d pixels is too large", width, height);
  CT_CHECK_ARG(max_bounces >= 0 && max_bounces <= 1024, "max_bounces %d outside [0, 1024]", max_bounces);
  const double* v = frame->origin;
  for (int k = 0; k < 16; k++)
    CT_CHECK_ARG(std::isfinite(v[k]), "camera frame has a non-finite value");
  return CT_OK;
}

// Runs `passes` passes starting at frame index `first` and adds them to the
// device sums accum (and sumsq when non-NULL).
ct_status run_passes(ct_scene* s, const ct_camera_frame& frame, uint32_t width, uint32_t height, uint32_t first,
                     uint32_t passes, const ct_trace_options& o, float* accum, float* sumsq, cudaStream_t stream) {
  const uint64_t pixels = (uint64_t)width * height;
  const uint64_t wave_paths = s->opt_wave_paths > 0 ? (uint64_t)s->opt_wave_paths : kMaxWavePaths;
  const uint64_t per_wave = std::max<uint64_t>(1, std::min<uint64_t>(passes, wave_paths / pixels));
  const uint64_t cap = per_wave * pixels;
  const int32_t B = o.max_bounces;
  // Layout of the path buffer: 2 queues + shadow queue (3 float4 each per
  // path), radiance (float4), hit prim/t, counters.
  const size_t q_bytes = cap * sizeof(float4);
  // [0, B+2) path queue sizes, [B+2, 2B+4) shadow queue sizes, 2B+6 fp64
  // fallbacks, [2B+8, 3B+10) work counters of the persistent trace launches.
  const size_t counter_words = 3 * (size_t)B + 12;
  const size_t bytes = 10 * q_bytes + cap * 8 + counter_words * 4 + 16 * 256;
  if (s->paths.buf.bytes < bytes) {
    DeviceBuffer cached;
    if (path_cache_take(s->device, bytes, cached)) {
      s->paths.buf.release(&s->device_bytes);
      s->paths.buf = cached;
      s->device_bytes += cached.bytes;
    }
  }
  ct_status st = s->paths.buf.reserve(bytes, &s->device_bytes);
  if (st != CT_OK) return st;
  char* base = s->paths.buf.as<char>();
  auto take = [&](size_t n) {
    char* p = base;
    base += (n + 255) & ~size_t(255);
    return p;
  };
  WaveArgs a{};
  a.scene = s->dev;
  a.frame = to_frame(frame);
  a.cur = Queue{(float4*)take(q_bytes), (float4*)take(q_bytes), (float4*)take(q_bytes)};
  a.next = Queue{(float4*)take(q_bytes), (float4*)take(q_bytes), (float4*)take(q_bytes)};
  a.shadow = ShadowQueue{(float4*)take(q_bytes), (float4*)take(q_bytes), (float4*)take(q_bytes)};
  a.radiance = (float4*)take(q_bytes);
  a.hit_prim = (int32_t*)take(cap * 4);
  a.hit_t = (float*)take(cap * 4);
  a.counts = (uint32_t*)take(counter_words * 4);
  a.width = width;
  a.height = height;
  a.pixels = (uint32_t)pixels;
  a.max_bounces = B;
  a.rr = o.russian_roulette;
  a.nee = o.nee;
  a.sky_kind = s->sky.kind;
  for (int k = 0; k < 3; k++) {
    a.sky_zenith[k] = (float)s->sky.zenith[k];
    a.sky_horizon[k] = (float)s->sky.horizon[k];
  }
  a.sky_strength = (float)s->sky.strength;
  const Grids& g = grids();
  const int form = walk_form(s);
  auto trace = [&](const WaveArgs& w, int32_t b) {
    ProfScope ps("trace", stream);
    launch_trace(form, w, b, stream);
  };
  for (uint64_t done = 0; done < passes; done += per_wave) {
    const uint32_t p = (uint32_t)std::min<uint64_t>(per_wave, passes - done);
    a.paths = (uint32_t)(p * pixels);
    a.first_frame = first + (uint32_t)done;
    CT_CUDA(cudaMemsetAsync(a.counts, 0, counter_words * 4, stream));
    {
      ProfScope ps("generate", stream);
      k_generate<<<g.gen, kBlock, 0, stream>>>(a);
    }
    WaveArgs w = a;
    for (int32_t b = 0; b <= B; b++) {
      trace(w, b);
      {
        ProfScope ps("shade", stream);
        k_shade<<<g.shade, kBlock, 0, stream>>>(w, b);
      }
      std::swap(w.cur, w.next);
    }
    trace(w, B + 1);
    {
      ProfScope ps("accumulate", stream);
      k_accumulate<<<g.acc, kBlock, 0, stream>>>(a.radiance, a.pixels, p, accum, sumsq);
    }
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
}  // namespace ct

extern "C" {

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
  st = scene->io.reserve(n * sizeof(float), &scene->device_bytes);
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
  ct_status st = scene->io.reserve(n * sizeof(float), &scene->device_bytes);
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
// Some callers cannot allocate device memory at the time they render: code
// that is recording a CUDA graph (cudaMalloc is not allowed while a stream is
// being captured), real-time loops that forbid allocation per frame, and
// plugin hosts that hand the library a fixed memory budget at load time and
// own every later allocation. ct_accumulate_pass_noalloc serves them: its
// scratch (path queues, shadow queue, per-path radiance, hit records, queue
// counters) lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits. The scene (created earlier
// with ct_scene_create) and the accumulation buffer are the caller's.
namespace ct {
namespace {

constexpr uint32_t kNoAllocMaxPixels = CT_NOALLOC_MAX_PIXELS;
constexpr size_t kNoAllocPathBytes = 10 * sizeof(float4) + 2 * sizeof(uint32_t);  // per path slot
constexpr size_t kNoAllocCounterWords = 4096;
constexpr size_t kNoAllocScratchBytes =
    (size_t)kNoAllocMaxPixels * kNoAllocPathBytes + kNoAllocCounterWords * 4 + 16 * 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (the host symbol itself is only a stand-in for it).
ct_status noalloc_scratch(int device, void** out) {
  CT_CHECK_ARG(device >= 0 && device < kMaxDevices, "device %d beyond %d", device, kMaxDevices);
  std::lock_guard<std::mutex> guard(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    CT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[device] = p;
  }
  *out = g_noalloc_ptr[device];
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
  const size_t counter_words = 3 * (size_t)B + 12;
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
    base += (n + 255) & ~size_t(255);
    return p;
  };
  const size_t q = pixels * sizeof(float4);
  WaveArgs a{};
  a.scene = scene->dev;
  a.frame = to_frame(*frame);
  a.cur = Queue{(float4*)take(q), (float4*)take(q), (float4*)take(q)};
  a.next = Queue{(float4*)take(q), (float4*)take(q), (float4*)take(q)};
  a.shadow = ShadowQueue{(float4*)take(q), (float4*)take(q), (float4*)take(q)};
  a.radiance = (float4*)take(q);
  a.hit_prim = (int32_t*)take(pixels * 4);
  a.hit_t = (float*)take(pixels * 4);
  a.counts = (uint32_t*)take(counter_words * 4);
  CT_CHECK_ARG((size_t)(base - static_cast<char*>(scratch)) <= kNoAllocScratchBytes, "static scratch layout overflow");
  a.width = (uint32_t)width;
  a.height = (uint32_t)height;
  a.pixels = (uint32_t)pixels;
  a.paths = (uint32_t)pixels;
  a.first_frame = frame_index;
  a.max_bounces = B;
  a.rr = opts->russian_roulette;
  a.nee = opts->nee;
  a.sky_kind = scene->sky.kind;
  for (int k = 0; k < 3; k++) {
    a.sky_zenith[k] = (float)scene->sky.zenith[k];
    a.sky_horizon[k] = (float)scene->sky.horizon[k];
  }
  a.sky_strength = (float)scene->sky.strength;

  // The array keeps the previous call's contents: the counters must start at zero.
  CT_CUDA(cudaMemsetAsync(a.counts, 0, counter_words * 4, s));
  const Grids& g = grids();
  const int form = walk_form(scene);
  k_generate<<<g.gen, kBlock, 0, s>>>(a);
  WaveArgs w = a;
  for (int32_t b = 0; b <= B + 1; b++) {
    launch_trace(form, w, b, s);
    if (b > B) break;
    k_shade<<<g.shade, kBlock, 0, s>>>(w, b);
    std::swap(w.cur, w.next);
  }
  k_accumulate<<<g.acc, kBlock, 0, s>>>(a.radiance, a.pixels, 1, accum, nullptr);
  CT_CUDA(cudaGetLastError());
  return CT_OK;
}

}  // extern "C"
