// Display transforms on the device: tonemapBuffer (tonemap.ts:41-62) into
// RGBA8 and a binary PPM (ppm.ts:4-16) straight from the sum buffer.
//
// Each channel is computed in float32 (ACES fit or Reinhard, then the sRGB
// curve, whose power x^(1/2.4) is taken as exp2f(log2f(x) / 2.4)); its scaled
// value y = 255 * srgb carries an error below 4e-4 (for x in [0.0031308, 1],
// |log2 x| <= 8.33: log2f's 1 ulp is at most 9.6e-7, the division by 2.4 adds
// 1 ulp of a value below 3.5, exp2f's 2 ulp add 2.4e-7 relative, so the power
// is within 9e-7 relative and y within 255 * 1.055 * 9e-7 = 2.4e-4, plus the
// roundings of the curve and of the scaling). Only a channel whose y lies
// within 1e-3 of a rounding boundary (k + 0.5), or is not a number, is
// recomputed in float64 in the reference's operation order (its power as
// exp(log(x) / 2.4), within about 1e-15 relative of the exact power), so
// every byte is the one the reference's float64 code stores unless y lies
// within about 1e-12 of a boundary. One thread per pixel: 12 bytes read, 4
// (or 3) written. The float64 recomputations (about 0.2 % of channels) do not
// run where they arise: a thread queues the channel in its block's shared
// memory and stores a provisional byte, and the block later recomputes its
// queue with every lane busy, so the slow float64 unit never runs with one
// lane of a warp active while the other 31 wait.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "profile.hpp"
#include "scene.hpp"

namespace ct {
namespace {

constexpr float kRoundMargin = 1e-3f;
constexpr int kBlock = 256;

// tonemap.ts:7-15 and 18-20, float64
__device__ double aces64(double x) {
  const double v = (x * (2.51 * x + 0.03)) / (x * (2.43 * x + 0.59) + 0.14);
  return v < 0 ? 0 : v > 1 ? 1 : v;
}
__device__ double reinhard64(double x) { return x <= 0 ? 0 : x / (1 + x); }
// tonemap.ts:27-31
__device__ double srgb64(double x) {
  if (x <= 0) return 0;
  if (x >= 1) return 1;
  return x <= 0.0031308 ? 12.92 * x : 1.055 * exp(log(x) / 2.4) - 0.055;
}
// Math.round (halves toward +infinity), then the Uint8ClampedArray store
// (clamp to [0, 255], NaN -> 0).
__device__ uint8_t store_byte(double y) {
  const double f = floor(y);
  const double v = y - f >= 0.5 ? f + 1 : f;
  return (uint8_t)(v >= 0 && v <= 255 ? v : v > 255 ? 255 : 0);
}

// The same curves in float32.
__device__ float aces32(float x) {
  const float v = (x * __fmaf_rn(2.51f, x, 0.03f)) / __fmaf_rn(x, __fmaf_rn(2.43f, x, 0.59f), 0.14f);
  return v < 0.0f ? 0.0f : v > 1.0f ? 1.0f : v;
}
__device__ float reinhard32(float x) { return x <= 0.0f ? 0.0f : x / (1.0f + x); }
__device__ float srgb32(float x) {
  if (x <= 0.0f) return 0.0f;
  if (x >= 1.0f) return 1.0f;
  return x <= 0.0031308f ? 12.92f * x : __fmaf_rn(1.055f, exp2f(log2f(x) * (1.0f / 2.4f)), -0.055f);
}

// The float32 byte of a channel; false when y is within kRoundMargin of a
// rounding boundary or not a number, where only the float64 path decides.
__device__ __forceinline__ bool channel32(float a, float inv32, int aces, uint8_t& byte) {
  const float x = a * inv32;
  const float y = srgb32(aces ? aces32(x) : reinhard32(x)) * 255.0f;
  const float frac = y - floorf(y);
  byte = (uint8_t)(frac > 0.5f ? floorf(y) + 1.0f : floorf(y));
  return fabsf(frac - 0.5f) > kRoundMargin;
}

// The reference's float64 path (tonemap.ts:41-62) for one channel.
__device__ __noinline__ uint8_t channel64(float a, double inv, int aces) {
  const double xd = (double)a * inv;
  return store_byte(srgb64(aces ? aces64(xd) : reinhard64(xd)) * 255.0);
}

// RGBA (stride 4, alpha 255) or the PPM payload (stride 3) after `offset`
// header bytes, which block 0 writes from `header`.
struct Header {
  char bytes[32];
  uint32_t len;
};

constexpr uint32_t kQueue = 2048;  // float64 recomputations a block queues before it drains them

// Recomputes the block's queued channels (indices into accum) in float64 and
// stores their bytes over the provisional ones; every thread of the block calls it.
__device__ __forceinline__ void drain(const float* __restrict__ accum, double inv, int aces, uint8_t* px_out,
                                      uint32_t stride, const uint32_t* queue, uint32_t* count) {
  __syncthreads();  // the provisional stores and the queue entries are visible to the block
  const uint32_t n = *count;
  for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
    const uint32_t ch = queue[k];
    px_out[(size_t)(ch / 3) * stride + ch % 3] = channel64(accum[ch], inv, aces);
  }
  __syncthreads();
  if (threadIdx.x == 0) *count = 0;
  __syncthreads();
}

__global__ void __launch_bounds__(kBlock) k_tonemap(const float* __restrict__ accum, uint32_t pixels, double inv,
                                                    float inv32, int aces, uint8_t* __restrict__ out,
                                                    uint32_t stride, Header header) {
  __shared__ uint32_t queue[kQueue];
  __shared__ uint32_t count;
  if (threadIdx.x == 0) count = 0;
  if (blockIdx.x == 0 && threadIdx.x < header.len) out[threadIdx.x] = (uint8_t)header.bytes[threadIdx.x];
  uint8_t* px_out = out + header.len;
  const uint32_t grid = gridDim.x * blockDim.x;
  __syncthreads();
  // Block-uniform trip count (the drains synchronise the block).
  for (uint32_t base = blockIdx.x * blockDim.x; base < pixels; base += grid) {
    const uint32_t i = base + threadIdx.x;
    if (i < pixels) {
      const float r = accum[3 * (size_t)i], g = accum[3 * (size_t)i + 1], b = accum[3 * (size_t)i + 2];
      uint8_t br, bg, bb;
      const bool okr = channel32(r, inv32, aces, br), okg = channel32(g, inv32, aces, bg),
                 okb = channel32(b, inv32, aces, bb);
      if (!(okr && okg && okb)) {
        const uint32_t n = (uint32_t)!okr + (uint32_t)!okg + (uint32_t)!okb;
        uint32_t k = atomicAdd(&count, n);
        if (!okr) queue[k++] = 3 * i;
        if (!okg) queue[k++] = 3 * i + 1;
        if (!okb) queue[k] = 3 * i + 2;
      }
      if (stride == 4) {
        reinterpret_cast<uchar4*>(px_out)[i] = make_uchar4(br, bg, bb, 255);
      } else {
        uint8_t* o = px_out + 3 * (size_t)i;
        o[0] = br, o[1] = bg, o[2] = bb;
      }
    }
    __syncthreads();
    if (count > kQueue - 3 * kBlock) drain(accum, inv, aces, px_out, stride, queue, &count);
  }
  drain(accum, inv, aces, px_out, stride, queue, &count);
}

ct_status launch_tonemap(const float* accum, int32_t width, int32_t height, double samples, double exposure_ev,
                         int32_t mode, uint8_t* out, uint32_t stride, const Header& header, void* stream) {
  const uint64_t pixels = (uint64_t)width * (uint64_t)height;
  // tonemap.ts:49: inv = 2^ev / samples, 0 without samples
  const double inv = samples > 0 ? std::pow(2.0, exposure_ev) / samples : 0.0;
  int dev = 0, sms = 0;
  CT_CUDA(cudaGetDevice(&dev));
  CT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint64_t need = (pixels + kBlock - 1) / kBlock;
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sms * 8));
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  ProfScope ps("tonemap", s);
  k_tonemap<<<grid, kBlock, 0, s>>>(accum, (uint32_t)pixels, inv, (float)inv, mode == 0, out, stride, header);
  CT_CUDA(cudaGetLastError());
  return CT_OK;
}

ct_status check_image(const float* accum, int32_t width, int32_t height, int32_t mode, const void* out) {
  CT_CHECK_ARG(accum != nullptr && out != nullptr, "NULL device pointer");
  CT_CHECK_ARG(width > 0 && height > 0, "image size %dx%d is not positive", width, height);
  CT_CHECK_ARG((uint64_t)width * (uint64_t)height <= (1ull << 30), "image of %dx%d pixels is too large", width, height);
  CT_CHECK_ARG(mode == 0 || mode == 1, "tone map mode %d is not 0 (ACES) or 1 (Reinhard)", mode);
  return CT_OK;
}

}  // namespace
}  // namespace ct

extern "C" {

ct_status ct_tonemap_device(const float* accum, int32_t width, int32_t height, double samples, double exposure_ev,
                            int32_t mode, uint8_t* rgba, void* stream) {
  ct::clear_error();
  ct_status st = ct::check_image(accum, width, height, mode, rgba);
  if (st != CT_OK) return st;
  CT_CHECK_ARG(((uintptr_t)rgba & 3u) == 0, "rgba must be 4-byte aligned");
  return ct::launch_tonemap(accum, width, height, samples, exposure_ev, mode, rgba, 4, ct::Header{{0}, 0}, stream);
}

ct_status ct_ppm_device(const float* accum, int32_t width, int32_t height, double samples, double exposure_ev,
                        int32_t mode, uint8_t* ppm, uint64_t capacity, uint64_t* size, void* stream) {
  ct::clear_error();
  ct_status st = ct::check_image(accum, width, height, mode, ppm);
  if (st != CT_OK) return st;
  ct::Header h{};
  const int n = std::snprintf(h.bytes, sizeof h.bytes, "P6\n%d %d\n255\n", width, height);
  CT_CHECK_ARG(n > 0 && n < (int)sizeof h.bytes, "PPM header does not fit");
  h.len = (uint32_t)n;
  const uint64_t total = h.len + (uint64_t)width * (uint64_t)height * 3;
  if (size) *size = total;
  CT_CHECK_ARG(capacity >= total, "PPM needs %llu bytes, buffer holds %llu", (unsigned long long)total,
               (unsigned long long)capacity);
  return ct::launch_tonemap(accum, width, height, samples, exposure_ev, mode, ppm, 3, h, stream);
}

}  // extern "C"
