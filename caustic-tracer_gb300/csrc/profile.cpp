// Per-kernel event timing (see profile.hpp) and its C ABI.
#include "profile.hpp"

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.hpp"

namespace ct {

namespace {

struct Rec {
  const char* name;
  cudaEvent_t start, end;
};

std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Rec> g_open, g_done;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

}  // namespace

bool profiling() { return g_on.load(std::memory_order_relaxed); }

void prof_mark(const char* name, cudaStream_t stream, bool end) {
  std::lock_guard<std::mutex> guard(g_mu);
  if (!end) {
    Rec r{name, take_event(), nullptr};
    cudaEventRecord(r.start, stream);
    g_open.push_back(r);
    return;
  }
  for (size_t i = g_open.size(); i-- > 0;) {
    if (g_open[i].name == name) {
      Rec r = g_open[i];
      g_open.erase(g_open.begin() + (long)i);
      r.end = take_event();
      cudaEventRecord(r.end, stream);
      g_done.push_back(r);
      return;
    }
  }
}

}  // namespace ct

extern "C" {

void ct_profile_enable(int32_t on) { ct::g_on.store(on != 0); }

void ct_profile_reset(void) {
  std::lock_guard<std::mutex> guard(ct::g_mu);
  for (auto& r : ct::g_done) {
    cudaEventSynchronize(r.end);
    ct::g_pool.push_back(r.start);
    ct::g_pool.push_back(r.end);
  }
  ct::g_done.clear();
}

int32_t ct_profile_read(const char** names, double* ms, uint64_t* launches, int32_t capacity) {
  std::lock_guard<std::mutex> guard(ct::g_mu);
  int32_t n = 0;
  for (auto& r : ct::g_done) {
    float dt = 0.0f;
    cudaEventSynchronize(r.end);
    cudaEventElapsedTime(&dt, r.start, r.end);
    int32_t k = 0;
    while (k < n && std::strcmp(names[k], r.name) != 0) k++;
    if (k == n) {
      if (n == capacity) continue;
      names[n] = r.name;
      ms[n] = 0;
      launches[n] = 0;
      n++;
    }
    ms[k] += dt;
    launches[k] += 1;
  }
  return n;
}

}  // extern "C"
