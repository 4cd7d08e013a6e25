// Optional per-kernel timing: CUDA events recorded around each launch on its
// stream while profiling is enabled (ct_profile_enable). Used by benchmarks
// to attribute device time to kernels without a profiler attached.
#pragma once

#include <cuda_runtime.h>

namespace ct {

bool profiling();
// Records the start/end event of one launch of kernel `name` on `stream`.
void prof_mark(const char* name, cudaStream_t stream, bool end);

struct ProfScope {
  const char* name;
  cudaStream_t stream;
  bool on;
  ProfScope(const char* n, cudaStream_t s) : name(n), stream(s), on(profiling()) {
    if (on) prof_mark(name, stream, false);
  }
  ~ProfScope() {
    if (on) prof_mark(name, stream, true);
  }
};

}  // namespace ct
