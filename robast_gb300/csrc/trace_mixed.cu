// trace_mixed.cu -- mixed-precision tracer (placeholder until implemented).
#include <cuda_runtime.h>

#include "scene_internal.h"
#include "tracer.cuh"

namespace rbg {
struct KernelRays;
struct KernelOut;
int launch_mixed(rbg_scene*, const KernelRays&, const KernelOut&, int64_t, const rbg_trace_opts&, cudaStream_t,
                 int*) {
  return RBG_ERR_UNSUPPORTED;
}
}  // namespace rbg
