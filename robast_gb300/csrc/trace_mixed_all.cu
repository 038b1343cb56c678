// trace_mixed_all.cu -- the all-features instance of the mixed-precision
// tracer (CSG primitives, Winston cones, lenses, thin films, roughness,
// BVHs), compiled on its own so that the build runs it in parallel.
#include "trace_mixed.cuh"

namespace rbg {

int launch_mixed_all(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n,
                     const rbg_trace_opts& o, cudaStream_t st, unsigned* err_flags, unsigned long long* counter) {
  return launch_mixed_impl<kFeatAll>(S, in, out, n, o, st, err_flags, counter);
}

}  // namespace rbg
