// trace_mixed_coated.cu -- instance of the mixed-precision tracer for scenes whose
// features are a subset of {kFeatCSG, kFeatLens, kFeatMultilayer, kFeatBVH}:
// CSG, lenses and thin-film mirrors under a BVH (catadioptric telescopes).  Each instance carries only the code its features need, which
// keeps the kernel's instruction footprint small.
#include "trace_mixed.cuh"

namespace rbg {

int launch_mixed_coated(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n,
                     const rbg_trace_opts& o, cudaStream_t st, unsigned* err_flags, unsigned long long* counter) {
  return launch_mixed_impl<kFeatCSG | kFeatLens | kFeatMultilayer | kFeatBVH>(S, in, out, n, o, st, err_flags, counter);
}

}  // namespace rbg
