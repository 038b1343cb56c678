// trace_mixed_facets.cu -- instance of the mixed-precision tracer for scenes whose
// features are a subset of {kFeatCSG, kFeatRough, kFeatBVH}:
// CSG mirrors with roughness under a BVH (segmented reflectors).  Each instance carries only the code its features need, which
// keeps the kernel's instruction footprint small.
#include "trace_mixed.cuh"

namespace rbg {

int launch_mixed_facets(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n,
                     const rbg_trace_opts& o, cudaStream_t st, unsigned* err_flags, unsigned long long* counter) {
  // 256 threads per block: 4.5 % faster than 128 on the Davies-Cotton dish
  return launch_mixed_impl<kFeatCSG | kFeatRough | kFeatBVH, 256>(S, in, out, n, o, st, err_flags, counter);
}

}  // namespace rbg
