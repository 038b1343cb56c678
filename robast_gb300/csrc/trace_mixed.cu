// trace_mixed.cu -- launcher of the mixed-precision tracer: scenes made of
// boxes and aspheric disks with mirrors, obscurations and focal surfaces
// only (two-mirror telescopes) run the lean instance compiled here; any
// other scene runs the all-features instance (trace_mixed_all.cu).
#include "trace_mixed.cuh"

namespace rbg {

int launch_mixed_all(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n,
                     const rbg_trace_opts& o, cudaStream_t st, unsigned* err_flags, unsigned long long* counter);

int launch_mixed(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o,
                 cudaStream_t st, unsigned* err_flags, unsigned long long* counter, int* launches) {
  const int rc = S.features == 0 ? launch_mixed_impl<0u>(S, in, out, n, o, st, err_flags, counter)
                                 : launch_mixed_all(S, in, out, n, o, st, err_flags, counter);
  if (rc == RBG_OK) *launches = 1;
  return rc;
}

}  // namespace rbg
