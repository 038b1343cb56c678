// trace_mixed.cu -- launcher of the mixed-precision tracer.  A scene runs
// the smallest compiled instance whose feature set covers its own
// (rbg_scene::features): the lean instance compiled here for scenes of
// boxes and aspheric disks with mirrors, obscurations and focal surfaces
// only (two-mirror telescopes), an instance per common scene class, and
// the all-features instance (trace_mixed_all.cu) for anything else.
#include "trace_mixed.cuh"

namespace rbg {

#define RBG_MIXED_LAUNCHER(name)                                                                              \
  int name(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o, \
           cudaStream_t st, unsigned* err_flags, unsigned long long* counter);
RBG_MIXED_LAUNCHER(launch_mixed_csg)
RBG_MIXED_LAUNCHER(launch_mixed_facets)
RBG_MIXED_LAUNCHER(launch_mixed_cones)
RBG_MIXED_LAUNCHER(launch_mixed_coated)
RBG_MIXED_LAUNCHER(launch_mixed_all)
#undef RBG_MIXED_LAUNCHER

namespace {
// the lean instance at 256 threads per block unless the options ask for 128
int launch_mixed_lean(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n,
                      const rbg_trace_opts& o, cudaStream_t st, unsigned* err_flags, unsigned long long* counter) {
  if (o.block_size == 128) return launch_mixed_impl<0u, 128>(S, in, out, n, o, st, err_flags, counter);
  return launch_mixed_impl<0u, 256>(S, in, out, n, o, st, err_flags, counter);
}

typedef int (*MixedLauncher)(const DevScene&, const KernelRays&, const KernelOut&, int64_t, const rbg_trace_opts&,
                             cudaStream_t, unsigned*, unsigned long long*);
struct Instance {
  unsigned features;
  MixedLauncher launch;
  int block;  // threads per block (0: 256, or 128 when the options ask for it)
};
// in order of growing feature sets; the last covers every scene
const Instance kInstances[] = {
    {0u, launch_mixed_lean, 0},
    {kFeatCSG, launch_mixed_csg, 128},
    {kFeatCSG | kFeatRough | kFeatBVH, launch_mixed_facets, 256},
    {kFeatWinston | kFeatLens | kFeatBVH, launch_mixed_cones, 128},
    {kFeatCSG | kFeatLens | kFeatMultilayer | kFeatBVH, launch_mixed_coated, 128},
    {kFeatAll, launch_mixed_all, 128},
};
}  // namespace

// the block size the mixed tracer runs a scene of these features with;
// 0 when only the lean instance's two sizes (256, 128) are open to tuning
int mixed_block_size(unsigned features) {
  for (const Instance& inst : kInstances)
    if (!(features & ~inst.features)) return inst.block;
  return 128;
}

int launch_mixed(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o,
                 cudaStream_t st, unsigned* err_flags, unsigned long long* counter, int* launches) {
  for (const Instance& inst : kInstances) {
    if (S.features & ~inst.features) continue;
    const int rc = inst.launch(S, in, out, n, o, st, err_flags, counter);
    if (rc == RBG_OK) *launches += 1;
    return rc;
  }
  return RBG_ERR_UNSUPPORTED;
}

}  // namespace rbg
