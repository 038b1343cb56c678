// trace_fp64.cu -- the plain FP64 tracer: one thread per ray, the whole
// path in registers, every shape query in FP64.  It is the comparator of the
// mixed-precision tracer and the GPU form closest to the reference's own
// per-ray loop (src/AOpticsManager.cxx:335-520).
#include <cuda_runtime.h>

#include "scene_internal.h"
#include "device_state.cuh"
#include "tracer.cuh"

namespace rbg {

__global__ void __launch_bounds__(128) trace_fp64_kernel(DevScene S, KernelRays in, KernelOut out, int64_t n,
                                                         int limit, int disable_fresnel, uint64_t seed,
                                                         uint64_t id_offset, unsigned* err_flags) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    // slot q -> ray: in a take-up order (ray_order.cu) the ray keeps its
    // own index for its outputs and random draws
    const int64_t i = in.order ? (int64_t)in.order[q] : q;
    const int64_t src = in.gathered ? q : i;
    if ((uint64_t)i >= (uint64_t)n) {
      atomicOr(err_flags, ERR_BIT_CAP);  // not a permutation: never expected
      continue;
    }
    Ray r;
    if (load_ray(in, out, src, i, seed, id_offset, r)) trace_ray<false>(S, r, limit, disable_fresnel != 0);
    if (r.err) atomicOr(err_flags, r.err);
    store_ray(out, i, r);
  }
}

int launch_fp64(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o,
                cudaStream_t st, unsigned* err_flags, int* launches) {
  int block = o.block_size > 0 ? o.block_size : 128;
  if (block > 128) block = 128;
  int64_t blocks64 = (n + block - 1) / block;
  int64_t cap = (int64_t)sm_count() * 64;
  int blocks = (int)(blocks64 < cap ? blocks64 : cap);
  trace_fp64_kernel<<<blocks, block, 0, st>>>(S, in, out, n, o.limit, o.disable_fresnel, o.seed, o.ray_id_offset,
                                              err_flags);
  if (cudaGetLastError() != cudaSuccess) return RBG_ERR_CUDA;
  *launches += 1;
  return RBG_OK;
}

}  // namespace rbg
