// trace_mixed.cuh -- the mixed-precision tracer ("chosen form").
//
// A persistent kernel: one launch fills every SM with resident warps; each
// warp keeps 32 rays in flight and advances them one boundary step at a
// time.  Lanes whose ray has terminated are refilled from a global ray
// counter: one __ballot_sync finds the free lanes, one atomicAdd per warp
// reserves that many consecutive rays and each free lane takes its slot
// (warp-ballot compaction of live rays), so lanes do not idle while the
// warp's longest path finishes.  The per-step arithmetic uses the MIXED
// instantiation of the tracer: FP32 screening and Newton iterations with an
// FP64 polish of each accepted root, FP32 thin-film matrices and Fresnel
// coefficients; ray positions, times and accepted intersection distances
// stay FP64.
#pragma once
#include <cuda_runtime.h>

#include "scene_internal.h"
#include "device_state.cuh"
#include "tracer.cuh"

namespace rbg {

// threads per block, by default; the lean instance comes at 128 and 256
// (rbg_trace_opts.block_size, tuned by rbg_scene_autotune) and the
// segmented-reflector instance at 256: there the compiler's budget of 128
// registers per thread gives 16 resident warps per SM against 12 at 128
// threads and 168 registers
constexpr int kMixedBlock = 128;
// compaction threshold when neither the options nor the scene's tuning
// give one
constexpr int kDefaultCompaction = 32;

// Instances: F = kFeatAll runs any scene; F = 0 (boxes and aspheric disks,
// mirrors, obscurations and focal surfaces only, e.g. two-mirror
// telescopes) compiles every other code path out, which frees registers.
template <unsigned F, int B>
__global__ void __launch_bounds__(B) trace_mixed_kernel(DevScene S, KernelRays in, KernelOut out,
                                                                  int64_t n, int limit, int disable_fresnel,
                                                                  uint64_t seed, uint64_t id_offset,
                                                                  int refill_min, unsigned* err_flags,
                                                                  unsigned long long* next_ray) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lanes_below = (1u << lane) - 1u;
  Ray r;
  Nav nv;
  int64_t idx = -1;
  bool active = false;
  bool drained = false;  // warp-uniform: the global queue is empty
  unsigned err = 0;
  r.status = RBG_STOP;
#ifdef RBG_COUNT_EVENTS
  for (int k = threadIdx.x; k < EV_COUNT; k += blockDim.x) rbg_block_events[k] = 0;
  __syncthreads();
#endif
  for (;;) {
    unsigned need = __ballot_sync(FULL, !active);
    // refill once enough lanes are idle (compaction threshold): fewer,
    // larger refills keep a warp's rays consecutive and their paths alike
    if (need && !drained && (need == FULL || __popc(need) >= refill_min)) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(next_ray, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (base >= (unsigned long long)n) drained = true;
      if (!active) {
        unsigned long long mine = base + __popc(need & lanes_below);
        if (mine < (unsigned long long)n) {
          // queue slot -> ray: the ray keeps its own index (inputs,
          // outputs, random draws) whatever the take-up order
          idx = in.order ? (int64_t)in.order[mine] : (int64_t)mine;
          const int64_t src = in.gathered ? (int64_t)mine : idx;
          if ((uint64_t)idx >= (uint64_t)n) {
            err |= ERR_BIT_CAP;  // not a permutation of the batch: never expected
          } else if (load_ray_f(in, out, src, idx, seed, id_offset, r)) {
            trace_begin<true, F>(S, r, nv);
            active = true;
          } else {
            err |= r.err;
            store_ray(out, idx, r);
          }
        }
      }
    }
    if (!__any_sync(FULL, active)) {
      if (drained) break;
      continue;
    }
    if (active) {
      trace_step<true, F>(S, r, nv, limit, disable_fresnel != 0);
      if (r.status != RBG_RUN) {
        err |= r.err;
        store_ray(out, idx, r);
        active = false;
      }
    }
  }
  if (err) atomicOr(err_flags, err);
#ifdef RBG_COUNT_EVENTS
  __syncthreads();
  for (int k = threadIdx.x; k < EV_COUNT; k += blockDim.x) atomicAdd(&rbg_event_totals[k], rbg_block_events[k]);
#endif
}

// Launch over n rays on stream st: one block per resident slot of every SM
// (occupancy queried once per instantiation), never more blocks than rays
// need; the queue head is reset on the stream first.
template <unsigned F, int B = kMixedBlock>
int launch_mixed_impl(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n,
                      const rbg_trace_opts& o, cudaStream_t st, unsigned* err_flags, unsigned long long* counter) {
  // resident blocks per SM, queried once per instantiation and device
  constexpr int kMaxDev = 64;
  static int bps_of[kMaxDev] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return RBG_ERR_CUDA;
  if (dev >= kMaxDev) return RBG_ERR_UNSUPPORTED;
  if (bps_of[dev] == 0) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, trace_mixed_kernel<F, B>, B, 0) != cudaSuccess)
      return RBG_ERR_CUDA;
    bps_of[dev] = b < 1 ? 1 : b;
  }
  const int bps = bps_of[dev];
  const int sms = sm_count();
  int64_t want = (n + B - 1) / B;
  int64_t grid = (int64_t)sms * bps;
  if (want < grid) grid = want;
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st) != cudaSuccess) return RBG_ERR_CUDA;
  const int refill = o.compaction < 1 ? kDefaultCompaction : (o.compaction > 32 ? 32 : o.compaction);
  trace_mixed_kernel<F, B><<<(int)grid, B, 0, st>>>(S, in, out, n, o.limit, o.disable_fresnel, o.seed,
                                                          o.ray_id_offset, refill, err_flags, counter);
  if (cudaGetLastError() != cudaSuccess) return RBG_ERR_CUDA;
  return RBG_OK;
}

}  // namespace rbg
