// device_state.cuh -- the device mirror a scene owns once uploaded.
#pragma once
#include <vector>

#include "device_scene.cuh"

struct rbg_device_scene {
  rbg::DevScene view;
  std::vector<void*> allocations;
  unsigned* err_flags;          // device word of error bits
  unsigned long long* counter;  // ray queue head of the persistent kernel
  unsigned long long* adj_skip; // rays the adjoint skipped
  cudaStream_t host_streams[2] = {nullptr, nullptr};  // rbg_trace_host pipeline
};

namespace rbg {
int ensure_device(rbg_scene* s);  // upload on first use (capi.cu)
int sm_count();     // SMs of the current device
// precalculated thin-film tables of s into `tables` (device), tmm.cu
int fill_tmm_tables(const rbg_scene* s, const DevScene& S, double* tables, cudaStream_t st);
}  // namespace rbg
