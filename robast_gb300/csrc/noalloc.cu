// noalloc.cu -- rbg_trace_noalloc: the mixed-precision trace with every
// piece of library-owned device memory in one fixed, statically allocated
// array instead of cudaMalloc'd buffers.
//
// Who needs it: a caller embedded in a host framework that owns all device
// memory (a telescope camera's real-time trigger or data-acquisition chain
// with a fixed memory budget, a serving process with a preallocated pool)
// and must not let a library allocate or free device memory while it runs:
// cudaMalloc can fail under such a budget, and cudaFree synchronises the
// whole device, stalling the caller's other streams.  rbg_trace allocates
// once per scene and device (the uploaded scene tables, an error word and
// the ray-queue counter); this entry point allocates nothing at all.
//
// The array g_trace_scratch (RBG_NOALLOC_SCRATCH_BYTES = 4 MiB) exists once
// per GPU that loads the library, for the life of the process.  Each call
// copies the scene's flattened tables into it, zeroes the error word and the
// queue counter, and launches the same persistent kernel as rbg_trace with
// RBG_PREC_MIXED.  Consequences for callers:
//   * calls share the array and it keeps the last call's contents, so two
//     calls whose work overlaps on the GPU (different streams, different
//     scenes, or the same scene) race -- serialise them;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first
//     call before any stream capture begins;
//   * scenes whose tables exceed the array are rejected with
//     RBG_ERR_TOO_LARGE before any device work.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "scene_internal.h"
#include "device_state.cuh"
#include "tracer.cuh"

#define RBG_NOALLOC_SCRATCH_BYTES (4u << 20)

static __device__ __align__(256) unsigned char g_trace_scratch[RBG_NOALLOC_SCRATCH_BYTES];

namespace rbg {

int launch_mixed(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o,
                 cudaStream_t st, unsigned* err_flags, unsigned long long* counter, int* launches);

namespace {

constexpr int kMaxDevices = 64;
constexpr size_t kHeader = 256;  // error word at 0, queue counter at 8
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {nullptr};

size_t round_up(size_t v) { return (v + 255) & ~size_t(255); }

// device address of g_trace_scratch on the current device (set up once)
int scratch_address(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return RBG_ERR_NODEVICE;
  if (dev >= kMaxDevices) return RBG_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_trace_scratch) != cudaSuccess || !p) return RBG_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_addr[dev];
  return RBG_OK;
}

template <typename T>
size_t table_bytes(const std::vector<T>& v) {
  return round_up(v.size() * sizeof(T));
}

// copy one table into the array at *offset; returns its device pointer
template <typename T>
int place(const std::vector<T>& v, unsigned char* base, size_t* offset, cudaStream_t st, const T** out) {
  *out = nullptr;
  if (v.empty()) return RBG_OK;
  unsigned char* dst = base + *offset;
  if (cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return RBG_ERR_CUDA;
  *out = reinterpret_cast<const T*>(dst);
  *offset += table_bytes(v);
  return RBG_OK;
}

}  // namespace
}  // namespace rbg

using namespace rbg;

extern "C" int rbg_trace_noalloc(rbg_scene* s, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* opts,
                                 void* stream) {
  if (!s || !in || !out || !opts) return RBG_ERR_ARG;
  if (in->n < 0 || opts->limit <= 0) return RBG_ERR_ARG;
  if (in->n > 0 && (!in->x || !in->y || !in->z || !in->dx || !in->dy || !in->dz || !in->lambda)) return RBG_ERR_ARG;
  if (out->hist_cap < 0 || (out->hist_cap > 0 && (!out->hist_xyzt || !out->hist_node))) return RBG_ERR_ARG;
  if (opts->precision != RBG_PREC_MIXED) return RBG_ERR_UNSUPPORTED;
  const size_t need = kHeader + table_bytes(s->nodes) + table_bytes(s->children) + table_bytes(s->bvh) +
                      table_bytes(s->bvh_items) + table_bytes(s->shapes) + table_bytes(s->volumes) +
                      table_bytes(s->tables) + table_bytes(s->indices) + table_bytes(s->layers) +
                      table_bytes(s->multilayers) + table_bytes(s->borders) + table_bytes(s->params) +
                      table_bytes(s->node_aux) + table_bytes(s->fparams) + table_bytes(s->trig) +
                      table_bytes(s->trig_off) + table_bytes(s->tmm_tables) + table_bytes(s->tmm_off);
  if (need > RBG_NOALLOC_SCRATCH_BYTES) return RBG_ERR_TOO_LARGE;
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  if (in->n == 0) return RBG_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  DevScene v;
  std::memset(&v, 0, sizeof(v));
  size_t off = kHeader;
  if ((rc = place(s->nodes, base, &off, st, &v.nodes)) || (rc = place(s->children, base, &off, st, &v.children)) ||
      (rc = place(s->bvh, base, &off, st, &v.bvh)) || (rc = place(s->bvh_items, base, &off, st, &v.bvh_items)) ||
      (rc = place(s->shapes, base, &off, st, &v.shapes)) || (rc = place(s->volumes, base, &off, st, &v.volumes)) ||
      (rc = place(s->tables, base, &off, st, &v.tables)) || (rc = place(s->indices, base, &off, st, &v.indices)) ||
      (rc = place(s->layers, base, &off, st, &v.layers)) ||
      (rc = place(s->multilayers, base, &off, st, &v.multilayers)) ||
      (rc = place(s->borders, base, &off, st, &v.borders)) || (rc = place(s->params, base, &off, st, &v.params)) ||
      (rc = place(s->node_aux, base, &off, st, &v.aux)) || (rc = place(s->fparams, base, &off, st, &v.fparams)) ||
      (rc = place(s->trig, base, &off, st, &v.trig)) || (rc = place(s->trig_off, base, &off, st, &v.trig_off)) ||
      (rc = place(s->tmm_tables, base, &off, st, &v.tmm_tables)) ||
      (rc = place(s->tmm_off, base, &off, st, &v.tmm_off)))
    return rc;
  v.n_nodes = (int32_t)s->nodes.size();
  v.n_borders = (int32_t)s->borders.size();
  v.n_multilayers = (int32_t)s->multilayers.size();
  v.n_tables = (int32_t)s->tables.size();
  v.features = s->features;
  if (!s->tmm_ready) {
    // precalculated thin-film tables not computed yet (no rbg_trace on this
    // scene so far): fill them in place in the array, keep a host copy
    double* tab = const_cast<double*>(v.tmm_tables);
    if ((rc = fill_tmm_tables(s, v, tab, st))) return rc;
    if (cudaMemcpyAsync(s->tmm_tables.data(), tab, s->tmm_tables.size() * sizeof(double), cudaMemcpyDeviceToHost,
                        st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return RBG_ERR_CUDA;
    s->tmm_ready = true;
  }
  unsigned* err_flags = reinterpret_cast<unsigned*>(base);
  unsigned long long* counter = reinterpret_cast<unsigned long long*>(base + 8);
  // the error word and the queue head must start at zero on every call
  if (cudaMemsetAsync(base, 0, 16, st) != cudaSuccess) return RBG_ERR_CUDA;
  KernelRays kr{in->x, in->y, in->z, in->t, in->dx, in->dy, in->dz, in->lambda};
  KernelOut ko{out->status, out->npoints, out->last_node, out->x, out->y, out->z, out->t,
               out->dx, out->dy, out->dz, out->hist_cap, out->hist_xyzt, out->hist_node};
  int launches = 0;
  if ((rc = launch_mixed(v, kr, ko, in->n, *opts, st, err_flags, counter, &launches))) return rc;
  unsigned bits = 0;
  if (cudaMemcpyAsync(&bits, err_flags, sizeof(bits), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return RBG_ERR_CUDA;
  if (bits & ERR_BIT_NAN) return RBG_ERR_NAN;
  if (bits & ERR_BIT_CAP) return RBG_ERR_CAP;
  return RBG_OK;
}
