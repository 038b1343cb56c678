// capi.cu -- C ABI of the tracer: device upload of a flattened scene,
// device- and host-buffer tracing and focal-plane reductions.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "scene_internal.h"
#include "device_state.cuh"
#include "tracer.cuh"

namespace rbg {

namespace {

template <typename T>
int upload(std::vector<void*>& allocs, const std::vector<T>& v, const T** out) {
  *out = nullptr;
  if (v.empty()) return RBG_OK;
  void* p = nullptr;
  if (cudaMalloc(&p, v.size() * sizeof(T)) != cudaSuccess) return RBG_ERR_NOMEM;
  allocs.push_back(p);
  if (cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return RBG_ERR_CUDA;
  *out = static_cast<const T*>(p);
  return RBG_OK;
}

int current_device(int* dev) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return RBG_ERR_NODEVICE;
  if (cudaGetDevice(dev) != cudaSuccess) return RBG_ERR_CUDA;
  return RBG_OK;
}

}  // namespace

void release_device(rbg_scene* s) {
  if (!s || !s->dev) return;
  int prev = -1;
  cudaGetDevice(&prev);
  if (s->dev_id >= 0) cudaSetDevice(s->dev_id);
  for (cudaStream_t& st : s->dev->host_streams)
    if (st) cudaStreamDestroy(st);
  for (void* p : s->dev->allocations) cudaFree(p);
  if (s->workspace) cudaFree(s->workspace);
  if (s->order_ws) cudaFree(s->order_ws);
  if (prev >= 0) cudaSetDevice(prev);
  delete s->dev;
  s->dev = nullptr;
  s->workspace = nullptr;
  s->workspace_bytes = 0;
  s->order_ws = nullptr;
  s->order_ws_bytes = 0;
  s->dev_id = -1;
}

int ensure_device(rbg_scene* s) {
  int dev;
  int rc = current_device(&dev);
  if (rc != RBG_OK) return rc;
  if (s->dev && s->dev_id == dev) return RBG_OK;
  release_device(s);
  auto* d = new rbg_device_scene();
  d->err_flags = nullptr;
  DevScene& v = d->view;
  std::memset(&v, 0, sizeof(v));
  if ((rc = upload(d->allocations, s->nodes, &v.nodes)) ||
      (rc = upload(d->allocations, s->children, &v.children)) ||
      (rc = upload(d->allocations, s->bvh, &v.bvh)) ||
      (rc = upload(d->allocations, s->bvh_items, &v.bvh_items)) ||
      (rc = upload(d->allocations, s->shapes, &v.shapes)) ||
      (rc = upload(d->allocations, s->volumes, &v.volumes)) ||
      (rc = upload(d->allocations, s->tables, &v.tables)) ||
      (rc = upload(d->allocations, s->indices, &v.indices)) ||
      (rc = upload(d->allocations, s->layers, &v.layers)) ||
      (rc = upload(d->allocations, s->multilayers, &v.multilayers)) ||
      (rc = upload(d->allocations, s->borders, &v.borders)) ||
      (rc = upload(d->allocations, s->params, &v.params)) ||
      (rc = upload(d->allocations, s->node_aux, &v.aux)) ||
      (rc = upload(d->allocations, s->fparams, &v.fparams)) ||
      (rc = upload(d->allocations, s->trig, &v.trig)) ||
      (rc = upload(d->allocations, s->trig_off, &v.trig_off)) ||
      (rc = upload(d->allocations, s->tmm_tables, &v.tmm_tables)) ||
      (rc = upload(d->allocations, s->tmm_off, &v.tmm_off))) {
    for (void* p : d->allocations) cudaFree(p);
    delete d;
    return rc;
  }
  void* ef = nullptr;
  if (cudaMalloc(&ef, 16) != cudaSuccess) {
    for (void* p : d->allocations) cudaFree(p);
    delete d;
    return RBG_ERR_NOMEM;
  }
  d->allocations.push_back(ef);
  d->err_flags = static_cast<unsigned*>(ef);
  d->counter = reinterpret_cast<unsigned long long*>(static_cast<char*>(ef) + 8);
  v.n_nodes = (int32_t)s->nodes.size();
  v.n_borders = (int32_t)s->borders.size();
  v.n_multilayers = (int32_t)s->multilayers.size();
  v.n_tables = (int32_t)s->tables.size();
  v.features = s->features;
  if (!s->tmm_ready) {
    // precalculated thin-film tables: fill on the device, keep a host copy
    double* tab = const_cast<double*>(v.tmm_tables);
    if ((rc = fill_tmm_tables(s, v, tab, 0)) ||
        cudaMemcpy(s->tmm_tables.data(), tab, s->tmm_tables.size() * sizeof(double), cudaMemcpyDeviceToHost) !=
            cudaSuccess) {
      for (void* p : d->allocations) cudaFree(p);
      delete d;
      return rc ? rc : RBG_ERR_CUDA;
    }
    s->tmm_ready = true;
  }
  s->dev = d;
  s->dev_id = dev;
  return RBG_OK;
}

int sm_count() {
  static int cached = 0;
  if (cached == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 1;
  }
  return cached;
}

int stack_ready() {
  static int done = 0;
  if (!done) {
    // the CSG walk and the rejection loops recurse/branch deeply: give each
    // thread enough local stack for composite trees of depth <= 6
    if (cudaDeviceSetLimit(cudaLimitStackSize, 8192) != cudaSuccess) return RBG_ERR_CUDA;
    done = 1;
  }
  return RBG_OK;
}

int read_errors(rbg_scene* s, cudaStream_t st, unsigned* bits) {
  if (cudaMemcpyAsync(bits, s->dev->err_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return RBG_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return RBG_ERR_CUDA;
  return RBG_OK;
}

}  // namespace rbg

using namespace rbg;

extern "C" int rbg_scene_upload(rbg_scene* s) {
  if (!s) return RBG_ERR_ARG;
  return ensure_device(s);
}

extern "C" int rbg_last_launch_count(const rbg_scene* s) { return s ? s->last_launches : -1; }

// the two tracer launchers (trace_mixed.cu, trace_fp64.cu)
namespace rbg {
int launch_mixed(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o,
                 cudaStream_t st, unsigned* err_flags, unsigned long long* counter, int* launches);
size_t ray_order_bytes(int64_t n);
int build_ray_order(const KernelRays& in, int64_t n, void* ws, KernelRays* sorted, cudaStream_t st);
// below this many rays the mixed tracer takes rays up in input order
constexpr int64_t kOrderMinRays = 1 << 14;
bool want_ray_order(const rbg_trace_opts& o, int64_t n) {
  return o.precision == RBG_PREC_MIXED && o.ray_order == RBG_ORDER_SPATIAL && n >= kOrderMinRays &&
         ray_order_bytes(n) > 0;
}
int launch_fp64(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o,
                cudaStream_t st, unsigned* err_flags, int* launches);
}

extern "C" int rbg_trace(rbg_scene* s, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* opts,
                         void* stream) {
  if (!s || !in || !out || !opts) return RBG_ERR_ARG;
  if (in->n < 0 || opts->limit <= 0) return RBG_ERR_ARG;
  if (in->n > 0 && (!in->x || !in->y || !in->z || !in->dx || !in->dy || !in->dz || !in->lambda)) return RBG_ERR_ARG;
  if (out->hist_cap < 0 || (out->hist_cap > 0 && (!out->hist_xyzt || !out->hist_node))) return RBG_ERR_ARG;
  int rc = ensure_device(s);
  if (rc) return rc;
  if ((rc = stack_ready())) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  s->last_launches = 0;
  if (in->n == 0) return RBG_OK;
  if (cudaMemsetAsync(s->dev->err_flags, 0, sizeof(unsigned), st) != cudaSuccess) return RBG_ERR_CUDA;
  KernelRays kr{in->x, in->y, in->z, in->t, in->dx, in->dy, in->dz, in->lambda};
  KernelOut ko{out->status, out->npoints, out->last_node, out->x, out->y, out->z, out->t,
               out->dx, out->dy, out->dz, out->hist_cap, out->hist_xyzt, out->hist_node};
  if (opts->precision == RBG_PREC_MIXED) {
    int launches = 0;
    rbg_trace_opts o = *opts;
    if (o.compaction == 0) o.compaction = s->tuned_compaction;
    if (want_ray_order(o, in->n)) {
      const size_t need = ray_order_bytes(in->n);
      if (s->order_ws_bytes < need) {
        // the previous workspace may still be read by work queued earlier
        // on another stream: wait for the device before freeing it
        if (s->order_ws && (cudaDeviceSynchronize() != cudaSuccess || cudaFree(s->order_ws) != cudaSuccess))
          return RBG_ERR_CUDA;
        s->order_ws = nullptr;
        s->order_ws_bytes = 0;
        if (cudaMalloc(&s->order_ws, need) != cudaSuccess) {
          s->order_ws = nullptr;
          return RBG_ERR_NOMEM;
        }
        s->order_ws_bytes = need;
      }
      if ((rc = build_ray_order(kr, in->n, s->order_ws, &kr, st))) return rc;
      launches += 7;
    }
    rc = launch_mixed(s->dev->view, kr, ko, in->n, o, st, s->dev->err_flags, s->dev->counter, &launches);
    if (rc) return rc;
    s->last_launches = launches;
  } else {
    int launches = 0;
    rc = launch_fp64(s->dev->view, kr, ko, in->n, *opts, st, s->dev->err_flags, &launches);
    if (rc) return rc;
    s->last_launches = launches;
  }
  unsigned bits = 0;
  if ((rc = read_errors(s, st, &bits))) return rc;
  if (bits & ERR_BIT_NAN) return RBG_ERR_NAN;
  if (bits & ERR_BIT_CAP) return RBG_ERR_CAP;
  return RBG_OK;
}

// The autotuner of the mixed tracer's compaction threshold: trace the
// caller's rays once to warm up, then once per candidate threshold, timed
// with events on the stream, and keep the fastest in the scene (used by
// every later call whose options leave the threshold at 0).  The results
// in `out` are those of any single trace: they do not depend on the
// threshold.
extern "C" int rbg_scene_autotune(rbg_scene* s, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* opts,
                                  void* stream, int32_t* chosen) {
  if (!s || !in || !out || !opts) return RBG_ERR_ARG;
  static const int32_t kCandidates[] = {1, 8, 16, 32};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rbg_trace_opts o = *opts;
  o.precision = RBG_PREC_MIXED;
  o.compaction = 32;
  int rc = rbg_trace(s, in, out, &o, stream);
  if (rc != RBG_OK && rc != RBG_ERR_NAN && rc != RBG_ERR_CAP) return rc;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return RBG_ERR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return RBG_ERR_CUDA;
  }
  float best_ms = 0.f;
  int32_t best = 32;
  for (int32_t c : kCandidates) {
    o.compaction = c;
    float ms = 0.f;
    if (cudaEventRecord(e0, st) != cudaSuccess) {
      rc = RBG_ERR_CUDA;
      break;
    }
    rc = rbg_trace(s, in, out, &o, stream);
    if (rc != RBG_OK && rc != RBG_ERR_NAN && rc != RBG_ERR_CAP) break;
    if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      rc = RBG_ERR_CUDA;
      break;
    }
    if (c == kCandidates[0] || ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != RBG_OK && rc != RBG_ERR_NAN && rc != RBG_ERR_CAP) return rc;
  s->tuned_compaction = best;
  if (chosen) *chosen = best;
  return rc;
}

namespace rbg {
namespace {

constexpr int kHostStreams = 2;
constexpr int64_t kHostChunk = int64_t(1) << 21;  // rays per pipeline stage

int launch_trace(rbg_scene* s, const KernelRays& kr, const KernelOut& ko, int64_t n, const rbg_trace_opts& o,
                 cudaStream_t st, unsigned* err, unsigned long long* counter, int* launches) {
  if (o.precision == RBG_PREC_MIXED) return launch_mixed(s->dev->view, kr, ko, n, o, st, err, counter, launches);
  return launch_fp64(s->dev->view, kr, ko, n, o, st, err, launches);
}

// the scene's device workspace, grown to at least `bytes`; it is kept
// between calls (freed with the scene), so repeated calls allocate nothing
int grow_workspace(rbg_scene* s, size_t bytes, char** out) {
  if (s->workspace_bytes < bytes) {
    if (s->workspace) cudaFree(s->workspace);
    s->workspace = nullptr;
    s->workspace_bytes = 0;
    if (cudaMalloc(&s->workspace, bytes) != cudaSuccess) {
      s->workspace = nullptr;
      return RBG_ERR_NOMEM;
    }
    s->workspace_bytes = bytes;
  }
  *out = static_cast<char*>(s->workspace);
  return RBG_OK;
}

// One pipeline slot: its own queue head and error word (a 256-byte
// header), the chunk's 8 input and 7 output arrays, fates, point counts,
// last nodes, optional histories and the ray-order workspace, for up to
// `cap` rays.
struct Slot {
  unsigned* err;
  unsigned long long* counter;
  double* in[8];
  double* out[7];
  int32_t* npoints;
  int32_t* last_node;
  uint8_t* status;
  double* hist;
  int32_t* hist_node;
  void* order_ws;
};

size_t slot_bytes(int64_t cap, int hist_cap) {
  return 256 + (size_t)cap * (15 * 8 + 2 * 4 + 8) + (size_t)cap * hist_cap * (4 * 8 + 4) + ray_order_bytes(cap);
}

Slot slot_at(char* base, int64_t cap, int hist_cap) {
  Slot sl;
  sl.err = reinterpret_cast<unsigned*>(base);
  sl.counter = reinterpret_cast<unsigned long long*>(base + 8);
  char* p = base + 256;
  for (int k = 0; k < 8; ++k, p += cap * 8) sl.in[k] = reinterpret_cast<double*>(p);
  for (int k = 0; k < 7; ++k, p += cap * 8) sl.out[k] = reinterpret_cast<double*>(p);
  sl.npoints = reinterpret_cast<int32_t*>(p);
  p += cap * 4;
  sl.last_node = reinterpret_cast<int32_t*>(p);
  p += cap * 4;
  sl.status = reinterpret_cast<uint8_t*>(p);
  p += cap * 8;
  sl.hist = hist_cap ? reinterpret_cast<double*>(p) : nullptr;
  p += (size_t)cap * hist_cap * 32;
  sl.hist_node = hist_cap ? reinterpret_cast<int32_t*>(p) : nullptr;
  p += (size_t)cap * hist_cap * 4;
  sl.order_ws = p;
  return sl;
}

}  // namespace
}  // namespace rbg

// The call a host-side AOpticsManager::TraceNonSequential makes: host
// arrays in and out.  The batch runs as a pipeline of chunks of 2^21 rays
// over two streams, so that the copies of one chunk overlap the tracing of
// the other; each chunk has its own queue head and error word, and its ray
// ids continue the batch's (opts->ray_id_offset + index), so the Philox
// draws -- and the results -- are those of one rbg_trace over the batch.
// Device memory is the scene's workspace, reused across calls.  Host arrays
// in page-locked memory overlap best; pageable ones work, staged by CUDA.
extern "C" int rbg_trace_host(rbg_scene* s, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* opts) {
  if (!s || !in || !out || !opts || in->n < 0 || opts->limit <= 0) return RBG_ERR_ARG;
  if (in->n > 0 && (!in->x || !in->y || !in->z || !in->dx || !in->dy || !in->dz || !in->lambda)) return RBG_ERR_ARG;
  if (out->hist_cap < 0 || (out->hist_cap > 0 && (!out->hist_xyzt || !out->hist_node))) return RBG_ERR_ARG;
  int rc = ensure_device(s);
  if (rc) return rc;
  if ((rc = stack_ready())) return rc;
  const int64_t n = in->n;
  s->last_launches = 0;
  if (n == 0) return RBG_OK;
  const int hcap = out->hist_cap;
  const int64_t cap = ((n < kHostChunk ? n : kHostChunk) + 255) / 256 * 256;
  const int64_t chunks = (n + cap - 1) / cap;
  const int nslots = chunks < kHostStreams ? (int)chunks : kHostStreams;
  const size_t sb = slot_bytes(cap, hcap);
  char* ws = nullptr;
  if ((rc = grow_workspace(s, sb * nslots, &ws))) return rc;
  Slot slots[kHostStreams];
  for (int k = 0; k < nslots; ++k) {
    cudaStream_t& st = s->dev->host_streams[k];
    if (!st && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return RBG_ERR_CUDA;
    slots[k] = slot_at(ws + sb * k, cap, hcap);
    if (cudaMemsetAsync(slots[k].err, 0, 16, st) != cudaSuccess) return RBG_ERR_CUDA;
  }
  const double* src[8] = {in->x, in->y, in->z, in->t, in->dx, in->dy, in->dz, in->lambda};
  double* dst[7] = {out->x, out->y, out->z, out->t, out->dx, out->dy, out->dz};
  int launches = 0;
  for (int64_t c = 0; c < chunks; ++c) {
    const int k = (int)(c % nslots);
    cudaStream_t st = s->dev->host_streams[k];
    const Slot& sl = slots[k];
    const int64_t off = c * cap, m = n - off < cap ? n - off : cap;
    for (int a = 0; a < 8; ++a)
      if (src[a] && cudaMemcpyAsync(sl.in[a], src[a] + off, m * 8, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return RBG_ERR_CUDA;
    KernelRays kr{sl.in[0], sl.in[1], sl.in[2], in->t ? sl.in[3] : nullptr, sl.in[4], sl.in[5], sl.in[6], sl.in[7]};
    KernelOut ko{out->status ? sl.status : nullptr, out->npoints ? sl.npoints : nullptr,
                 out->last_node ? sl.last_node : nullptr, dst[0] ? sl.out[0] : nullptr, dst[1] ? sl.out[1] : nullptr,
                 dst[2] ? sl.out[2] : nullptr, dst[3] ? sl.out[3] : nullptr, dst[4] ? sl.out[4] : nullptr,
                 dst[5] ? sl.out[5] : nullptr, dst[6] ? sl.out[6] : nullptr, hcap, sl.hist, sl.hist_node};
    rbg_trace_opts o = *opts;
    o.ray_id_offset = opts->ray_id_offset + (uint64_t)off;
    if (o.compaction == 0) o.compaction = s->tuned_compaction;
    int nl = 0;
    if (want_ray_order(o, m)) {
      if ((rc = build_ray_order(kr, m, sl.order_ws, &kr, st))) return rc;
      nl += 7;
    }
    if ((rc = launch_trace(s, kr, ko, m, o, st, sl.err, sl.counter, &nl))) return rc;
    launches += nl;
    if (out->status && cudaMemcpyAsync(out->status + off, sl.status, m, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return RBG_ERR_CUDA;
    if (out->npoints &&
        cudaMemcpyAsync(out->npoints + off, sl.npoints, m * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return RBG_ERR_CUDA;
    if (out->last_node &&
        cudaMemcpyAsync(out->last_node + off, sl.last_node, m * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return RBG_ERR_CUDA;
    for (int a = 0; a < 7; ++a)
      if (dst[a] && cudaMemcpyAsync(dst[a] + off, sl.out[a], m * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return RBG_ERR_CUDA;
    if (hcap) {
      if (cudaMemcpyAsync(out->hist_xyzt + off * hcap * 4, sl.hist, (size_t)m * hcap * 32, cudaMemcpyDeviceToHost,
                          st) != cudaSuccess ||
          cudaMemcpyAsync(out->hist_node + off * hcap, sl.hist_node, (size_t)m * hcap * 4, cudaMemcpyDeviceToHost,
                          st) != cudaSuccess)
        return RBG_ERR_CUDA;
    }
  }
  unsigned bits = 0;
  for (int k = 0; k < nslots; ++k) {
    unsigned b = 0;
    cudaStream_t st = s->dev->host_streams[k];
    if (cudaMemcpyAsync(&b, slots[k].err, sizeof(b), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return RBG_ERR_CUDA;
    bits |= b;
  }
  s->last_launches = launches;
  if (bits & ERR_BIT_NAN) return RBG_ERR_NAN;
  if (bits & ERR_BIT_CAP) return RBG_ERR_CAP;
  return RBG_OK;
}

// ---------------------------------------------------------------------
// focal-plane reductions
// ---------------------------------------------------------------------
namespace rbg {

__global__ void focal_moments_kernel(int64_t n, const uint8_t* status, const double* x, const double* y,
                                     const double* t, const int32_t* group, int32_t n_groups, double* sums) {
  // per-block shared accumulators for up to 64 groups, then one atomic
  // pass; larger group counts go straight to global atomics
  __shared__ double acc[64 * 6];
  const bool shared = n_groups <= 64;
  if (shared)
    for (int k = threadIdx.x; k < n_groups * 6; k += blockDim.x) acc[k] = 0;
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (status[i] != RBG_FOCUS) continue;
    int g = group ? group[i] : 0;
    if (g < 0 || g >= n_groups) continue;
    double v[6] = {1.0, x[i], y[i], x[i] * x[i], y[i] * y[i], t ? t[i] : 0.0};
    double* dst = shared ? acc + g * 6 : sums + g * 6;
    for (int k = 0; k < 6; ++k) atomicAdd(dst + k, v[k]);
  }
  __syncthreads();
  if (shared)
    for (int k = threadIdx.x; k < n_groups * 6; k += blockDim.x)
      if (acc[k] != 0) atomicAdd(sums + k, acc[k]);
}

__global__ void focal_hist_kernel(int64_t n, const uint8_t* status, const double* x, const double* y, int32_t nx,
                                  double xlo, double xhi, int32_t ny, double ylo, double yhi, double* counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (status[i] != RBG_FOCUS) continue;
    double fx = (x[i] - xlo) / (xhi - xlo) * nx, fy = (y[i] - ylo) / (yhi - ylo) * ny;
    if (!(fx >= 0) || !(fy >= 0) || fx >= nx || fy >= ny) continue;
    atomicAdd(counts + (int64_t)fx * ny + (int64_t)fy, 1.0);
  }
}

// SumInRadius (src/AGeoUtil.cxx:18-42) for a batch of probes
__global__ void sum_in_radius_kernel(const double* counts, int32_t nx, double xlo, double xw, int32_t ny,
                                     double ylo, double yw, const double* probes, int nprobe, double* sums) {
  extern __shared__ double part[];
  for (int p = 0; p < nprobe; ++p) part[p * blockDim.x + threadIdx.x] = 0;
  int64_t nb = (int64_t)nx * ny;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
    double c = counts[b];
    if (c <= 0) continue;
    int ix = (int)(b / ny), iy = (int)(b % ny);
    double cx = xlo + (ix + 0.5) * xw, cy = ylo + (iy + 0.5) * yw;
    for (int p = 0; p < nprobe; ++p) {
      double dx = cx - probes[3 * p], dy = cy - probes[3 * p + 1], r = probes[3 * p + 2];
      if (dx * dx + dy * dy <= r * r) part[p * blockDim.x + threadIdx.x] += c;
    }
  }
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int p = 0; p < nprobe; ++p) part[p * blockDim.x + threadIdx.x] += part[p * blockDim.x + threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int p = 0; p < nprobe; ++p) atomicAdd(sums + p, part[p * blockDim.x]);
}

}  // namespace rbg

extern "C" int rbg_focal_moments(int64_t n, const uint8_t* status, const double* x, const double* y,
                                 const double* t, const int32_t* group, int32_t n_groups, double* sums,
                                 void* stream) {
  if (n < 0 || n_groups <= 0 || !status || !x || !y || !sums) return RBG_ERR_ARG;
  if (n == 0) return RBG_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
  focal_moments_kernel<<<blocks, 256, 0, st>>>(n, status, x, y, t, group, n_groups, sums);
  return cudaGetLastError() == cudaSuccess ? RBG_OK : RBG_ERR_CUDA;
}

extern "C" int rbg_focal_histogram(int64_t n, const uint8_t* status, const double* x, const double* y, int32_t nx,
                                   double xlo, double xhi, int32_t ny, double ylo, double yhi, double* counts,
                                   void* stream) {
  if (n < 0 || nx <= 0 || ny <= 0 || !(xhi > xlo) || !(yhi > ylo) || !status || !x || !y || !counts)
    return RBG_ERR_ARG;
  if (n == 0) return RBG_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
  focal_hist_kernel<<<blocks, 256, 0, st>>>(n, status, x, y, nx, xlo, xhi, ny, ylo, yhi, counts);
  return cudaGetLastError() == cudaSuccess ? RBG_OK : RBG_ERR_CUDA;
}

namespace {
struct ProbeBatch {
  double* dprobe = nullptr;
  double* dsum = nullptr;
  ~ProbeBatch() {
    if (dprobe) cudaFree(dprobe);
    if (dsum) cudaFree(dsum);
  }
};
}  // namespace

// AGeoUtil::ContainmentRadius with device SumInRadius probes
extern "C" int rbg_containment_radius(const double* counts, int32_t nx, double xlo, double xhi, int32_t ny,
                                      double ylo, double yhi, double fraction, double* pr, double* px, double* py,
                                      void* stream) {
  if (!counts || nx <= 0 || ny <= 0 || !pr || !px || !py || !(xhi > xlo) || !(yhi > ylo)) return RBG_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double xw = (xhi - xlo) / nx, yw = (yhi - ylo) / ny;
  ProbeBatch pb;
  const int kMaxProbe = 8;
  if (cudaMalloc(&pb.dprobe, 3 * kMaxProbe * sizeof(double)) != cudaSuccess) return RBG_ERR_NOMEM;
  if (cudaMalloc(&pb.dsum, kMaxProbe * sizeof(double)) != cudaSuccess) return RBG_ERR_NOMEM;
  const int block = 256;
  const int blocks = (int)std::min<int64_t>(((int64_t)nx * ny + block - 1) / block, (int64_t)sm_count() * 4);
  int failed = 0;
  auto probe = [&](int np, const double* xyr, double* out) {
    if (failed) {
      for (int i = 0; i < np; ++i) out[i] = 0;
      return;
    }
    if (cudaMemcpyAsync(pb.dprobe, xyr, 3 * np * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(pb.dsum, 0, np * sizeof(double), st) != cudaSuccess) {
      failed = 1;
      return;
    }
    sum_in_radius_kernel<<<blocks, block, np * block * sizeof(double), st>>>(counts, nx, xlo, xw, ny, ylo, yw,
                                                                             pb.dprobe, np, pb.dsum);
    if (cudaMemcpyAsync(out, pb.dsum, np * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      failed = 1;
    }
  };
  auto sum_in_radius = [&](double x, double y, double r) {
    double q[3] = {x, y, r}, o = 0;
    probe(1, q, &o);
    return o;
  };
  // moments from bin centres: r = 1 probe at "infinite" radius is not enough,
  // so read the histogram moments with one pass of 5 probes-worth of sums
  std::vector<double> hc((size_t)nx * ny);
  if (cudaMemcpyAsync(hc.data(), counts, hc.size() * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return RBG_ERR_CUDA;
  double sw = 0, sx = 0, sy = 0, sxx = 0, syy = 0;
  for (int ix = 0; ix < nx; ++ix) {
    double cx = xlo + (ix + 0.5) * xw;
    for (int iy = 0; iy < ny; ++iy) {
      double cy = ylo + (iy + 0.5) * yw, c = hc[(size_t)ix * ny + iy];
      sw += c;
      sx += c * cx;
      sy += c * cy;
      sxx += c * cx * cx;
      syy += c * cy * cy;
    }
  }
  double x = sw ? sx / sw : 0, y = sw ? sy / sw : 0;
  double vx = sw ? sxx / sw - x * x : 0, vy = sw ? syy / sw - y * y : 0;
  double sdx = vx > 0 ? std::sqrt(vx) : 0, sdy = vy > 0 ? std::sqrt(vy) : 0;
  double r = std::sqrt(sdx * sdx + sdy * sdy) * 1.5;
  double dr = 0.1 * r;
  double sum_goal = sw * fraction;
  int no_shift = 0, no_stable = 0;
  for (int i = 0; i < 100 && no_shift < 30; i++) {
    bool stable_r = false, stable_x = true, stable_y = true;
    double sum0 = sum_in_radius(x, y, r);
    double next_r = r;
    if (sum0 < sum_goal) {
      double sum1 = sum_in_radius(x, y, r + dr);
      if (sum1 == sum0) {
        dr *= 2.;
        continue;
      }
      next_r = r + dr * (sum_goal - sum0) / (sum1 - sum0);
    } else if (sum0 != sum_goal) {
      double sum1 = sum_in_radius(x, y, r - dr);
      if (sum1 == sum0) {
        dr *= 2.;
        continue;
      }
      next_r = r - dr * (sum0 - sum_goal) / (sum0 - sum1);
    }
    if (next_r < 0.) next_r = 0.5 * r;
    if (next_r < 0.5 * r) next_r = 0.5 * r;
    if (next_r > 2. * r) next_r = 2. * r;
    stable_r = std::fabs(next_r - r) < 0.0001 * r;
    r = next_r;
    {
      double sum1 = sum_in_radius(x, y, r);
      dr *= sum0 != sum_goal ? std::fabs((sum1 - sum_goal) / (sum0 - sum_goal)) : 0.5;
      if (dr > 0.5 * r) dr = 0.5 * r;
      if (dr < 0.0005 * r) dr = 0.0005 * r;
      no_shift++;
      for (double dx = 0.25 * r; dx > 0.1 * dr; dx *= 0.25) {
        double q[6] = {x + dx, y, r, x - dx, y, r}, o[2];
        probe(2, q, o);
        double sx1 = o[0], sx2 = o[1];
        while (sx1 > sum1) {
          no_shift = 0;
          x += dx;
          sx2 = sum1;
          sum1 = sx1;
          sx1 = sum_in_radius(x + dx, y, r);
          stable_x = false;
        }
        while (sx2 > sum1) {
          no_shift = 0;
          x -= dx;
          sx1 = sum1;
          sum1 = sx2;
          sx2 = sum_in_radius(x - dx, y, r);
          stable_x = false;
        }
      }
    }
    for (double dy = 0.1 * r; dy > 0.1 * dr; dy *= 0.25) {
      double q[9] = {x, y, r, x, y + dy, r, x, y - dy, r}, o[3];
      probe(3, q, o);
      double sum1 = o[0], sy1 = o[1], sy2 = o[2];
      while (sy1 > sum1) {
        no_shift = 0;
        y += dy;
        sy2 = sum1;
        sum1 = sy1;
        sy1 = sum_in_radius(x, y + dy, r);
        stable_y = false;
      }
      while (sy2 > sum1) {
        no_shift = 0;
        y -= dy;
        sy1 = sum1;
        sum1 = sy2;
        sy2 = sum_in_radius(x, y - dy, r);
        stable_y = false;
      }
    }
    if (stable_r && stable_x && stable_y) no_stable++;
    else no_stable = 0;
    if (no_stable >= 4) break;
  }
  if (failed) return RBG_ERR_CUDA;
  *pr = r;
  *px = x;
  *py = y;
  return RBG_OK;
}
