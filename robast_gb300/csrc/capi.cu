// capi.cu -- C ABI of the tracer: device upload of a flattened scene, its
// workspace reservation, and device- and host-buffer tracing.
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
  for (void*& e : s->tev) {
    if (e) cudaEventDestroy(static_cast<cudaEvent_t>(e));
    e = nullptr;
  }
  s->timing = false;
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
  // one 256-byte block: the error word at 0, the persistent kernel's queue
  // head at 8, the adjoint's skip counter at 16
  void* ef = nullptr;
  if (cudaMalloc(&ef, 256) != cudaSuccess) {
    for (void* p : d->allocations) cudaFree(p);
    delete d;
    return RBG_ERR_NOMEM;
  }
  d->allocations.push_back(ef);
  d->err_flags = static_cast<unsigned*>(ef);
  d->counter = reinterpret_cast<unsigned long long*>(static_cast<char*>(ef) + 8);
  d->adj_skip = reinterpret_cast<unsigned long long*>(static_cast<char*>(ef) + 16);
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

// Per-device cache: a process may drive several GPUs.
constexpr int kMaxDevices = 64;

int sm_count() {
  static int cached[kMaxDevices] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
  if (cached[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = v > 0 ? v : 1;
  }
  return cached[dev];
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

// CUDA events around the tracer kernel of every later rbg_trace on the scene
// (created here, destroyed with the scene's device state)
extern "C" int rbg_scene_set_timing(rbg_scene* s, int32_t on) {
  if (!s) return RBG_ERR_ARG;
  int rc = ensure_device(s);
  if (rc) return rc;
  if (on && !s->tev[0]) {
    for (auto& e : s->tev) {
      cudaEvent_t ev;
      if (cudaEventCreate(&ev) != cudaSuccess) return RBG_ERR_CUDA;
      e = ev;
    }
  }
  s->timing = on != 0;
  return RBG_OK;
}

extern "C" double rbg_last_kernel_ms(const rbg_scene* s) { return s && s->timing ? s->last_kernel_ms : -1.0; }

// the two tracer launchers (trace_mixed.cu, trace_fp64.cu)
namespace rbg {
size_t ray_order_bytes(int64_t n);
int build_ray_order(const KernelRays& in, int64_t n, void* ws, KernelRays* sorted, cudaStream_t st);
int mixed_block_size(unsigned features);
int launch_mixed(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o,
                 cudaStream_t st, unsigned* err_flags, unsigned long long* counter, int* launches);
// below this many rays the mixed tracer takes rays up in input order
constexpr int64_t kOrderMinRays = 1 << 14;
bool want_ray_order(const rbg_trace_opts& o, int64_t n) {
  return o.ray_order == RBG_ORDER_SPATIAL && n >= kOrderMinRays && ray_order_bytes(n) > 0;
}
int launch_fp64(const DevScene& S, const KernelRays& in, const KernelOut& out, int64_t n, const rbg_trace_opts& o,
                cudaStream_t st, unsigned* err_flags, int* launches);
}

namespace rbg {
int host_workspace_reserve(rbg_scene* s, int64_t max_rays, int32_t hist_cap);  // below
}

extern "C" size_t rbg_trace_workspace_bytes(int64_t n) { return n >= kOrderMinRays ? ray_order_bytes(n) : 0; }

// Every device allocation a scene makes for tracing up to max_rays rays,
// made here once on the current device: the scene tables (upload), the
// take-up order workspace of rbg_trace and the two pipeline slots of
// rbg_trace_host for hist_cap history points.  (No tracer kernel recurses,
// so the per-thread stack the driver sizes at each launch from the kernel's
// static need is enough: no stack limit is set anywhere.)  A
// smaller reservation than an earlier one keeps the larger workspaces.
extern "C" int rbg_scene_reserve(rbg_scene* s, int64_t max_rays, int32_t hist_cap) {
  if (!s || max_rays < 0 || hist_cap < 0) return RBG_ERR_ARG;
  int rc = ensure_device(s);
  if (rc) return rc;
  const size_t need = max_rays >= kOrderMinRays ? ray_order_bytes(max_rays) : 0;
  if (need > s->order_ws_bytes) {
    // the old workspace may still be read by work queued on a stream
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
  return host_workspace_reserve(s, max_rays, hist_cap);
}

namespace rbg {
namespace {
// Everything a trace puts on the stream -- the error word's reset, the
// take-up order, the tracer kernel (and its timing events) -- without
// reading anything back
int trace_enqueue(rbg_scene* s, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* opts, cudaStream_t st,
                  bool timed) {
  if (!s || !in || !out || !opts) return RBG_ERR_ARG;
  if (in->n < 0 || opts->limit <= 0) return RBG_ERR_ARG;
  if (in->n > 0 && (!in->x || !in->y || !in->z || !in->dx || !in->dy || !in->dz || !in->lambda)) return RBG_ERR_ARG;
  if (out->hist_cap < 0 || (out->hist_cap > 0 && (!out->hist_xyzt || !out->hist_node))) return RBG_ERR_ARG;
  if (opts->workspace && (reinterpret_cast<uintptr_t>(opts->workspace) & 255)) return RBG_ERR_ARG;
  int rc = ensure_device(s);
  if (rc) return rc;
  s->last_launches = 0;
  if (cudaMemsetAsync(s->dev->err_flags, 0, sizeof(unsigned), st) != cudaSuccess) return RBG_ERR_CUDA;
  if (in->n == 0) return RBG_OK;
  KernelRays kr{in->x, in->y, in->z, in->t, in->dx, in->dy, in->dz, in->lambda};
  KernelOut ko{out->status, out->npoints, out->last_node, out->x, out->y, out->z, out->t,
               out->dx, out->dy, out->dz, out->hist_cap, out->hist_xyzt, out->hist_node};
  int launches = 0;
  rbg_trace_opts o = *opts;
  if (o.compaction == 0) o.compaction = s->tuned_compaction;
  if (o.block_size == 0 && o.precision == RBG_PREC_MIXED) o.block_size = s->tuned_block;
  // the take-up order needs a workspace: the caller's, else the one
  // rbg_scene_reserve sized; a batch beyond both is taken up in input order
  // (same results, nothing allocated)
  if (want_ray_order(o, in->n)) {
    const size_t need = ray_order_bytes(in->n);
    void* ws = nullptr;
    if (o.workspace && o.workspace_bytes >= need) ws = o.workspace;
    else if (s->order_ws && s->order_ws_bytes >= need) ws = s->order_ws;
    if (ws) {
      if ((rc = build_ray_order(kr, in->n, ws, &kr, st))) return rc;
      launches += 7;
    }
  }
  cudaEvent_t* tev = reinterpret_cast<cudaEvent_t*>(s->tev);
  if (timed && cudaEventRecord(tev[0], st) != cudaSuccess) return RBG_ERR_CUDA;
  if (o.precision == RBG_PREC_MIXED)
    rc = launch_mixed(s->dev->view, kr, ko, in->n, o, st, s->dev->err_flags, s->dev->counter, &launches);
  else
    rc = launch_fp64(s->dev->view, kr, ko, in->n, o, st, s->dev->err_flags, &launches);
  if (rc) return rc;
  if (timed && cudaEventRecord(tev[1], st) != cudaSuccess) return RBG_ERR_CUDA;
  s->last_launches = launches;
  return RBG_OK;
}

int status_of(unsigned bits) {
  if (bits & ERR_BIT_NAN) return RBG_ERR_NAN;
  if (bits & ERR_BIT_CAP) return RBG_ERR_CAP;
  return RBG_OK;
}
}  // namespace
}  // namespace rbg

extern "C" int rbg_trace(rbg_scene* s, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* opts,
                         void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool timed = s && s->timing;
  int rc = trace_enqueue(s, in, out, opts, st, timed);
  if (rc) return rc;
  if (in->n == 0) return RBG_OK;
  unsigned bits = 0;
  if ((rc = read_errors(s, st, &bits))) return rc;
  cudaEvent_t* tev = reinterpret_cast<cudaEvent_t*>(s->tev);
  if (timed && cudaEventElapsedTime(&s->last_kernel_ms, tev[0], tev[1]) != cudaSuccess) return RBG_ERR_CUDA;
  return status_of(bits);
}

// rbg_trace without the read-back: stream-ordered, so that a host loop or
// a CUDA graph can hold it
extern "C" int rbg_trace_async(rbg_scene* s, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* opts,
                               void* stream) {
  if (s && !s->dev) return RBG_ERR_ARG;  // the scene must be on the device already (rbg_scene_reserve)
  return trace_enqueue(s, in, out, opts, static_cast<cudaStream_t>(stream), false);
}

extern "C" int rbg_trace_status(rbg_scene* s, void* stream) {
  if (!s || !s->dev) return RBG_ERR_ARG;
  unsigned bits = 0;
  int rc = read_errors(s, static_cast<cudaStream_t>(stream), &bits);
  return rc ? rc : status_of(bits);
}

extern "C" int rbg_scene_tuning(const rbg_scene* s, int32_t* block_size, int32_t* compaction) {
  if (!s) return RBG_ERR_ARG;
  const int fixed = mixed_block_size(s->features);
  if (block_size) *block_size = fixed ? fixed : (s->tuned_block ? s->tuned_block : 256);
  if (compaction) *compaction = s->tuned_compaction ? s->tuned_compaction : 32;
  return RBG_OK;
}

extern "C" int rbg_scene_set_tuning(rbg_scene* s, int32_t block_size, int32_t compaction) {
  if (!s || compaction < 0 || compaction > 32) return RBG_ERR_ARG;
  if (block_size != 0 && block_size != 128 && block_size != 256) return RBG_ERR_ARG;
  s->tuned_block = block_size;
  s->tuned_compaction = compaction;
  return RBG_OK;
}

// The autotuner of the mixed tracer: trace the caller's rays once to warm
// up, then once per candidate (block size, compaction threshold) -- block
// sizes 256 and 128 for scenes the lean instance traces, the instance's
// fixed 128 otherwise; thresholds 1, 8, 16, 32 -- timed with events on the
// stream, and keep the fastest in the scene (used by every later call
// whose options leave them at 0).  The results in `out` are those of any
// single trace: they depend on neither.
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
  const bool lean = mixed_block_size(s->features) == 0;
  static const int32_t kLeanBlocks[] = {256, 128};
  const int n_blocks = lean ? 2 : 1;
  constexpr int kCand = sizeof(kCandidates) / sizeof(kCandidates[0]);
  // two rounds over every candidate, each candidate's best time kept: the
  // candidates differ by a few percent, one sample each can be misread
  float ms_of[2][kCand];
  for (int round = 0; round < 2; ++round)
    for (int b = 0; b < n_blocks && (rc == RBG_OK || rc == RBG_ERR_NAN || rc == RBG_ERR_CAP); ++b) {
      o.block_size = lean ? kLeanBlocks[b] : 0;
      for (int ci = 0; ci < kCand; ++ci) {
        o.compaction = kCandidates[ci];
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
        ms_of[b][ci] = round == 0 ? ms : (ms < ms_of[b][ci] ? ms : ms_of[b][ci]);
      }
    }
  float best_ms = 0.f;
  int32_t best = 32, best_block = lean ? 256 : 0;
  bool first = true;
  for (int b = 0; b < n_blocks; ++b)
    for (int ci = 0; ci < kCand; ++ci)
      if (first || ms_of[b][ci] < best_ms) {
        best_ms = ms_of[b][ci];
        best = kCandidates[ci];
        best_block = lean ? kLeanBlocks[b] : 0;
        first = false;
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != RBG_OK && rc != RBG_ERR_NAN && rc != RBG_ERR_CAP) return rc;
  s->tuned_compaction = best;
  s->tuned_block = best_block;
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
    // a call that failed part-way may have left copies queued on the
    // pipeline streams: let them finish before the old block goes
    for (cudaStream_t st : s->dev->host_streams)
      if (st && cudaStreamSynchronize(st) != cudaSuccess) return RBG_ERR_CUDA;
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

// rays per pipeline chunk and number of slots for a batch of n rays
void host_plan(int64_t n, int64_t* cap, int* nslots) {
  *cap = ((n < kHostChunk ? n : kHostChunk) + 255) / 256 * 256;
  const int64_t chunks = *cap > 0 ? (n + *cap - 1) / *cap : 0;
  *nslots = chunks < kHostStreams ? (int)chunks : kHostStreams;
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

int host_workspace_reserve(rbg_scene* s, int64_t max_rays, int32_t hist_cap) {
  int64_t cap;
  int nslots;
  host_plan(max_rays, &cap, &nslots);
  if (nslots == 0) return RBG_OK;
  char* ws = nullptr;
  return grow_workspace(s, slot_bytes(cap, hist_cap) * nslots, &ws);
}

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
  const int64_t n = in->n;
  s->last_launches = 0;
  if (n == 0) return RBG_OK;
  const int hcap = out->hist_cap;
  int64_t cap;
  int nslots;
  host_plan(n, &cap, &nslots);
  const int64_t chunks = (n + cap - 1) / cap;
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
    if (o.block_size == 0 && o.precision == RBG_PREC_MIXED) o.block_size = s->tuned_block;
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
