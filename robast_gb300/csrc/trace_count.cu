// trace_count.cu -- the mixed-precision tracer with its work counted.
//
// This translation unit compiles the lean instance of the persistent tracer
// (scenes of boxes and aspheric disks: two-mirror telescopes) with
// RBG_COUNT_EVENTS defined, so that every counted event of events.h adds to
// a per-block tally; the totals give the FP64 and FP32 flops of a trace from
// the per-event counts of rbg_event_flops.  The counting build traces the
// same rays to the same results; it is a measurement, not the timed path.
#define RBG_COUNT_EVENTS 1
#include "trace_mixed.cuh"

namespace rbg {

// the lean instance's features, plus a bit no scene uses: a distinct
// instantiation of the kernel and of its device functions
constexpr unsigned kCountInstance = 0x80000000u;

}  // namespace rbg

using namespace rbg;

// Flops of one event, counted from the formulas it evaluates (an FMA, a
// multiply-add, counts 2; a square root or a division 1):
//   SEGMENT      p += (s + push) d: 1 add + 3 FMA                        FP64 7
//   RAY          |d|^2 (5), refined 1/sqrt (9), d * inv (3)             FP64 17
//   XFORM_T      p - t                                                   FP64 3
//   XFORM_G      R^T (p - t) (18) and R^T d (15)                         FP64 33
//   POLISH       q = p + t d (3 FMA), h2 (3), poly * h (1),
//                e = s (x - qz) (2), t += e (1)                          FP64 13
//   HORNER64     one FMA term of a sag or slope polynomial               FP64 2
//   ACCEPT       q.x, q.y (2 FMA), h2 (3)                                FP64 7
//   NORMAL       h2 (3), g = -2 p F' (4), |g|^2 (4), refined
//                1/sqrt (9), n = g * inv (2), n . d (5)                  FP64 27
//   NORMAL_EXACT r (4), four safeties (14), the winning face's
//                normalised gradient (13), n . d (5), sags (8)           FP64 44
//   CONTAINS_EX  h2 (3), r^2 bounds (2), poly * h (1), two sags (2)      FP64 8
//   BOX64        o = p - c (3), per axis refined 1/d and a plane
//                distance (6)                                            FP64 21
//   DIST_EXACT   the reference's Newton: first guess (25) and about
//                three iterations of 45 + 4 npol (8 terms: 77)           FP64 256
//   WALL_EXACT   the cylinder roots of DistToInner/Outer                FP64 35
//   REFLECT      d.n (5), d - 2 (d.n) n (7), renormalisation (11),
//                time (3), step back (6)                                 FP64 32
//   NEWTON32     h2 (3), gradient (5), d.g (5), step (3), advance
//                (7), stop test (6)                                      FP32 29
//   HORNER32     sag term (2), slope term (4)                            FP32 6
//   SCREEN32     a float box, tube, wall or sag screen                   FP32 25
static const double kEventFp64[EV_COUNT] = {7, 17, 3, 33, 13, 2, 7, 27, 44, 8, 21, 256, 35, 32, 0, 0, 0};
static const double kEventFp32[EV_COUNT] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 29, 6, 25};

extern "C" int rbg_event_kinds(void) { return EV_COUNT; }

extern "C" int rbg_event_flops(int32_t kind, double* fp64, double* fp32) {
  if (kind < 0 || kind >= EV_COUNT || !fp64 || !fp32) return RBG_ERR_ARG;
  *fp64 = kEventFp64[kind];
  *fp32 = kEventFp32[kind];
  return RBG_OK;
}

namespace rbg {
size_t ray_order_bytes(int64_t n);
int build_ray_order(const KernelRays& in, int64_t n, void* ws, KernelRays* sorted, cudaStream_t st);
}  // namespace rbg

// rbg_trace (mixed precision) through the counting build: counts[k] gets
// the number of events of kind k (events.h) the trace made
extern "C" int rbg_trace_count_events(rbg_scene* s, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* opts,
                                      void* stream, uint64_t* counts, int32_t n_counts) {
  if (!s || !in || !out || !opts || !counts || n_counts < EV_COUNT) return RBG_ERR_ARG;
  if (in->n < 0 || opts->limit <= 0) return RBG_ERR_ARG;
  if (in->n > 0 && (!in->x || !in->y || !in->z || !in->dx || !in->dy || !in->dz || !in->lambda)) return RBG_ERR_ARG;
  if (s->features != 0) return RBG_ERR_UNSUPPORTED;  // only the lean instance is counted
  int rc = ensure_device(s);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned long long zero[EV_COUNT] = {0};
  if (cudaMemcpyToSymbolAsync(rbg_event_totals, zero, sizeof(zero), 0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(s->dev->err_flags, 0, sizeof(unsigned), st) != cudaSuccess)
    return RBG_ERR_CUDA;
  KernelRays kr{in->x, in->y, in->z, in->t, in->dx, in->dy, in->dz, in->lambda};
  KernelOut ko{out->status, out->npoints, out->last_node, out->x, out->y, out->z, out->t,
               out->dx, out->dy, out->dz, out->hist_cap, out->hist_xyzt, out->hist_node};
  // the take-up order of rbg_trace, when the caller lends its workspace
  if (in->n >= (1 << 14) && opts->ray_order == RBG_ORDER_SPATIAL && opts->workspace &&
      opts->workspace_bytes >= ray_order_bytes(in->n))
    if ((rc = build_ray_order(kr, in->n, opts->workspace, &kr, st))) return rc;
  rbg_trace_opts o = *opts;
  if (o.compaction == 0) o.compaction = s->tuned_compaction;
  if (in->n > 0 &&
      (rc = launch_mixed_impl<kCountInstance>(s->dev->view, kr, ko, in->n, o, st, s->dev->err_flags, s->dev->counter)))
    return rc;
  unsigned long long tot[EV_COUNT];
  if (cudaMemcpyFromSymbolAsync(tot, rbg_event_totals, sizeof(tot), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return RBG_ERR_CUDA;
  for (int k = 0; k < EV_COUNT; ++k) counts[k] = tot[k];
  return RBG_OK;
}
