// events.h -- counted work of the mixed-precision tracer, for its roofline.
//
// The tracer's arithmetic is not a fixed number of operations per ray or per
// segment: how many Newton iterations and FP64 polish steps a crossing
// takes, whether a screen decides or its FP64 fallback runs, depends on the
// ray.  A counting build of the tracer (trace_count.cu, the only translation
// unit that defines RBG_COUNT_EVENTS) tallies each such event as it happens;
// everywhere else RBG_EVENT compiles to nothing.  The FP64 and FP32 flops of
// each event are counted from the formulas it evaluates (rbg_event_flops in
// trace_count.cu lists them), an FMA counting two.
#pragma once

namespace rbg {

enum RbgEvent : int {
  EV_SEGMENT = 0,         // a boundary step: the point moves along the ray (FP64)
  EV_RAY,                 // a ray taken up: direction normalised (FP64)
  EV_XFORM_T,             // master -> local point, translation node (FP64)
  EV_XFORM_G,             // master -> local point and direction, general node (FP64)
  EV_POLISH,              // one FP64 polish step of an aspheric root (without its Horner terms)
  EV_HORNER64,            // one FP64 Horner term (polish, containment, normal)
  EV_ACCEPT,              // an aspheric root's acceptance test (FP64)
  EV_NORMAL,              // an aspheric face normal (FP64, without its Horner terms)
  EV_NORMAL_EXACT,        // the full closest-surface normal choice (FP64, without its Horner terms)
  EV_CONTAINS_EXACT,      // an FP64 containment test of an aspheric disk (without its Horner terms)
  EV_BOX64,               // an FP64 box crossing (slab) test
  EV_DIST_EXACT,          // an FP64 reference Newton solve (fallback of the FP32 one)
  EV_WALL_EXACT,          // an FP64 cylinder-wall crossing of an aspheric disk
  EV_REFLECT,             // a specular reflection (FP64)
  EV_NEWTON32,            // one FP32 Newton iteration (without its Horner terms)
  EV_HORNER32,            // one FP32 Horner term of the Newton iteration
  EV_SCREEN32,            // an FP32 screen: a box / tube / wall / sag test
  EV_COUNT
};

}  // namespace rbg

#ifdef RBG_COUNT_EVENTS
// per-block tallies; the counting kernel zeroes them on entry and adds them
// to the device totals on exit
static __shared__ unsigned long long rbg_block_events[rbg::EV_COUNT];
static __device__ unsigned long long rbg_event_totals[rbg::EV_COUNT];
namespace rbg {
// one shared-memory atomic per converged group of lanes (their counts summed)
__device__ __forceinline__ void count_event(int k, unsigned n) {
  const unsigned m = __activemask();
  const unsigned tot = __reduce_add_sync(m, n);
  if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(&rbg_block_events[k], (unsigned long long)tot);
}
}  // namespace rbg
#define RBG_EVENT(k) ::rbg::count_event((k), 1u)
#define RBG_EVENT_N(k, n) ::rbg::count_event((k), (unsigned)(n))
#else
#define RBG_EVENT(k) ((void)0)
#define RBG_EVENT_N(k, n) ((void)0)
#endif
