// shoot.cu -- ARayShooter generators (src/ARayShooter.cxx:122-459) on the
// GPU, writing DEVICE ray arrays: one thread per ray, ray i drawing from the
// Philox stream (seed, first_id + i, stream 1) exactly as the host
// generators of shoot.cpp do.  Every position and direction is computed
// operation by operation in the host's order with round-to-nearest
// intrinsics (no contraction into FMAs), so the rays of the random-circle,
// -cone and -rectangle sources and of the grids equal the host's bit for
// bit; the sphere sources call cos / sin / acos, which may differ from the
// host library's in the last bit.
#include <cuda_runtime.h>

#include <cmath>

#include "device_state.cuh"
#include "philox.h"
#include "robast_gb.h"

namespace rbg {
namespace {

constexpr int kShootThreads = 256;

struct ShootArgs {
  int kind;
  double p[4];
  double R[9];
  double t[3];
  double ld[3];  // the local direction of the parallel sources
  bool has_rot;
  uint64_t seed, first_id;
  double lambda;
  int nr, nphi, nx, ny;
};

__device__ __forceinline__ double dot_rn(const double* r, double a, double b, double c) {
  return __dadd_rn(__dadd_rn(__dmul_rn(r[0], a), __dmul_rn(r[1], b)), __dmul_rn(r[2], c));
}
__device__ __forceinline__ void rot_rn(const ShootArgs& A, const double* v, double* o) {
  if (!A.has_rot) {
    o[0] = v[0];
    o[1] = v[1];
    o[2] = v[2];
    return;
  }
  for (int i = 0; i < 3; ++i) o[i] = dot_rn(A.R + 3 * i, v[0], v[1], v[2]);
}
__device__ __forceinline__ void place_rn(const ShootArgs& A, const double* l, double* x) {
  double tmp[3];
  rot_rn(A, l, tmp);
  for (int k = 0; k < 3; ++k) x[k] = __dadd_rn(tmp[k], A.t[k]);
}

__global__ void __launch_bounds__(kShootThreads) shoot_kernel(ShootArgs A, int64_t n, double* X, double* Y,
                                                              double* Z, double* T, double* DX, double* DY,
                                                              double* DZ, double* L) {
  const double kTwoPi = 2.0 * 3.14159265358979323846;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double x[3], d[3];
    rot_rn(A, A.ld, d);
    RayRng g;
    g.init(A.seed, A.first_id + (uint64_t)i, 1);
    switch (A.kind) {
      case RBG_SHOOT_RANDOM_CIRCLE: {
        const double rmax = A.p[0];
        double rx = 0, ry = 0;
        for (int tries = 0; tries < 1000; ++tries) {
          const Philox4 b = g.next();
          rx = __dadd_rn(-rmax, __dmul_rn(__dmul_rn(2.0, rmax), u53(b.v[0], b.v[1])));
          ry = __dadd_rn(-rmax, __dmul_rn(__dmul_rn(2.0, rmax), u53(b.v[2], b.v[3])));
          if (__dsqrt_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry))) <= rmax) break;
        }
        const double l[3] = {rx, ry, 0};
        place_rn(A, l, x);
        break;
      }
      case RBG_SHOOT_RANDOM_CONE: {
        const double r = A.p[0], dd = A.p[1];
        double px = 0, py = 0;
        for (int tries = 0; tries < 1000; ++tries) {
          const Philox4 b = g.next();
          px = __dadd_rn(-r, __dmul_rn(__dmul_rn(2.0, r), u53(b.v[0], b.v[1])));
          py = __dadd_rn(-r, __dmul_rn(__dmul_rn(2.0, r), u53(b.v[2], b.v[3])));
          if (!(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)) > __dmul_rn(r, r))) break;
        }
        const double goal[3] = {px, py, dd};
        double tmp[3];
        rot_rn(A, goal, tmp);
        for (int k = 0; k < 3; ++k) {
          x[k] = A.t[k];
          d[k] = __dsub_rn(__dadd_rn(tmp[k], A.t[k]), A.t[k]);
        }
        break;
      }
      case RBG_SHOOT_RANDOM_RECTANGLE: {
        const Philox4 b = g.next();
        const double l[3] = {__dadd_rn(-A.p[0] / 2., __dmul_rn(A.p[0], u53(b.v[0], b.v[1]))),
                             __dadd_rn(-A.p[1] / 2., __dmul_rn(A.p[1], u53(b.v[2], b.v[3]))), 0};
        place_rn(A, l, x);
        break;
      }
      case RBG_SHOOT_RANDOM_SPHERE: {
        const Philox4 b = g.next();
        const double z = __dadd_rn(-1.0, __dmul_rn(2.0, u53(b.v[0], b.v[1])));
        const double phi = __dmul_rn(kTwoPi, u53(b.v[2], b.v[3]));
        const double s = __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(z, z)));
        double sp, cp;
        sincos(phi, &sp, &cp);
        d[0] = __dmul_rn(s, cp);
        d[1] = __dmul_rn(s, sp);
        d[2] = z;
        x[0] = A.t[0];
        x[1] = A.t[1];
        x[2] = A.t[2];
        break;
      }
      case RBG_SHOOT_RANDOM_SPHERICAL_CONE: {
        const Philox4 b = g.next();
        const double c0 = cos(__dmul_rn(A.p[0], 3.14159265358979323846) / 180.0);
        const double ran = __dadd_rn(c0, __dmul_rn(__dsub_rn(1.0, c0), u53(b.v[0], b.v[1])));
        const double th = acos(ran);
        const double phi = __dmul_rn(kTwoPi, u53(b.v[2], b.v[3]));
        double st, ct, sp, cp;
        sincos(th, &st, &ct);
        sincos(phi, &sp, &cp);
        const double l[3] = {__dmul_rn(st, cp), __dmul_rn(st, sp), ct};
        rot_rn(A, l, d);
        x[0] = A.t[0];
        x[1] = A.t[1];
        x[2] = A.t[2];
        break;
      }
      case RBG_SHOOT_RECTANGLE: {
        const int ix = (int)(i / A.ny), iy = (int)(i - (int64_t)ix * A.ny);
        const double deltax = A.nx == 1 ? A.p[0] / 2 : A.p[0] / (A.nx - 1);
        const double deltay = A.ny == 1 ? A.p[1] / 2 : A.p[1] / (A.ny - 1);
        const double l[3] = {__dsub_rn(__dmul_rn((double)ix, deltax), A.p[0] / 2),
                             __dsub_rn(__dmul_rn((double)iy, deltay), A.p[1] / 2), 0};
        place_rn(A, l, x);
        break;
      }
      default: {  // RBG_SHOOT_CIRCLE: the centre, then ring k of nphi k points
        if (i == 0) {
          x[0] = A.t[0];
          x[1] = A.t[1];
          x[2] = A.t[2];
          break;
        }
        // ring k (1-based) holds points 1 + nphi k (k - 1) / 2 .. 1 + nphi k (k + 1) / 2 - 1
        int64_t k = (int64_t)floor((-1.0 + sqrt(1.0 + 8.0 * (double)(i - 1) / A.nphi)) / 2.0) + 1;
        while (k > 1 && 1 + A.nphi * k * (k - 1) / 2 > i) --k;
        while (1 + A.nphi * (k + 1) * k / 2 <= i) ++k;
        const int64_t j = i - (1 + A.nphi * k * (k - 1) / 2);
        const double r = A.p[0] * (double)k / A.nr;
        const double phi = 2 * 3.14159265358979323846 / A.nphi / (double)k * (double)j;
        double sp, cp;
        sincos(phi, &sp, &cp);
        const double l[3] = {__dmul_rn(r, cp), __dmul_rn(r, sp), 0};
        place_rn(A, l, x);
        break;
      }
    }
    X[i] = x[0];
    Y[i] = x[1];
    Z[i] = x[2];
    if (T) T[i] = 0.0;
    DX[i] = d[0];
    DY[i] = d[1];
    DZ[i] = d[2];
    L[i] = A.lambda;
  }
}

}  // namespace
}  // namespace rbg

// rbg_shoot with DEVICE outputs (robast_gb.h)
extern "C" int rbg_shoot_device(int32_t kind, const double* p, int64_t n, const double* rot, const double* tr,
                                const double* dir, uint64_t seed, uint64_t first_id, double lambda,
                                rbg_rays* out, void* stream) {
  using namespace rbg;
  if (!out || !out->x || !out->y || !out->z || !out->dx || !out->dy || !out->dz || !out->lambda) return RBG_ERR_ARG;
  if (n < 0 || out->n < 0) return RBG_ERR_ARG;
  ShootArgs A{};
  A.kind = kind;
  A.has_rot = rot != nullptr;
  for (int k = 0; k < 9; ++k) A.R[k] = rot ? rot[k] : (k % 4 == 0 ? 1.0 : 0.0);
  for (int k = 0; k < 3; ++k) A.t[k] = tr ? tr[k] : 0.0;
  A.ld[0] = dir ? dir[0] : 0.0;
  A.ld[1] = dir ? dir[1] : 0.0;
  A.ld[2] = dir ? dir[2] : 1.0;
  A.seed = seed;
  A.first_id = first_id;
  A.lambda = lambda;
  int64_t count = n;
  switch (kind) {
    case RBG_SHOOT_CIRCLE:
      if (!p) return RBG_ERR_ARG;
      A.p[0] = p[0];
      A.nr = (int)p[1];
      A.nphi = (int)p[2];
      if (0 > p[0] || A.nr < 1 || A.nphi < 1) count = 0;
      else count = 1 + (int64_t)A.nphi * A.nr * (A.nr + 1) / 2;
      break;
    case RBG_SHOOT_RECTANGLE:
      if (!p) return RBG_ERR_ARG;
      A.p[0] = p[0];
      A.p[1] = p[1];
      A.nx = (int)p[2];
      A.ny = (int)p[3];
      count = (p[0] < 0 || p[1] < 0 || A.nx < 1 || A.ny < 1) ? 0 : (int64_t)A.nx * A.ny;
      break;
    case RBG_SHOOT_RANDOM_CIRCLE:
      if (!p) return RBG_ERR_ARG;
      A.p[0] = p[0];
      if (0 > p[0]) count = 0;
      break;
    case RBG_SHOOT_RANDOM_CONE:
    case RBG_SHOOT_RANDOM_RECTANGLE:
      if (!p) return RBG_ERR_ARG;
      A.p[0] = p[0];
      A.p[1] = p[1];
      if (kind == RBG_SHOOT_RANDOM_RECTANGLE && (p[0] < 0 || p[1] < 0)) count = 0;
      break;
    case RBG_SHOOT_RANDOM_SPHERICAL_CONE:
      if (!p) return RBG_ERR_ARG;
      A.p[0] = p[0];
      break;
    case RBG_SHOOT_RANDOM_SPHERE:
      break;
    default:
      return RBG_ERR_ARG;
  }
  if (count > out->n) return RBG_ERR_ARG;
  out->n = count;
  if (count == 0) return RBG_OK;
  const int64_t want = (count + kShootThreads - 1) / kShootThreads;
  const int blocks = (int)(want < (int64_t)sm_count() * 16 ? want : (int64_t)sm_count() * 16);
  shoot_kernel<<<blocks, kShootThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      A, count, const_cast<double*>(out->x), const_cast<double*>(out->y), const_cast<double*>(out->z),
      const_cast<double*>(out->t), const_cast<double*>(out->dx), const_cast<double*>(out->dy),
      const_cast<double*>(out->dz), const_cast<double*>(out->lambda));
  return cudaGetLastError() == cudaSuccess ? RBG_OK : RBG_ERR_CUDA;
}
