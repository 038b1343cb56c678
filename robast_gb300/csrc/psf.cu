// psf.cu -- focal-plane reductions on the device: focused-ray moments per
// group, the 2D histogram of focused rays, and AGeoUtil::ContainmentRadius
// (src/AGeoUtil.cxx:198-308) with its SumInRadius probes (:18-42).
//
// ContainmentRadius is a sequential search (a secant step on the radius,
// then hill-climbing shifts of the centre in x and in y, repeated until
// four rounds change nothing), and every step needs SumInRadius over the
// whole histogram.  Here the search runs as ONE launch of one thread-block
// cluster (kCrCtas CTAs on as many SMs): every thread of every CTA runs the
// reference's control flow on the same scalars, and each SumInRadius is a
// cluster-wide pass over the histogram -- each CTA sums its share of the
// bins, the partial sums meet through distributed shared memory, and every
// CTA adds the kCrCtas partials in rank order, so all CTAs hold bitwise the
// same totals and take the same branches.  The probes the reference makes
// back to back on the same centre (sum0 with the r +- dr probes, sum1 with
// the first x pair, sum1 with the y pair) share one pass.  A pass reads
// only the bins within the probes' bounding boxes and decides each bin with
// an FP32 distance, falling back to the reference's FP64 expression
// (rounded operation by operation, no contraction) when the FP32 value lies
// within its error bound of r^2; the sums are therefore those of the
// reference's loop, exact for integer counts.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "robast_gb.h"
#include "device_state.cuh"

namespace cg = cooperative_groups;

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
  // a warp whose rays all belong to one group (batches are laid out group
  // by group) sums its values by shuffles and adds once; other warps add
  // per ray.  Rays that are not focused add zeros to their group.
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int g = -1;
    double v[6] = {0, 0, 0, 0, 0, 0};
    if (i < n) {
      g = group ? group[i] : 0;
      if (g < 0 || g >= n_groups) g = -1;
      if (g >= 0 && status[i] == RBG_FOCUS) {
        v[0] = 1.0;
        v[1] = x[i];
        v[2] = y[i];
        v[3] = x[i] * x[i];
        v[4] = y[i] * y[i];
        v[5] = t ? t[i] : 0.0;
      }
    }
    const unsigned peers = __match_any_sync(FULL, g);
    if (peers == FULL) {
      if (g >= 0) {
#pragma unroll
        for (int k = 0; k < 6; ++k)
          for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_xor_sync(FULL, v[k], off);
        double* dst = shared ? acc + g * 6 : sums + g * 6;
        if (lane == 0 && v[0] != 0)
          for (int k = 0; k < 6; ++k) atomicAdd(dst + k, v[k]);
      }
    } else if (g >= 0 && v[0] != 0) {
      double* dst = shared ? acc + g * 6 : sums + g * 6;
      for (int k = 0; k < 6; ++k) atomicAdd(dst + k, v[k]);
    }
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

// ---------------------------------------------------------------------
// ContainmentRadius: one cluster
// ---------------------------------------------------------------------
constexpr int kCrCtas = 8;  // the portable cluster size
constexpr int kCrThreads = 1024;
constexpr int kCrWarps = kCrThreads / 32;
constexpr int kCrMaxVals = 5;         // values one pass reduces (the moments)
constexpr int kCrMaxPasses = 200000;  // the reference's loops end far sooner

struct CrHist {
  const double* c;  // counts[ix * ny + iy]
  int nx, ny;
  double xlo, xw, ylo, yw;
};

struct CrShared {
  double warp_part[kCrWarps][kCrMaxVals];
  double slot[2][kCrMaxVals];  // this CTA's partials, alternating passes
  double tot[kCrMaxVals];      // the cluster's totals
};

struct CrState {
  int parity;
  int passes;
  bool bail;
};

// Sum `nv` per-thread values over the cluster; every thread gets the same
// totals (the partials of the CTAs added in rank order).
__device__ void cr_reduce(double* v, int nv, CrShared& sh, cg::cluster_group& cl, CrState& s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < nv; ++k) {
    double a = v[k];
    for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
    if (lane == 0) sh.warp_part[warp][k] = a;
  }
  __syncthreads();
  if ((int)threadIdx.x < nv) {
    double a = 0;
    for (int w = 0; w < kCrWarps; ++w) a += sh.warp_part[w][threadIdx.x];
    sh.slot[s.parity][threadIdx.x] = a;
  }
  // a CTA writes slot[parity] again two passes later, after every CTA has
  // passed the next cluster barrier and so finished reading it
  cl.sync();
  if ((int)threadIdx.x < nv) {
    double a = 0;
    for (int q = 0; q < kCrCtas; ++q) a += *cl.map_shared_rank(&sh.slot[s.parity][threadIdx.x], q);
    sh.tot[threadIdx.x] = a;
  }
  __syncthreads();
  for (int k = 0; k < nv; ++k) v[k] = sh.tot[k];
  s.parity ^= 1;
}

// bins [a, b] along one axis whose centres lie within |r| of c
__device__ void cr_range(double c, double r, double lo, double w, int n, int& a, int& b) {
  const double ar = fabs(r);
  const double fa = (c - ar - lo) / w - 0.5, fb = (c + ar - lo) / w - 0.5;
  if (!(fa > -1e9 && fb < 1e9)) {  // also NaN
    a = 0;
    b = n - 1;
    return;
  }
  a = max(0, (int)floor(fa) - 1);
  b = min(n - 1, (int)ceil(fb) + 1);
}

// SumInRadius's test for bin (ix, iy) as the reference evaluates it
__device__ __forceinline__ bool cr_exact_in(const CrHist& h, int ix, int iy, double x, double y, double r2) {
  const double cx = __dadd_rn(h.xlo, __dmul_rn((double)ix + 0.5, h.xw));
  const double cy = __dadd_rn(h.ylo, __dmul_rn((double)iy + 0.5, h.yw));
  const double dx = __dsub_rn(cx, x), dy = __dsub_rn(cy, y);
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) <= r2;
}

// SumInRadius(h, x[p], y[p], r[p]) for np <= 3 probes in one pass.
__device__ void cr_probe(const CrHist& h, int np, const double* px, const double* py, const double* pr,
                         double* out, CrShared& sh, cg::cluster_group& cl, CrState& s) {
  if (s.bail || ++s.passes > kCrMaxPasses) {
    // identical in every CTA: the search ends without further barriers
    s.bail = true;
    for (int p = 0; p < np; ++p) out[p] = -INFINITY;
    return;
  }
  int ix0 = h.nx, ix1 = -1, iy0 = h.ny, iy1 = -1;
  double r2[3];
  float r2f[3], b0f[3], eyf[3], gf[3];
  const float ywf = (float)h.yw;
  for (int p = 0; p < np; ++p) {
    int a, b;
    cr_range(px[p], pr[p], h.xlo, h.xw, h.nx, a, b);
    ix0 = min(ix0, a);
    ix1 = max(ix1, b);
    cr_range(py[p], pr[p], h.ylo, h.yw, h.ny, a, b);
    iy0 = min(iy0, a);
    iy1 = max(iy1, b);
    r2[p] = __dmul_rn(pr[p], pr[p]);
    r2f[p] = (float)r2[p];
    // FP32 row offset dy = b0 + iy * yw: its error bound, and a guard for
    // the FP64 rounding of the reference's own expression
    const double b0 = h.ylo + 0.5 * h.yw - py[p];
    b0f[p] = (float)b0;
    eyf[p] = (float)(1.2e-7 * (fabs(b0) + h.ny * h.yw));
    const double span = fabs(h.xlo) + h.nx * h.xw + fabs(px[p]) + fabs(h.ylo) + h.ny * h.yw + fabs(py[p]);
    gf[p] = (float)(1e-13 * span * (fabs(pr[p]) + h.xw + h.yw + 1.0));
  }
  double part[3] = {0, 0, 0};
  const int lane = threadIdx.x & 31;
  const int gwarp = (int)cl.block_rank() * kCrWarps + (threadIdx.x >> 5);
  for (int ix = ix0 + gwarp; ix <= ix1; ix += kCrCtas * kCrWarps) {
    const double cx = h.xlo + (ix + 0.5) * h.xw;
    float dx2f[3];
    for (int p = 0; p < np; ++p) {
      const double d = cx - px[p];
      dx2f[p] = (float)(d * d);
    }
    const double* row = h.c + (int64_t)ix * h.ny;
    for (int iy = iy0 + lane; iy <= iy1; iy += 32) {
      const double c = __ldg(row + iy);
      if (c <= 0) continue;
      for (int p = 0; p < np; ++p) {
        const float dyf = fmaf((float)iy, ywf, b0f[p]);
        const float d2f = dx2f[p] + dyf * dyf;
        const float m = 4.8e-7f * (d2f + r2f[p]) + 2.5f * (fabsf(dyf) + eyf[p]) * eyf[p] + gf[p];
        bool in;
        if (d2f < r2f[p] - m) in = true;
        else if (d2f > r2f[p] + m) in = false;
        else in = cr_exact_in(h, ix, iy, px[p], py[p], r2[p]);
        if (in) part[p] += c;
      }
    }
  }
  cr_reduce(part, np, sh, cl, s);
  for (int p = 0; p < np; ++p) out[p] = part[p];
}

// out: r, x, y, status (0 ok, -1 pass cap reached)
__global__ void __cluster_dims__(kCrCtas, 1, 1) __launch_bounds__(kCrThreads, 1)
    containment_radius_kernel(CrHist h, double fraction, double* out) {
  __shared__ CrShared sh;
  cg::cluster_group cl = cg::this_cluster();
  CrState s{0, 0, false};
  // moments from the bin centres (the oracle's initial guess)
  double mom[kCrMaxVals] = {0, 0, 0, 0, 0};
  const int64_t nb = (int64_t)h.nx * h.ny;
  const int64_t gtid = (int64_t)cl.block_rank() * kCrThreads + threadIdx.x;
  for (int64_t b = gtid; b < nb; b += (int64_t)kCrCtas * kCrThreads) {
    const int ix = (int)(b / h.ny), iy = (int)(b - (int64_t)ix * h.ny);
    const double cx = h.xlo + (ix + 0.5) * h.xw, cy = h.ylo + (iy + 0.5) * h.yw;
    const double c = h.c[b];
    mom[0] += c;
    mom[1] += c * cx;
    mom[2] += c * cy;
    mom[3] += c * cx * cx;
    mom[4] += c * cy * cy;
  }
  cr_reduce(mom, 5, sh, cl, s);
  const double sw = mom[0];
  double x = sw ? mom[1] / sw : 0, y = sw ? mom[2] / sw : 0;
  const double vx = sw ? mom[3] / sw - x * x : 0, vy = sw ? mom[4] / sw - y * y : 0;
  const double sdx = vx > 0 ? sqrt(vx) : 0, sdy = vy > 0 ? sqrt(vy) : 0;
  double r = sqrt(sdx * sdx + sdy * sdy) * 1.5;
  double dr = 0.1 * r;
  const double sum_goal = sw * fraction;
  int no_shift = 0, no_stable = 0;
  double qx[3], qy[3], qr[3], o[3];
  for (int i = 0; i < 100 && no_shift < 30; i++) {
    bool stable_r = false, stable_x = true, stable_y = true;
    // sum0 at r, with the r + dr and r - dr probes of either branch
    qx[0] = qx[1] = qx[2] = x;
    qy[0] = qy[1] = qy[2] = y;
    qr[0] = r;
    qr[1] = r + dr;
    qr[2] = r - dr;
    cr_probe(h, 3, qx, qy, qr, o, sh, cl, s);
    const double sum0 = o[0];
    double next_r = r;
    if (sum0 < sum_goal) {
      const double sum1 = o[1];
      if (sum1 == sum0) {
        dr *= 2.;
        continue;
      }
      next_r = r + dr * (sum_goal - sum0) / (sum1 - sum0);
    } else if (sum0 != sum_goal) {
      const double sum1 = o[2];
      if (sum1 == sum0) {
        dr *= 2.;
        continue;
      }
      next_r = r - dr * (sum0 - sum_goal) / (sum0 - sum1);
    }
    if (next_r < 0.) next_r = 0.5 * r;
    if (next_r < 0.5 * r) next_r = 0.5 * r;
    if (next_r > 2. * r) next_r = 2. * r;
    stable_r = fabs(next_r - r) < 0.0001 * r;
    r = next_r;
    {
      // sum1 at the new radius, with the first x pair
      double dx = 0.25 * r;
      qx[0] = x;
      qx[1] = x + dx;
      qx[2] = x - dx;
      qy[0] = qy[1] = qy[2] = y;
      qr[0] = qr[1] = qr[2] = r;
      cr_probe(h, 3, qx, qy, qr, o, sh, cl, s);
      double sum1 = o[0];
      dr *= sum0 != sum_goal ? fabs((sum1 - sum_goal) / (sum0 - sum_goal)) : 0.5;
      if (dr > 0.5 * r) dr = 0.5 * r;
      if (dr < 0.0005 * r) dr = 0.0005 * r;
      no_shift++;
      bool first = true;
      for (; dx > 0.1 * dr; dx *= 0.25) {
        double sx1, sx2;
        if (first) {
          sx1 = o[1];
          sx2 = o[2];
          first = false;
        } else {
          qx[0] = x + dx;
          qx[1] = x - dx;
          cr_probe(h, 2, qx, qy, qr, o, sh, cl, s);
          sx1 = o[0];
          sx2 = o[1];
        }
        while (sx1 > sum1) {
          no_shift = 0;
          x += dx;
          sx2 = sum1;
          sum1 = sx1;
          qx[0] = x + dx;
          cr_probe(h, 1, qx, qy, qr, o, sh, cl, s);
          sx1 = o[0];
          stable_x = false;
        }
        while (sx2 > sum1) {
          no_shift = 0;
          x -= dx;
          sx1 = sum1;
          sum1 = sx2;
          qx[0] = x - dx;
          cr_probe(h, 1, qx, qy, qr, o, sh, cl, s);
          sx2 = o[0];
          stable_x = false;
        }
      }
    }
    for (double dy = 0.1 * r; dy > 0.1 * dr; dy *= 0.25) {
      qx[0] = qx[1] = qx[2] = x;
      qy[0] = y;
      qy[1] = y + dy;
      qy[2] = y - dy;
      qr[0] = qr[1] = qr[2] = r;
      cr_probe(h, 3, qx, qy, qr, o, sh, cl, s);
      double sum1 = o[0], sy1 = o[1], sy2 = o[2];
      while (sy1 > sum1) {
        no_shift = 0;
        y += dy;
        sy2 = sum1;
        sum1 = sy1;
        qy[0] = y + dy;
        cr_probe(h, 1, qx, qy, qr, o, sh, cl, s);
        sy1 = o[0];
        stable_y = false;
      }
      while (sy2 > sum1) {
        no_shift = 0;
        y -= dy;
        sy1 = sum1;
        sum1 = sy2;
        qy[0] = y - dy;
        cr_probe(h, 1, qx, qy, qr, o, sh, cl, s);
        sy2 = o[0];
        stable_y = false;
      }
    }
    if (stable_r && stable_x && stable_y) no_stable++;
    else no_stable = 0;
    if (no_stable >= 4) break;
  }
  if (cl.block_rank() == 0 && threadIdx.x == 0) {
    out[0] = r;
    out[1] = x;
    out[2] = y;
    out[3] = s.bail ? -1.0 : 0.0;
  }
  // no CTA leaves while another may still read its shared memory
  cl.sync();
}

namespace {
// the host-output entry point's result slot (4 doubles per call; calls
// are serialised by g_cr_mutex)
__device__ double g_cr_out[4];
std::mutex g_cr_mutex;
constexpr int kMaxDev = 64;
int g_cr_ok[kMaxDev] = {0};  // 1: a cluster fits on the device, -1: it does not

int cr_check_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return RBG_ERR_CUDA;
  if (dev >= kMaxDev) return RBG_ERR_UNSUPPORTED;
  if (g_cr_ok[dev] == 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kCrCtas, 1, 1);
    cfg.blockDim = dim3(kCrThreads, 1, 1);
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, containment_radius_kernel, &cfg) != cudaSuccess)
      return RBG_ERR_CUDA;
    g_cr_ok[dev] = clusters >= 1 ? 1 : -1;
  }
  return g_cr_ok[dev] == 1 ? RBG_OK : RBG_ERR_UNSUPPORTED;
}
}  // namespace

}  // namespace rbg

using namespace rbg;

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

// AGeoUtil::ContainmentRadius into DEVICE memory out[0..3] = r, x, y,
// status; stream-ordered, one launch, nothing allocated
extern "C" int rbg_containment_radius_async(const double* counts, int32_t nx, double xlo, double xhi, int32_t ny,
                                            double ylo, double yhi, double fraction, double* out, void* stream) {
  if (!counts || !out || nx <= 0 || ny <= 0 || !(xhi > xlo) || !(yhi > ylo)) return RBG_ERR_ARG;
  int rc = cr_check_device();
  if (rc) return rc;
  // bin widths as the reference's TAxis computes them
  CrHist h{counts, nx, ny, xlo, (xhi - xlo) / nx, ylo, (yhi - ylo) / ny};
  containment_radius_kernel<<<kCrCtas, kCrThreads, 0, static_cast<cudaStream_t>(stream)>>>(h, fraction, out);
  return cudaGetLastError() == cudaSuccess ? RBG_OK : RBG_ERR_CUDA;
}

// The same with host outputs: one launch and one 32-byte copy back
extern "C" int rbg_containment_radius(const double* counts, int32_t nx, double xlo, double xhi, int32_t ny,
                                      double ylo, double yhi, double fraction, double* pr, double* px, double* py,
                                      void* stream) {
  if (!counts || nx <= 0 || ny <= 0 || !pr || !px || !py || !(xhi > xlo) || !(yhi > ylo)) return RBG_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lock(g_cr_mutex);
  double* slot = nullptr;
  if (cudaGetSymbolAddress(reinterpret_cast<void**>(&slot), g_cr_out) != cudaSuccess || !slot) return RBG_ERR_CUDA;
  int rc = rbg_containment_radius_async(counts, nx, xlo, xhi, ny, ylo, yhi, fraction, slot, stream);
  if (rc) return rc;
  double res[4];
  if (cudaMemcpyAsync(res, slot, sizeof(res), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return RBG_ERR_CUDA;
  if (res[3] != 0.0) return RBG_ERR_CAP;
  *pr = res[0];
  *px = res[1];
  *py = res[2];
  return RBG_OK;
}
