// corsika_rays.cu -- ACorsikaIACTFile::GetRayArray on the GPU
// (src/ACorsikaIACTFile.cxx:71-133): photon bunches become rays.
//
// A bunch of p photons (fractional) yields ceil(p) rays, as the
// reference's `for (j = 0; j < photons; j++)`.  Three kernels:
//   1. per tile of kTile bunches: photon counts, their exclusive scan
//      inside the tile (shared memory) and the tile total;
//   2. one block: exclusive scan of the tile totals, and the grand total;
//   3. one warp per 32 consecutive bunches: each lane back-projects its
//      bunch once (the reference's per-bunch quantities, :112-117), a warp
//      scan of the ray counts places the warp's rays, and the lanes then
//      write those rays 32 at a time, each taking its bunch's values from
//      the owning lane by shuffle (a 5-step search over the warp scan), so
//      every store of a field is 32 consecutive doubles.
// All scratch lives in the caller's workspace.
#include <cuda_runtime.h>

#include <cmath>

#include "philox.h"
#include "robast_gb.h"

namespace rbg {
namespace {

constexpr int kTile = 1024;  // bunches per block of kernel 1
constexpr double kSpeedOfLightCm = 2.99792458e10;
constexpr double kNs = 1e-9;  // s
constexpr double kNm = 1e-7;  // cm

constexpr float kMaxBunchRays = 4294967296.f;  // 2^32

__device__ __forceinline__ int64_t bunch_rays(float photons) {
  // j < photons for j = 0, 1, ...: ceil(photons) iterations; none for
  // photons <= 0 or NaN.  Counts are capped at 2^32 (with at most 2^31
  // bunches the sum stays below 2^63; such a total then exceeds any
  // capacity and the call fails instead of writing)
  if (!(photons > 0.f)) return 0;
  return photons >= kMaxBunchRays ? (int64_t)kMaxBunchRays : (int64_t)ceilf(photons);
}

__global__ void __launch_bounds__(kTile) count_scan_kernel(const float* photons, int64_t n, int64_t* offsets,
                                                           int64_t* tile_sum) {
  __shared__ int64_t s[kTile];
  const int64_t i = (int64_t)blockIdx.x * kTile + threadIdx.x;
  const int64_t c = i < n ? bunch_rays(photons[i]) : 0;
  s[threadIdx.x] = c;
  __syncthreads();
  // Hillis-Steele inclusive scan over the tile
  for (int d = 1; d < kTile; d <<= 1) {
    const int64_t v = threadIdx.x >= d ? s[threadIdx.x - d] : 0;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  if (i < n) offsets[i] = s[threadIdx.x] - c;  // exclusive within the tile
  if (threadIdx.x == kTile - 1) tile_sum[blockIdx.x] = s[kTile - 1];
}

// exclusive scan of the tile totals in one block; total at tile_sum[ntiles]
__global__ void __launch_bounds__(kTile) tile_scan_kernel(int64_t* tile_sum, int64_t ntiles) {
  __shared__ int64_t s[kTile];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < ntiles; base += kTile) {
    const int64_t i = base + threadIdx.x;
    const int64_t c = i < ntiles ? tile_sum[i] : 0;
    s[threadIdx.x] = c;
    __syncthreads();
    for (int d = 1; d < kTile; d <<= 1) {
      const int64_t v = threadIdx.x >= d ? s[threadIdx.x - d] : 0;
      __syncthreads();
      s[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < ntiles) tile_sum[i] = carry + s[threadIdx.x] - c;
    __syncthreads();
    if (threadIdx.x == kTile - 1) carry += s[kTile - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_sum[ntiles] = carry;
}

constexpr int kExpandThreads = 256;

__global__ void __launch_bounds__(kExpandThreads)
    expand_kernel(rbg_bunches b, const int64_t* offsets, const int64_t* tile_off, double z, double tel_z,
                  double speed, double inv_lmin, double inv_lmax, uint64_t seed, double* x, double* y, double* zz,
                  double* t, double* dx, double* dy, double* dz, double* lam) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t first = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) << 5;
  if (first >= b.n) return;  // warp-uniform
  const int64_t i = first + lane;
  const bool valid = i < b.n;
  const int64_t c = valid ? bunch_rays(b.photons[i]) : 0;
  // inclusive scan of the warp's ray counts
  int64_t incl = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int64_t v = __shfl_up_sync(full, incl, d);
    if (lane >= d) incl += v;
  }
  const int64_t wtotal = __shfl_sync(full, incl, 31);
  // global offset of the warp's first ray (kTile is a multiple of 32, so
  // the warp's bunches share one tile)
  const int64_t base = tile_off[first / kTile] + offsets[first];
  // this lane's bunch, back-projected to height z (:112-117)
  double px = 0, py = 0, pt = 0, cx = 0, cy = 0, cz = 0, l = 0;
  if (c > 0) {
    cx = b.cx[i];
    cy = b.cy[i];
    cz = b.cz[i];
    const double airmass = -1. / cz;
    const double tel_dist = (z - tel_z) * airmass;
    px = (double)b.x[i] - tel_dist * cx;
    py = (double)b.y[i] - tel_dist * cy;
    pt = (double)b.time[i] * kNs - tel_dist / speed;
    l = b.lambda[i];
  }
  for (int64_t r0 = 0; r0 < wtotal; r0 += 32) {
    const int64_t rl = r0 + lane;
    // owning lane: the number of lanes whose inclusive count is <= rl
    int s = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const int64_t v = __shfl_sync(full, incl, s + step - 1);
      if (v <= rl) s += step;
    }
    const double vx = __shfl_sync(full, px, s), vy = __shfl_sync(full, py, s), vt = __shfl_sync(full, pt, s);
    const double vcx = __shfl_sync(full, cx, s), vcy = __shfl_sync(full, cy, s), vcz = __shfl_sync(full, cz, s);
    double vl = __shfl_sync(full, l, s);
    if (rl < wtotal) {
      const int64_t r = base + rl;
      if (vl == 0) {
        RayRng g;
        g.init(seed, (uint64_t)r, 2u);
        vl = 1. / (inv_lmin - g.uniform() * (inv_lmin - inv_lmax));
      }
      x[r] = vx;
      y[r] = vy;
      zz[r] = z;
      t[r] = vt;
      dx[r] = vcx;
      dy[r] = vcy;
      dz[r] = vcz;
      lam[r] = vl * kNm;
    }
  }
}

}  // namespace
}  // namespace rbg

using namespace rbg;

extern "C" size_t rbg_bunches_workspace_bytes(int64_t n_bunches) {
  if (n_bunches < 0) return 0;
  const int64_t ntiles = (n_bunches + kTile - 1) / kTile;
  return (size_t)(n_bunches + ntiles + 1) * sizeof(int64_t) + 256;
}

extern "C" int rbg_bunches_to_rays(const rbg_bunches* b, double z, double tel_z, double refractive_index,
                                   double lambda_min, double lambda_max, uint64_t seed, void* workspace,
                                   rbg_rays* out, int64_t capacity, int64_t* n_rays, void* stream) {
  if (!b || !n_rays || b->n < 0 || !(refractive_index > 0)) return RBG_ERR_ARG;
  *n_rays = 0;
  if (b->n == 0) {
    if (out) out->n = 0;
    return RBG_OK;
  }
  if (!workspace || !b->photons || !b->x || !b->y || !b->time || !b->cx || !b->cy || !b->cz || !b->lambda)
    return RBG_ERR_ARG;
  if (!(lambda_min > 0) || !(lambda_max > 0)) return RBG_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t n = b->n;
  if (n > 0x7fffffff) return RBG_ERR_TOO_LARGE;
  const int64_t ntiles = (n + kTile - 1) / kTile;
  int64_t* offsets = static_cast<int64_t*>(workspace);
  int64_t* tile_sum = offsets + n;
  count_scan_kernel<<<(unsigned)ntiles, kTile, 0, st>>>(b->photons, n, offsets, tile_sum);
  tile_scan_kernel<<<1, kTile, 0, st>>>(tile_sum, ntiles);
  if (cudaGetLastError() != cudaSuccess) return RBG_ERR_CUDA;
  int64_t total = 0;
  if (cudaMemcpyAsync(&total, tile_sum + ntiles, sizeof(total), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return RBG_ERR_CUDA;
  *n_rays = total;
  if (!out) return RBG_OK;
  if (total > capacity) return RBG_ERR_TOO_LARGE;
  if (total > 0) {
    if (!out->x || !out->y || !out->z || !out->t || !out->dx || !out->dy || !out->dz || !out->lambda)
      return RBG_ERR_ARG;
    // one warp per 32 bunches
    const int64_t blocks = (n + kExpandThreads - 1) / kExpandThreads;
    if (blocks > 0x7fffffff) return RBG_ERR_TOO_LARGE;
    expand_kernel<<<(unsigned)blocks, kExpandThreads, 0, st>>>(
        *b, offsets, tile_sum, z, tel_z, kSpeedOfLightCm / refractive_index, 1. / lambda_min,
        1. / lambda_max, seed, const_cast<double*>(out->x), const_cast<double*>(out->y), const_cast<double*>(out->z),
        const_cast<double*>(out->t), const_cast<double*>(out->dx), const_cast<double*>(out->dy),
        const_cast<double*>(out->dz), const_cast<double*>(out->lambda));
    if (cudaGetLastError() != cudaSuccess) return RBG_ERR_CUDA;
  }
  out->n = total;
  if (cudaStreamSynchronize(st) != cudaSuccess) return RBG_ERR_CUDA;
  return RBG_OK;
}
