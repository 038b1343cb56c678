// ray_order.cu -- the order in which the mixed tracer takes up the rays of a
// batch.
//
// Sources draw their rays at random over an aperture, so 32 consecutive
// rays of a batch start anywhere on it: one lane's ray hits the central
// hole, the next the secondary's shadow, the next a mirror edge, and the
// warp serialises their paths.  The persistent kernel therefore takes the
// rays up in the order of a counting sort by a cell key: the high bits a
// cell of the ray's direction, the low bits a cell of its start point,
// each numbered along a Morton curve whose bits go one at a time to the
// axis whose cells are then longest, over the bounding box of the batch's
// directions or start points (a batch that starts on a tilted plane spends
// few bits on its thin axis; rays of different field angles never share a
// cell).  Every ray keeps its own index for its inputs, its outputs and its
// random draws, so the results are those of input order; only which rays
// share a warp changes.
//
// Kernels: bounding boxes (ordered-integer atomics), cell keys and counts,
// a two-level exclusive scan of the counts, the scatter of the ray indices
// and a gather of the rays into that order, so the trace reads its inputs
// coalesced (its outputs go to each ray's own index).  Within a cell the
// order is whatever the atomics give.
#include <cuda_runtime.h>

#include <cstdint>

#include "robast_gb.h"
#include "tracer.cuh"

namespace rbg {
namespace {

// key bits: about 4 cells per ray, at most 2^24 cells; a quarter of the
// bits (at most 6) number the direction cell
constexpr int kMinKeyBits = 12, kMaxKeyBits = 24, kMaxDirBits = 6;
constexpr int kScanTile = 1024;
constexpr int kThreads = 256;

// doubles as unsigned integers in the same order (non-finite values are
// left out of the box by the caller)
__device__ __forceinline__ unsigned long long ordered_bits(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_ordered(unsigned long long k) {
  const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

// box[0..5] = min, box[6..11] = max (ordered bits) of x, y, z, dx, dy, dz;
// min words start at ~0, max words at 0
__global__ void __launch_bounds__(kThreads) bbox_kernel(KernelRays in, int64_t n, unsigned long long* box) {
  unsigned long long lo[6], hi[6];
  const double* v[6] = {in.x, in.y, in.z, in.dx, in.dy, in.dz};
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    lo[a] = ~0ull;
    hi[a] = 0ull;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      const double c = v[a][i];
      if (!isfinite(c)) continue;
      const unsigned long long k = ordered_bits(c);
      lo[a] = k < lo[a] ? k : lo[a];
      hi[a] = k > hi[a] ? k : hi[a];
    }
  }
#pragma unroll
  for (int a = 0; a < 6; ++a) {
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
      const unsigned long long l = __shfl_down_sync(0xffffffffu, lo[a], d);
      const unsigned long long h = __shfl_down_sync(0xffffffffu, hi[a], d);
      lo[a] = l < lo[a] ? l : lo[a];
      hi[a] = h > hi[a] ? h : hi[a];
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      atomicMin(&box[a], lo[a]);
      atomicMax(&box[6 + a], hi[a]);
    }
  }
}

// Morton cell of the point c[0..2] in `nbits` bits over the box lo + ext:
// each bit goes to the axis whose cells are then longest (ties to the
// lower axis); every thread derives the same assignment from the box
__device__ uint32_t morton_cell(const double* c, const double* lo, const double* ext, int nbits) {
  int bits[3] = {0, 0, 0};
  uint64_t seq = 0;  // 2 bits per key bit: its axis, most significant first
  double size[3] = {ext[0], ext[1], ext[2]};
  for (int b = 0; b < nbits; ++b) {
    const int a = size[0] >= size[1] ? (size[0] >= size[2] ? 0 : 2) : (size[1] >= size[2] ? 1 : 2);
    size[a] *= 0.5;
    ++bits[a];
    seq |= (uint64_t)a << (2 * b);
  }
  uint32_t q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double cells = (double)(1u << bits[a]);
    double f = ext[a] > 0 ? (c[a] - lo[a]) / ext[a] * cells : 0.0;
    if (!(f >= 0)) f = 0;  // below the box or NaN
    q[a] = f >= cells - 1 ? (1u << bits[a]) - 1u : (uint32_t)f;
  }
  uint32_t cell = 0;
  int used[3] = {0, 0, 0};
  for (int b = 0; b < nbits; ++b) {
    const int a = (int)((seq >> (2 * b)) & 3u);
    const int k = bits[a] - 1 - used[a]++;
    cell = (cell << 1) | ((q[a] >> k) & 1u);
  }
  return cell;
}

__global__ void __launch_bounds__(kThreads) key_kernel(KernelRays in, int64_t n, int dir_bits, int pos_bits,
                                                       const unsigned long long* box, uint32_t* keys,
                                                       uint32_t* counts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double lo[6], ext[6];
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    const bool ok = box[a] <= box[6 + a];
    lo[a] = ok ? from_ordered(box[a]) : 0.0;
    ext[a] = ok ? from_ordered(box[6 + a]) - lo[a] : 0.0;
  }
  const double p[3] = {in.x[i], in.y[i], in.z[i]}, d[3] = {in.dx[i], in.dy[i], in.dz[i]};
  const uint32_t key = (morton_cell(d, lo + 3, ext + 3, dir_bits) << pos_bits) | morton_cell(p, lo, ext, pos_bits);
  keys[i] = key;
  atomicAdd(&counts[key], 1u);
}

// exclusive scan inside tiles of kScanTile counts, tile totals to tile_sum
__global__ void __launch_bounds__(kScanTile) tile_scan_counts(uint32_t* counts, int64_t m, uint32_t* tile_sum) {
  __shared__ uint32_t s[kScanTile];
  const int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
  const uint32_t c = i < m ? counts[i] : 0u;
  s[threadIdx.x] = c;
  __syncthreads();
  for (int d = 1; d < kScanTile; d <<= 1) {
    const uint32_t v = threadIdx.x >= d ? s[threadIdx.x - d] : 0u;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  if (i < m) counts[i] = s[threadIdx.x] - c;
  if (threadIdx.x == kScanTile - 1) tile_sum[blockIdx.x] = s[kScanTile - 1];
}

// exclusive scan of the tile totals in one block
__global__ void __launch_bounds__(kScanTile) scan_tile_sums(uint32_t* tile_sum, int64_t ntiles) {
  __shared__ uint32_t s[kScanTile];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < ntiles; base += kScanTile) {
    const int64_t i = base + threadIdx.x;
    const uint32_t c = i < ntiles ? tile_sum[i] : 0u;
    s[threadIdx.x] = c;
    __syncthreads();
    for (int d = 1; d < kScanTile; d <<= 1) {
      const uint32_t v = threadIdx.x >= d ? s[threadIdx.x - d] : 0u;
      __syncthreads();
      s[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < ntiles) tile_sum[i] = carry + s[threadIdx.x] - c;
    __syncthreads();
    if (threadIdx.x == kScanTile - 1) carry += s[kScanTile - 1];
    __syncthreads();
  }
}

// the rays in queue order: slot q <- ray order[q] (coalesced stores; the
// trace then reads its inputs coalesced)
struct Dst {
  double* a[8];
};

__global__ void __launch_bounds__(kThreads) gather_kernel(KernelRays in, int64_t n, const int32_t* order, Dst dst) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int64_t i = order[q];
  if ((uint64_t)i >= (uint64_t)n) return;
  const double* src[8] = {in.x, in.y, in.z, in.t, in.dx, in.dy, in.dz, in.lambda};
#pragma unroll
  for (int a = 0; a < 8; ++a)
    if (src[a]) dst.a[a][q] = src[a][i];
}

__global__ void __launch_bounds__(kThreads) scatter_kernel(const uint32_t* keys, int64_t n, uint32_t* cursor,
                                                           const uint32_t* tile_sum, int32_t* order) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t key = keys[i];
  const uint32_t pos = tile_sum[key / kScanTile] + atomicAdd(&cursor[key], 1u);
  if (pos < (uint64_t)n) order[pos] = (int32_t)i;
}

struct Layout {
  int dir_bits, pos_bits;
  int64_t buckets, tiles;
  size_t box, keys, counts, tile_sum, order, sorted, total;
};

Layout layout(int64_t n) {
  Layout L;
  int kb = kMinKeyBits;
  while (kb < kMaxKeyBits && (int64_t(1) << kb) < 4 * n) ++kb;
  L.dir_bits = kb / 4 < kMaxDirBits ? kb / 4 : kMaxDirBits;
  L.pos_bits = kb - L.dir_bits;
  L.buckets = int64_t(1) << kb;
  L.tiles = (L.buckets + kScanTile - 1) / kScanTile;
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  L.box = 0;
  L.keys = L.box + 256;
  L.counts = L.keys + up((size_t)n * 4);
  L.tile_sum = L.counts + up((size_t)L.buckets * 4);
  L.order = L.tile_sum + up((size_t)L.tiles * 4);
  L.sorted = L.order + up((size_t)n * 4);  // 8 arrays of n doubles
  L.total = L.sorted + 8 * up((size_t)n * 8);
  return L;
}

}  // namespace

size_t ray_order_bytes(int64_t n) { return n > 0 && n <= 0x7fffffff ? layout(n).total : 0; }

// Write the take-up order of rays 0..n-1 and the rays in that order into
// `ws` (ray_order_bytes(n) bytes) on stream st; *sorted describes them
// (gathered, with the order).  n must fit in an int32.
int build_ray_order(const KernelRays& in, int64_t n, void* ws, KernelRays* sorted, cudaStream_t st) {
  if (n <= 0 || n > 0x7fffffff || !ws || !sorted) return RBG_ERR_ARG;
  const Layout L = layout(n);
  char* base = static_cast<char*>(ws);
  auto* box = reinterpret_cast<unsigned long long*>(base + L.box);
  auto* keys = reinterpret_cast<uint32_t*>(base + L.keys);
  auto* counts = reinterpret_cast<uint32_t*>(base + L.counts);
  auto* tile_sum = reinterpret_cast<uint32_t*>(base + L.tile_sum);
  auto* out = reinterpret_cast<int32_t*>(base + L.order);
  const size_t arr = (L.total - L.sorted) / 8;
  Dst dst;
  for (int a = 0; a < 8; ++a) dst.a[a] = reinterpret_cast<double*>(base + L.sorted + a * arr);
  if (cudaMemsetAsync(box, 0xff, 6 * sizeof(unsigned long long), st) != cudaSuccess ||
      cudaMemsetAsync(box + 6, 0, 6 * sizeof(unsigned long long), st) != cudaSuccess ||
      cudaMemsetAsync(counts, 0, (size_t)L.buckets * 4, st) != cudaSuccess)
    return RBG_ERR_CUDA;
  const int64_t blocks = (n + kThreads - 1) / kThreads;
  const int box_blocks = (int)(blocks < 4096 ? blocks : 4096);
  bbox_kernel<<<box_blocks, kThreads, 0, st>>>(in, n, box);
  key_kernel<<<(unsigned)blocks, kThreads, 0, st>>>(in, n, L.dir_bits, L.pos_bits, box, keys, counts);
  tile_scan_counts<<<(unsigned)L.tiles, kScanTile, 0, st>>>(counts, L.buckets, tile_sum);
  scan_tile_sums<<<1, kScanTile, 0, st>>>(tile_sum, L.tiles);
  scatter_kernel<<<(unsigned)blocks, kThreads, 0, st>>>(keys, n, counts, tile_sum, out);
  gather_kernel<<<(unsigned)blocks, kThreads, 0, st>>>(in, n, out, dst);
  if (cudaGetLastError() != cudaSuccess) return RBG_ERR_CUDA;
  *sorted = KernelRays{dst.a[0], dst.a[1], dst.a[2], in.t ? dst.a[3] : nullptr, dst.a[4], dst.a[5], dst.a[6],
                       dst.a[7], out, 1};
  return RBG_OK;
}

}  // namespace rbg
