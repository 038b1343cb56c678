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
// Kernels: bounding boxes (ordered-integer atomics), the key plan (one
// thread), cell keys and counts,
// a two-level exclusive scan of the counts, the scatter of the ray indices
// and a gather of the rays into that order, so the trace reads its inputs
// coalesced (its outputs go to each ray's own index).  Within a cell the
// order is whatever the atomics give.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "robast_gb.h"
#include "tracer.cuh"

namespace rbg {
namespace {

// key bits: about 4 cells per ray up to 2^24 cells, then about one cell
// per ray up to 2^26; a quarter of the bits (at most 6) number the
// direction cell
constexpr int kMinKeyBits = 12, kMaxKeyBits = 26, kMaxDirBits = 6;
// Index chunks (off): with kChunkShift = s > 0 the rays [c 2^s, (c + 1) 2^s)
// are ordered among themselves and chunk c's rays are taken up before chunk
// c + 1's (the chunk is the key's top field), so the rays in flight write
// their results into one or two chunks' stretch of the output arrays and L2
// completes more of their 32-byte sectors before writing them back.  On
// 1e7 Schwarzschild-Couder rays, s = 20 cut the trace kernel's DRAM traffic
// from 600 to 390 B per ray but made it 5-7 % slower (sparser cells, less
// coherent warps); s = 21 was 0.3-2 % slower on the light guide, the
// Davies-Cotton dish and 4e7 Schmidt-Cassegrain rays.  Throughput is what
// the trace is bound by, so the batch is ordered as one chunk.  s is raised until there are at most
// kMaxChunks chunks.
constexpr int kChunkShift = 0, kMaxChunks = 32;
constexpr int64_t kMaxBuckets = int64_t(1) << 26;
constexpr int kScanTile = 1024;
constexpr int kThreads = 256;

// The high 32 bits of a double as an unsigned integer in the same order
// (non-decreasing with the value; sign, exponent and 20 mantissa bits).
// Non-finite values give 0 and are left out of the box.
__device__ __forceinline__ uint32_t ordered_hi(double v, bool& finite) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  finite = ((u >> 52) & 0x7ffull) != 0x7ffull;
  const uint32_t h = (uint32_t)(u >> 32);
  return (h >> 31) ? ~h : (h | 0x80000000u);
}
// a double not above (low = true) / not below every value whose ordered
// high word is k
__host__ __device__ inline double from_ordered_hi(uint32_t k, bool low) {
  const uint32_t h = (k >> 31) ? (k & 0x7fffffffu) : ~k;
  // the low word that moves the value down (low) or up: for a positive
  // value 0 is the smallest magnitude, for a negative one the largest
  const bool neg = (h >> 31) != 0;
  const unsigned long long lw = (low != neg) ? 0ull : 0xffffffffull;
  const unsigned long long u = ((unsigned long long)h << 32) | lw;
  double d;
  memcpy(&d, &u, sizeof(d));
  return d;
}

// box[0..5] = min, box[6..11] = max ordered high words of x, y, z, dx, dy,
// dz; min words start at ~0, max words at 0
__global__ void __launch_bounds__(kThreads) bbox_kernel(KernelRays in, int64_t n, uint32_t* box) {
  uint32_t lo[6], hi[6];
  const double* v[6] = {in.x, in.y, in.z, in.dx, in.dy, in.dz};
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    lo[a] = ~0u;
    hi[a] = 0u;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      bool fin;
      const uint32_t k = ordered_hi(v[a][i], fin);
      if (!fin) continue;
      lo[a] = k < lo[a] ? k : lo[a];
      hi[a] = k > hi[a] ? k : hi[a];
    }
  }
  // warp, then block, then one atomic per word and block
  constexpr int kWarps = kThreads / 32;
  __shared__ uint32_t part[12][kWarps];
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    lo[a] = __reduce_min_sync(0xffffffffu, lo[a]);
    hi[a] = __reduce_max_sync(0xffffffffu, hi[a]);
    if ((threadIdx.x & 31) == 0) {
      part[a][warp] = lo[a];
      part[6 + a][warp] = hi[a];
    }
  }
  __syncthreads();
  if (threadIdx.x < 12) {
    const int w = threadIdx.x;
    uint32_t r = part[w][0];
    for (int k = 1; k < kWarps; ++k) r = w < 6 ? (part[w][k] < r ? part[w][k] : r) : (part[w][k] > r ? part[w][k] : r);
    if (w < 6) atomicMin(&box[w], r);
    else atomicMax(&box[w], r);
  }
}

// How a ray's cell key is formed, worked out once from the box: per axis
// (x, y, z, dx, dy, dz) the low edge and the cells per unit in FP32, the
// largest cell index, and the key bit each of its index bits lands on.
struct Plan {
  float lo[6], scale[6];
  uint32_t qmax[6];
  int32_t bits[6];
  int8_t pos[6][kMaxKeyBits];
  int32_t chunk_shift, cell_bits;  // key = (i >> chunk_shift) << cell_bits | cell
};

// Key bits go one at a time, most significant first, to the axis whose
// cells are then longest (ties to the lower axis): dir_bits among the
// direction axes, then pos_bits among the start-point axes.
__global__ void plan_kernel(const uint32_t* box, int dir_bits, int pos_bits, int chunk_shift, Plan* plan) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Plan P;
  P.chunk_shift = chunk_shift;
  P.cell_bits = dir_bits + pos_bits;
  double size[6];
  for (int a = 0; a < 6; ++a) {
    const bool ok = box[a] <= box[6 + a];
    const double lo = ok ? from_ordered_hi(box[a], true) : 0.0;
    const double hi = ok ? from_ordered_hi(box[6 + a], false) : 0.0;
    P.lo[a] = (float)lo;
    size[a] = hi > lo ? hi - lo : 0.0;
    P.bits[a] = 0;
  }
  const double ext[6] = {size[0], size[1], size[2], size[3], size[4], size[5]};
  // a batch of parallel rays (one direction) gives every key bit to the
  // start point
  if (!(size[3] > 0) && !(size[4] > 0) && !(size[5] > 0)) {
    pos_bits += dir_bits;
    dir_bits = 0;
  }
  int seq[kMaxKeyBits];
  const int total = dir_bits + pos_bits;
  for (int b = 0; b < total; ++b) {
    const int base = b < dir_bits ? 3 : 0;
    int a = base;
    for (int k = base + 1; k < base + 3; ++k)
      if (size[k] > size[a]) a = k;
    size[a] *= 0.5;
    ++P.bits[a];
    seq[b] = a;
  }
  int used[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < total; ++b) {
    const int a = seq[b];
    const int j = P.bits[a] - 1 - used[a]++;  // index bit j of axis a ...
    P.pos[a][j] = (int8_t)(total - 1 - b);     // ... lands on this key bit
  }
  for (int a = 0; a < 6; ++a) {
    P.qmax[a] = P.bits[a] ? (1u << P.bits[a]) - 1u : 0u;
    P.scale[a] = ext[a] > 0 ? (float)((double)(1u << P.bits[a]) / ext[a]) : 0.f;
  }
  *plan = P;
}

__global__ void __launch_bounds__(kThreads) key_kernel(KernelRays in, int64_t n, const Plan* plan, uint32_t* keys,
                                                       uint32_t* counts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* v[6] = {in.x, in.y, in.z, in.dx, in.dy, in.dz};
  uint32_t key = plan->chunk_shift > 0 ? (uint32_t)(i >> plan->chunk_shift) << plan->cell_bits : 0u;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    const float f = ((float)v[a][i] - plan->lo[a]) * plan->scale[a];
    const uint32_t qmax = plan->qmax[a];
    uint32_t q = 0u;  // below the box or NaN: 0
    if (f >= 1.f) q = f >= (float)qmax ? qmax : (uint32_t)f;
    for (int j = 0; j < plan->bits[a]; ++j) key |= ((q >> j) & 1u) << plan->pos[a][j];
  }
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
  int dir_bits, pos_bits, chunk_shift;
  int64_t buckets, tiles;
  size_t box, plan, keys, counts, tile_sum, order, sorted, total;
};

Layout layout(int64_t n) {
  Layout L;
  int cs = kChunkShift;
  if (cs > 0)
    while (((n - 1) >> cs) + 1 > kMaxChunks) ++cs;
  if (cs > 0 && (n - 1) >> cs == 0) cs = 0;  // one chunk
  const int64_t chunks = cs > 0 ? ((n - 1) >> cs) + 1 : 1;
  const int64_t per = cs > 0 ? (int64_t(1) << cs) : n;
  int kb = kMinKeyBits;
  const int64_t cells = std::min<int64_t>(4 * per, std::max<int64_t>(int64_t(1) << 24, per));
  while (kb < kMaxKeyBits && (int64_t(1) << kb) < cells) ++kb;
  while (kb > kMinKeyBits && (chunks << kb) > kMaxBuckets) --kb;
  L.chunk_shift = cs;
  L.dir_bits = kb / 4 < kMaxDirBits ? kb / 4 : kMaxDirBits;
  L.pos_bits = kb - L.dir_bits;
  L.buckets = chunks << kb;
  L.tiles = (L.buckets + kScanTile - 1) / kScanTile;
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  L.box = 0;
  L.plan = 256;
  L.keys = L.plan + up(sizeof(Plan));
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
  auto* box = reinterpret_cast<uint32_t*>(base + L.box);
  auto* plan = reinterpret_cast<Plan*>(base + L.plan);
  auto* keys = reinterpret_cast<uint32_t*>(base + L.keys);
  auto* counts = reinterpret_cast<uint32_t*>(base + L.counts);
  auto* tile_sum = reinterpret_cast<uint32_t*>(base + L.tile_sum);
  auto* out = reinterpret_cast<int32_t*>(base + L.order);
  const size_t arr = (L.total - L.sorted) / 8;
  Dst dst;
  for (int a = 0; a < 8; ++a) dst.a[a] = reinterpret_cast<double*>(base + L.sorted + a * arr);
  if (cudaMemsetAsync(box, 0xff, 6 * sizeof(uint32_t), st) != cudaSuccess ||
      cudaMemsetAsync(box + 6, 0, 6 * sizeof(uint32_t), st) != cudaSuccess ||
      cudaMemsetAsync(counts, 0, (size_t)L.buckets * 4, st) != cudaSuccess)
    return RBG_ERR_CUDA;
  const int64_t blocks = (n + kThreads - 1) / kThreads;
  const int box_blocks = (int)(blocks < 1216 ? blocks : 1216);
  bbox_kernel<<<box_blocks, kThreads, 0, st>>>(in, n, box);
  plan_kernel<<<1, 32, 0, st>>>(box, L.dir_bits, L.pos_bits, L.chunk_shift, plan);
  key_kernel<<<(unsigned)blocks, kThreads, 0, st>>>(in, n, plan, keys, counts);
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
