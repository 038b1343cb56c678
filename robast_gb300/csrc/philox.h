// philox.h -- counter-based Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), written for both
// host C++ and CUDA device code.
//
// Every random draw of a trace is a pure function of (seed, ray id, draw
// number), replacing the shared gRandom of the reference
// (src/AOpticsManager.cxx:86,138,202,214,216,276-280,407,508 and
// src/ARayShooter.cxx:213-214): results do not depend on thread count,
// launch shape or scheduling.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define RBG_HD __host__ __device__ __forceinline__
#else
#define RBG_HD inline
#endif

namespace rbg {

struct Philox4 {
  uint32_t v[4];
};

RBG_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  lo = a * b;
  hi = __umulhi(a, b);
#else
  uint64_t p = (uint64_t)a * (uint64_t)b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
#endif
}

// Ten rounds of Philox4x32 on counter c with key (k0, k1).
RBG_HD Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                             uint32_t c3, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(M0, c0, hi0, lo0);
    mulhilo32(M1, c2, hi1, lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += W0;
    k1 += W1;
  }
  Philox4 out;
  out.v[0] = c0; out.v[1] = c1; out.v[2] = c2; out.v[3] = c3;
  return out;
}

// 53-bit uniform in [0, 1) from two 32-bit words.
RBG_HD double u53(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)m * (1.0 / 9007199254740992.0);
}

// Per-ray stream: draw k of ray `id` uses counter (k, stream, id_lo, id_hi).
// Stream 0 is the tracer, stream 1 the ray sources.
struct RayRng {
  uint32_t k0, k1, id_lo, id_hi, n, stream;
  RBG_HD void init(uint64_t seed, uint64_t id, uint32_t s = 0) {
    k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
    id_lo = (uint32_t)id; id_hi = (uint32_t)(id >> 32);
    n = 0;
    stream = s;
  }
  RBG_HD Philox4 next() { return philox4x32_10(n++, stream, id_lo, id_hi, k0, k1); }
  // uniform in [0, 1)
  RBG_HD double uniform() {
    Philox4 r = next();
    return u53(r.v[0], r.v[1]);
  }
};

}  // namespace rbg
