// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), shared by the
// host code and the kernels.  The reference has no RNG of its own; every
// test model draws from this stream keyed by (seed, agent number, step,
// purpose tag), so CPU and GPU runs see the same numbers.
//
//   key     = (seed & 0xffffffff, seed >> 32)
//   counter = (agent_nr & 0xffffffff, agent_nr >> 32, step, tag)
//   u64     = out[1] << 32 | out[0]
//   double  = (u64 >> 11) * 2^-53                      in [0, 1)
//   bounded = (out[k] * range) >> 32  (multiply-high)   in [0, range)
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define VG_HD __host__ __device__ __forceinline__
#else
#define VG_HD inline
#endif

namespace vg {

enum PhiloxTag : uint32_t {
  TAG_INIT = 1,     // initial agent state
  TAG_EDGE = 2,     // graph generation
  TAG_INFECT = 3,   // SIR infection draw
  TAG_MOVE = 4,     // walker move
  TAG_SRC = 5,      // Chung-Lu edge source
  TAG_DST = 6,      // Chung-Lu edge target
  TAG_WEIGHT = 7,   // edge weight
  TAG_PARAM = 8,    // per-instance parameters of batched runs
};

struct Philox4 {
  uint32_t v[4];
};

VG_HD uint32_t mulhi32(uint32_t a, uint32_t b, uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *lo = (uint32_t)p;
  return (uint32_t)(p >> 32);
}

VG_HD Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                            uint32_t k0, uint32_t k1) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; r++) {
    uint32_t lo0, lo1;
    uint32_t hi0 = mulhi32(0xD2511F53u, c0, &lo0);
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c2, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  Philox4 o;
  o.v[0] = c0;
  o.v[1] = c1;
  o.v[2] = c2;
  o.v[3] = c3;
  return o;
}

VG_HD Philox4 philox_draw(uint64_t seed, uint64_t nr, uint32_t step,
                          uint32_t tag) {
  return philox4x32_10((uint32_t)nr, (uint32_t)(nr >> 32), step, tag,
                       (uint32_t)seed, (uint32_t)(seed >> 32));
}

VG_HD uint64_t philox_u64(const Philox4 &p) {
  return ((uint64_t)p.v[1] << 32) | p.v[0];
}

// top 53 bits scaled by 2^-53: exact in double, in [0, 1)
VG_HD double u64_to_unit(uint64_t x) {
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

// the bit pattern of u64_to_unit(x), built with integer operations (exact:
// the top 53 bits k scaled by 2^-53 have exponent bitlength(k) - 54 and
// k's bits below its leading one as the fraction)
VG_HD uint64_t u64_to_unit_bits(uint64_t x) {
  const uint64_t k = x >> 11;
  if (k == 0) return 0;
#ifdef __CUDA_ARCH__
  const int L = 64 - __clzll((long long)k);
#else
  const int L = 64 - __builtin_clzll(k);
#endif
  const uint64_t frac = (k << (53 - L)) & ((1ull << 52) - 1);
  return ((uint64_t)(1023 + L - 54) << 52) | frac;
}

// u64_to_unit(x) < p for a non-negative finite p, decided on the integer
// pipes: non-negative doubles are ordered as their bit patterns are
VG_HD bool unit_below(uint64_t x, double p) {
  union {
    double d;
    uint64_t u;
  } pb;
  pb.d = p;
  return u64_to_unit_bits(x) < pb.u;
}

// (top53 + 1) * 2^-53: in (0, 1]
VG_HD double u64_to_unit_open0(uint64_t x) {
  return (double)((x >> 11) + 1) * (1.0 / 9007199254740992.0);
}

VG_HD uint32_t bounded32(uint32_t x, uint32_t range) {
  return (uint32_t)(((uint64_t)x * (uint64_t)range) >> 32);
}

}  // namespace vg
