// Exact IEEE-754 binary64 round-to-nearest-even arithmetic on the integer
// pipe, for the hot gather kernels.
//
// GB300 executes FP64 at about 2 operations per clock per SM, 64x below
// its integer/FP32 issue rate.  The ordered neighbour folds need results
// bit-identical to sequential binary64 arithmetic, so this file implements
// the operations themselves with integer instructions, following the
// textbook algorithms (significand alignment with guard/round/sticky bits
// and normalisation for addition, the double-width significand product for
// multiplication, restoring quotient digits with a remainder test for
// division; e.g. J.-M. Muller et al., Handbook of Floating-Point Arithmetic,
// 2nd ed., Birkhauser 2018, ch. 7-8; D. Goldberg, What every computer
// scientist should know about floating-point arithmetic, 1991).
//
// Scope: non-negative, finite, normal operands and results (zero operands
// are handled).  Anything else sets ok = false and the caller uses the
// hardware instruction instead, so every result is the correctly rounded
// binary64 value.  A device self-test compares these functions with the
// hardware instructions on random and constructed operands.
#pragma once
#include <stdint.h>

namespace vg {

constexpr uint64_t EMU_M52 = (1ull << 52) - 1;
constexpr uint64_t EMU_H53 = 1ull << 52;

// a + b for non-negative doubles given as bit patterns.
__device__ __forceinline__ uint64_t emu_add_pos(uint64_t a, uint64_t b, bool &ok) {
  uint64_t hi = a > b ? a : b, lo = a > b ? b : a;  // bit order == value order
  if (lo == 0) return hi;
  unsigned eh = (unsigned)(hi >> 52), el = (unsigned)(lo >> 52);
  if (el == 0 || eh >= 2046) {  // subnormal operand or possible overflow
    ok = false;
    return 0;
  }
  uint64_t A = ((hi & EMU_M52) | EMU_H53) << 10;  // [2^62, 2^63), 10 low zero bits
  uint64_t B = ((lo & EMU_M52) | EMU_H53) << 10;
  unsigned d = eh - el;
  uint64_t Bs;
  if (d >= 64) Bs = 1;  // only the sticky bit remains
  else if (d) Bs = (B >> d) | (uint64_t)((B << (64 - d)) != 0);
  else Bs = B;
  uint64_t S = A + Bs;  // < 2^64
  unsigned e = eh;
  if (S >> 63) {
    S = (S >> 1) | (S & 1);
    e++;
  }
  uint64_t q = S >> 10;  // 53-bit significand
  unsigned r = (unsigned)S & 0x3FFu;  // guard bit 9, round/sticky below
  q += (r > 0x200u) || (r == 0x200u && (q & 1));
  if (q >> 53) {  // rounding carried out: q == 2^53
    q >>= 1;
    e++;
  }
  if (e >= 2047) {
    ok = false;
    return 0;
  }
  return ((uint64_t)e << 52) | (q & EMU_M52);
}

// a * b for non-negative doubles given as bit patterns.
__device__ __forceinline__ uint64_t emu_mul_pos(uint64_t a, uint64_t b, bool &ok) {
  if (a == 0 || b == 0) return 0;
  int ea = (int)(a >> 52), eb = (int)(b >> 52);
  if (ea == 0 || eb == 0 || ea == 2047 || eb == 2047) {
    ok = false;
    return 0;
  }
  uint64_t ma = (a & EMU_M52) | EMU_H53, mb = (b & EMU_M52) | EMU_H53;
  uint64_t lo = ma * mb, hi = __umul64hi(ma, mb);  // P in [2^104, 2^106)
  int e = ea + eb - 1023;
  int s = 52;
  if (hi >> 41) {  // P >= 2^105
    s = 53;
    e++;
  }
  uint64_t q = (hi << (64 - s)) | (lo >> s);  // top 53 bits
  uint64_t half = 1ull << (s - 1);
  uint64_t rem = lo & ((1ull << s) - 1);
  q += (rem > half) || (rem == half && (q & 1));
  if (q >> 53) {
    q >>= 1;
    e++;
  }
  if (e <= 0 || e >= 2047) {
    ok = false;
    return 0;
  }
  return ((uint64_t)e << 52) | (q & EMU_M52);
}

// a / b for positive normal doubles (b > 0), restoring division of the
// significands: 53 quotient bits, then the remainder decides the rounding.
__device__ __forceinline__ uint64_t emu_div_pos(uint64_t a, uint64_t b, bool &ok) {
  if (a == 0) return 0;
  int ea = (int)(a >> 52), eb = (int)(b >> 52);
  if (ea == 0 || eb == 0 || ea == 2047 || eb == 2047 || b == 0) {
    ok = false;
    return 0;
  }
  uint64_t ma = (a & EMU_M52) | EMU_H53, mb = (b & EMU_M52) | EMU_H53;
  int e = ea - eb + 1023;
  if (ma < mb) {  // bring the quotient into [1, 2)
    ma <<= 1;
    e--;
  }
  // quotient bits of ma / mb, most significant first; invariant R < 2 mb
  uint64_t R = ma, q = 0;
#pragma unroll 4
  for (int i = 0; i < 53; i++) {
    uint64_t t = R - mb;
    bool ge = R >= mb;
    q = (q << 1) | (uint64_t)ge;
    R = (ge ? t : R) << 1;
  }
  // R = 2 * remainder; compare with mb for the half-way point
  q += (R > mb) || (R == mb && (q & 1));
  if (q >> 53) {
    q >>= 1;
    e++;
  }
  if (e <= 0 || e >= 2047) {
    ok = false;
    return 0;
  }
  return ((uint64_t)e << 52) | (q & EMU_M52);
}

// a * b for positive doubles given as bit patterns, the form the gather
// kernels use: correctly rounded when both operands are normal and the
// product is normal (ok = false otherwise, and the caller multiplies on the
// FP64 pipe).  The significand product comes from four 32x32-bit multiplies
// with 64-bit addends; the rounded significand q (hidden bit included) is
// packed by adding it to (exponent - 1) << 52, so that a carry out of the
// rounding (q = 2^53) raises the exponent by itself.
template <bool GRID_A>
__device__ __forceinline__ uint64_t emu_mul_fast_t(uint64_t a, uint64_t b, bool &ok) {
  const uint32_t ahi = (uint32_t)(a >> 32), alo = (uint32_t)a;
  const uint32_t bhi = (uint32_t)(b >> 32), blo = (uint32_t)b;
  const uint32_t ea = ahi >> 20, eb = bhi >> 20;
  const uint32_t mah = (ahi & 0xFFFFFu) | 0x100000u, mbh = (bhi & 0xFFFFFu) | 0x100000u;
  const uint64_t L = (uint64_t)alo * blo;                 // product bits 0..63
  uint64_t S = (uint64_t)mah * blo + (L >> 32);           // < 2^53 + 2^32
  S += (uint64_t)alo * mbh;                               // bits 32.. (< 2^55)
  const uint64_t U = (uint64_t)mah * mbh + (S >> 32);     // bits 64.. (< 2^42 + 2^23)
  const uint32_t ul = (uint32_t)S;                        // bits 32..63
  const uint32_t big = (uint32_t)(U >> 41);               // product >= 2^105
  const uint32_t sh = 20u + big;
  uint64_t q = (U << (32u - sh)) | (uint64_t)(ul >> sh);  // 53 significant bits
  const uint32_t rb = (ul >> (sh - 1u)) & 1u;
  const uint32_t st = (ul & ((1u << (sh - 1u)) - 1u)) | (uint32_t)L;
  q += rb & ((uint32_t)(st != 0u) | (uint32_t)q);
  const int e = (int)ea + (int)eb - 1023 + (int)big;  // biased exponent before rounding
  if (GRID_A)  // a's exponent is 970..1023: only b's needs a check
    ok = (eb - 54u) <= 1990u;
  else
    ok = (e > 0) & (e < 2046) & (ea - 1u < 2046u) & (eb - 1u < 2046u);
  return ((uint64_t)(e - 1) << 52) + q;
}
__device__ __forceinline__ uint64_t emu_mul_fast(uint64_t a, uint64_t b, bool &ok) {
  return emu_mul_fast_t<false>(a, b, ok);
}
// the same for a weight a that is a multiple of 2^-53 in (0, 1]
__device__ __forceinline__ uint64_t emu_mul_grid(uint64_t a, uint64_t b, bool &ok) {
  return emu_mul_fast_t<true>(a, b, ok);
}

// a / b for positive doubles given as bit patterns, the per-row division of
// the gather kernels: correctly rounded when both operands are normal and
// the quotient is normal (ok = false otherwise, and the caller divides on
// the FP64 pipe).  Significands A in [B, 2B), B in [2^52, 2^53); quotient
// q = floor(A 2^52 / B).  A float reciprocal of B >> 29 gives y0 ~ 2^83/B
// (relative error < 2^-22), one Newton step gives Y ~ 2^115/B (< 2^-43),
// the quotient estimate from Y is corrected once through its remainder (the
// remainder stays below 2^62 in magnitude) and then exactly: the remainder
// N - q B is small enough to be exact in 64-bit two's complement.  The
// remainder decides the rounding (ties to even).  Newton-Raphson reciprocal
// refinement and remainder correction as in P. Markstein, IBM J. Res. Dev.
// 34(1), 1990.
__device__ __forceinline__ uint64_t emu_div_fast(uint64_t a, uint64_t b, bool &ok) {
  const uint32_t ea = (uint32_t)(a >> 52), eb = (uint32_t)(b >> 52);
  uint64_t A = (a & EMU_M52) | EMU_H53;
  const uint64_t B = (b & EMU_M52) | EMU_H53;
  int e = (int)ea - (int)eb + 1023;
  if (A < B) {
    A <<= 1;
    e--;
  }
  const float fb = __uint_as_float((150u << 23) | ((uint32_t)(B >> 29) & 0x7FFFFFu));  // B >> 29
  const uint32_t ub = __float_as_uint(__frcp_rn(fb));
  const uint64_t y0 = (uint64_t)((ub & 0x7FFFFFu) | 0x800000u) << ((ub >> 23) - 96u);
  const int64_t e1 = (int64_t)(0ull - B * y0);  // 2^83 - B y0 (fits: |.| < 2^62)
  const uint64_t Y = (y0 << 32) + (uint64_t)__mul64hi((long long)(y0 << 13), (long long)e1);
  const uint64_t N = A << 52;  // A 2^52 mod 2^64
  uint64_t q = __umul64hi(A << 1, Y);
  const int64_t r1 = (int64_t)(N - q * B);
  q += (uint64_t)(__mul64hi((long long)r1, (long long)(Y >> 1)) >> 50);
  int64_t r = (int64_t)(N - q * B);
#pragma unroll
  for (int k = 0; k < 2; k++)
    if (r < 0) {
      q--;
      r += (int64_t)B;
    }
#pragma unroll
  for (int k = 0; k < 2; k++)
    if (r >= (int64_t)B) {
      q++;
      r -= (int64_t)B;
    }
  const uint64_t r2 = (uint64_t)r << 1;
  q += (r2 > B) || (r2 == B && (q & 1));
  ok = (e > 0) & (e < 2046) & (ea - 1u < 2046u) & (eb - 1u < 2046u);
  return ((uint64_t)(e - 1) << 52) + q;
}

// x * 2^k for a positive double x (bit pattern) when x and the result are
// normal: exact; ok = false otherwise.
__device__ __forceinline__ uint64_t emu_scale2(uint64_t x, int k, bool &ok) {
  const int ex = (int)(x >> 52);
  ok = (ex >= 1) & (ex <= 2046) & (ex + k >= 1) & (ex + k <= 2046) & ((x >> 63) == 0);
  return x + ((uint64_t)(int64_t)k << 52);
}

}  // namespace vg
