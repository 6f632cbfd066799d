// Device self-tests of the integer-pipe binary64 arithmetic (vg_fp64emu.cuh)
// against the hardware instructions, reachable through the C ABI so that the
// test suite checks the exact code the kernels use.
#include "vg_fp64emu.cuh"
#include "vg_internal.h"
#include "vg_philox.cuh"

namespace vg {
namespace {

__device__ __forceinline__ uint64_t dbits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double bdbl(uint64_t x) { return __longlong_as_double((long long)x); }

// operand pairs of several shapes: random exponents, equal exponents, wide
// exponent gaps, all-ones significands (carries), exact half-way cases,
// numbers near the subnormal range, zeros, and values in [0, 1)
__device__ void make_pair(uint64_t i, uint64_t seed, uint64_t &a, uint64_t &b) {
  Philox4 r = philox_draw(seed, i, 0, 11);
  Philox4 s = philox_draw(seed, i, 1, 11);
  uint64_t ma = ((uint64_t)r.v[1] << 32 | r.v[0]) & EMU_M52;
  uint64_t mb = ((uint64_t)s.v[1] << 32 | s.v[0]) & EMU_M52;
  unsigned kind = r.v[2] % 9;
  int ea = 900 + (int)(r.v[3] % 200), eb = 900 + (int)(s.v[3] % 200);
  switch (kind) {
    case 1: eb = ea; break;
    case 2: eb = ea - (int)(s.v[2] % 70); break;
    case 3: ma = EMU_M52 - (r.v[3] & 7); mb = EMU_M52 - (s.v[3] & 7); eb = ea - (int)(s.v[2] % 4); break;
    case 4: {  // b is exactly half an ulp of a (or of a's neighbour) -> ties
      eb = ea - 53 + (int)(s.v[2] % 3);
      mb = (s.v[2] & 8) ? 0 : (1ull << 51);
      break;
    }
    case 5: ea = 1 + (int)(r.v[3] % 60); eb = 1 + (int)(s.v[3] % 60); break;
    case 6: ea = 0; ma = 0; break;
    case 7: ea = 1012 + (int)(r.v[3] % 11); eb = 1012 + (int)(s.v[3] % 11); break;
    case 8: eb = ea - 52 - (int)(s.v[2] % 4); break;
    default: break;
  }
  if (eb < 0) eb = 0;
  if (ea < 0) ea = 0;
  a = ((uint64_t)ea << 52) | ma;
  b = ((uint64_t)eb << 52) | mb;
  if (eb == 0) b = mb ? 0 : b;
}

__global__ void k_selftest(uint64_t n, uint64_t seed, unsigned long long *counts) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t a, b;
  make_pair(i, seed, a, b);
  // add
  {
    bool ok = true;
    uint64_t r = emu_add_pos(a, b, ok);
    if (ok) {
      if (r != dbits(__dadd_rn(bdbl(a), bdbl(b)))) atomicAdd(&counts[0], 1ull);
    } else {
      atomicAdd(&counts[3], 1ull);
    }
  }
  // mul: the general emulation and the gather kernels' form
  {
    bool ok = true;
    uint64_t r = emu_mul_pos(a, b, ok);
    const uint64_t hw = dbits(__dmul_rn(bdbl(a), bdbl(b)));
    if (ok) {
      if (r != hw) atomicAdd(&counts[1], 1ull);
    } else {
      atomicAdd(&counts[4], 1ull);
    }
    bool ok2 = true;
    uint64_t r2 = emu_mul_fast(a, b, ok2);
    if (ok2 && r2 != hw) atomicAdd(&counts[1], 1ull);
  }
  // div (b > 0): the general emulation and the gather kernels' form
  if (b) {
    bool ok = true;
    uint64_t r = emu_div_pos(a, b, ok);
    const uint64_t hw = dbits(__ddiv_rn(bdbl(a), bdbl(b)));
    if (ok) {
      if (r != hw) atomicAdd(&counts[2], 1ull);
    } else {
      atomicAdd(&counts[5], 1ull);
    }
    bool ok2 = true;
    uint64_t r2 = emu_div_fast(a, b, ok2);
    if (ok2 && r2 != hw) atomicAdd(&counts[2], 1ull);
  }
  // the gather kernels' product for a weight that is a multiple of 2^-53 in
  // (0, 1] (only the other operand's exponent is checked)
  {
    Philox4 g = philox_draw(seed, i, 2, 12);
    uint64_t u = (((uint64_t)g.v[1] << 32 | g.v[0]) >> 11) >> (g.v[2] % 53);
    if (g.v[3] % 17 == 0) u = 1ull << 53;
    if (u == 0) u = 1;
    const double w = (double)u * 0x1p-53;  // exact
    bool ok = true;
    uint64_t r = emu_mul_grid(dbits(w), b, ok);
    if (ok && r != dbits(__dmul_rn(w, bdbl(b)))) atomicAdd(&counts[1], 1ull);
  }
  // exact scaling by powers of two
  {
    bool ok = true;
    const int k = (int)(a % 7) - 3;
    uint64_t r = emu_scale2(b, k, ok);
    if (ok && r != dbits(__dmul_rn(bdbl(b), ldexp(1.0, k)))) atomicAdd(&counts[1], 1ull);
  }
}

// Throughput of one arithmetic form: every thread of the first `active`
// lanes of each warp runs `iters` rounds of 8 independent dependency chains
// (the other lanes branch around the loop, so the warp issues with a
// partial mask).  mode 0: binary64 add, 1: binary64 multiply, 2: fused
// multiply-add, 3: the gather kernels' integer-pipe product of a 2^-53-grid
// weight (emu_mul_grid), 4: a 32-bit integer chain u = u (u | 1) + c (two
// integer operations per round).
// The chains' results are stored so that nothing is optimised away.
__global__ void k_rate(int mode, uint32_t iters, uint32_t active, double *sink) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (lane >= active) return;
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = 1.0 + 1e-3 * (double)(k + (gid & 7));
  if (mode == 0) {
    const double c = 1e-12;
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
      for (int k = 0; k < 8; k++) v[k] = __dadd_rn(v[k], c);
    }
  } else if (mode == 1) {
    const double c = 1.0 + 1e-12;
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
      for (int k = 0; k < 8; k++) v[k] = __dmul_rn(v[k], c);
    }
  } else if (mode == 2) {
    const double c = 1.0 + 1e-12, d = 1e-12;
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
      for (int k = 0; k < 8; k++) v[k] = __fma_rn(v[k], c, d);
    }
  } else if (mode == 3) {
    const uint64_t w = dbits(0.75);  // 3 * 2^-2: on the 2^-53 grid
    uint64_t u[8];
#pragma unroll
    for (int k = 0; k < 8; k++) u[k] = dbits(v[k]);
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        bool ok;
        const uint64_t r = emu_mul_grid(w, u[k], ok);
        u[k] = ok ? (r | (1ull << 62)) & ~(1ull << 61) : u[k] + 1;  // stay in [1, 2)
      }
    }
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = bdbl(u[k]);
  } else {
    uint32_t u[8];
#pragma unroll
    for (int k = 0; k < 8; k++) u[k] = (uint32_t)gid + k;
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
      for (int k = 0; k < 8; k++) u[k] = u[k] * (u[k] | 1u) + 0x9e3779b9u;  // no closed form
    }
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = (double)u[k];
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += v[k];
  if (s == 12345.678) sink[gid & 1023] = s;  // practically never: keeps the chains live
}

}  // namespace
}  // namespace vg

using namespace vg;
namespace vg {
void set_last_error(const std::string &m);
}

extern "C" int vg_selftest_fp64(uint64_t n, uint64_t seed, uint64_t *counts_out) {
  try {
    unsigned long long *d = nullptr;
    VG_CUDA(cudaMalloc(&d, 6 * 8));
    VG_CUDA(cudaMemset(d, 0, 6 * 8));
    k_selftest<<<(unsigned)((n + 255) / 256), 256>>>(n, seed, d);
    VG_CUDA(cudaGetLastError());
    VG_CUDA(cudaMemcpy(counts_out, d, 6 * 8, cudaMemcpyDeviceToHost));
    VG_CUDA(cudaFree(d));
    return VG_OK;
  } catch (const Error &e) {
    set_last_error(e.msg);
    return e.code;
  }
}

extern "C" int vg_selftest_rate(int mode, uint32_t blocks, uint32_t iters, uint32_t active_lanes,
                                double *ms_out, double *lane_ops_out) {
  try {
    if (mode < 0 || mode > 4 || blocks == 0 || iters == 0 || active_lanes == 0 ||
        active_lanes > 32 || !ms_out || !lane_ops_out)
      fail(VG_ERR_ARG, "vg_selftest_rate: mode 0..4, blocks, iters > 0, 1..32 active lanes");
    double *sink = nullptr;
    VG_CUDA(cudaMalloc(&sink, 1024 * 8));
    cudaEvent_t a, b;
    VG_CUDA(cudaEventCreate(&a));
    VG_CUDA(cudaEventCreate(&b));
    k_rate<<<blocks, 256>>>(mode, iters / 8 + 1, active_lanes, sink);  // warm-up
    VG_CUDA(cudaEventRecord(a));
    k_rate<<<blocks, 256>>>(mode, iters, active_lanes, sink);
    VG_CUDA(cudaEventRecord(b));
    VG_CUDA(cudaEventSynchronize(b));
    VG_CUDA(cudaGetLastError());
    float ms = 0.f;
    VG_CUDA(cudaEventElapsedTime(&ms, a, b));
    VG_CUDA(cudaEventDestroy(a));
    VG_CUDA(cudaEventDestroy(b));
    VG_CUDA(cudaFree(sink));
    *ms_out = ms;
    *lane_ops_out = (double)blocks * (256.0 / 32.0) * active_lanes * (double)iters * 8.0;
    return VG_OK;
  } catch (const Error &e) {
    set_last_error(e.msg);
    return e.code;
  }
}
