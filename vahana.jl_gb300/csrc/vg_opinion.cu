// Bounded-confidence opinion step: the gather kernel of the headline
// workload (transition "bounded_confidence").
//
// Model (a test model of the transition step, written with the reference's
// accessors: edges/neighborstates over the agent's in-edges in insertion
// order, src/EdgeMethods.jl:705-781): Opinion{x::Float64}, in-edges with a
// Float64 weight w.  Sequentially over the in-edges: a neighbour with
// |x_j - x| < eps adds w_j to sw and w_j * x_j to swx; then
// x' = a * x + b * (swx / sw), or x when no neighbour qualifies.
//
// Degree buckets:
//   rows with in-degree <= hub_thr: one thread per row, folding in order;
//     bit-identical to the sequential binary64 computation.
//   rows above hub_thr ("hubs"): one warp per row, each lane folds a
//     contiguous chunk in order, the chunk sums are combined in a fixed
//     lane tree.  The additions are regrouped, so these rows agree with the
//     sequential fold to within 1e-12 relative; hub_thr = 2^32-1 disables
//     the split and keeps every row bit-exact.
//   The hub warps are the first blocks of the grid so that they start
//   first.
//
// Arithmetic placement on GB300, whose FP64 pipe issues about 2 operations
// per clock per SM: the threshold test runs on a float filter of the two
// doubles' high words (exact binary64 test only within 1e-5 of eps); the
// products w_j * x_j stay on the FP64 pipe; the additions of sw and swx and
// the per-row division and mixing run as exact round-to-nearest-even
// integer arithmetic (vg_fp64emu.cuh), falling back to the FP64
// instruction outside its range.  Every operation is the correctly
// rounded binary64 result in the reference's order.
#include <algorithm>
#include <cmath>

#include "vg_fp64emu.cuh"
#include "vg_internal.h"

namespace vg {
namespace {

constexpr int TPB = 256;

struct OpinionArgs {
  const uint32_t *__restrict__ rp;
  const uint32_t *__restrict__ src;
  const double *__restrict__ w;
  const double *__restrict__ x;
  double *__restrict__ xo;
  uint64_t n, nrows;
  const uint32_t *__restrict__ hub_rows;
  uint64_t nhub;
  uint32_t hub_thr;
  unsigned hub_blocks;
  double eps, a, b;
  float eps_lo, eps_hi;  // float filter: certainly inside / certainly outside
};

__device__ __forceinline__ uint64_t bits(double v) { return (uint64_t)__double_as_longlong(v); }
__device__ __forceinline__ double dbl(uint64_t v) { return __longlong_as_double((long long)v); }

// float image of a double in [2^-126, 2) from its high word (exponent
// re-biased, mantissa truncated to 20 bits); `ok` false outside that range
__device__ __forceinline__ float hi_float(double v, bool &ok) {
  uint32_t h = (uint32_t)__double2hiint(v);
  ok = (h - 0x38100000u) < (0x40000000u - 0x38100000u);
  return __int_as_float((int)((h - 0x38000000u) << 3));
}

// exact binary64 test, out of line so that it is never evaluated
// speculatively on the FP64 pipe
__device__ __noinline__ bool within_exact(double xj, double xi, double eps) {
  return fabs(__dsub_rn(xj, xi)) < eps;
}

// |x_j - x_i| < eps, exactly as binary64 would decide it
__device__ __forceinline__ bool within(double xj, double xi, float fxi, bool xi_ok,
                                       const OpinionArgs &p) {
  bool ok;
  float fxj = hi_float(xj, ok);
  if (ok && xi_ok) {
    float fd = fabsf(fxj - fxi);
    if (fd < p.eps_lo) return true;
    if (fd > p.eps_hi) return false;
  }
  return within_exact(xj, xi, p.eps);
}

__device__ __noinline__ uint64_t add_rn(uint64_t a, uint64_t b) {
  bool ok = ((a | b) >> 63) == 0;
  uint64_t r = ok ? emu_add_pos(a, b, ok) : 0;
  if (ok) return r;
  return bits(__dadd_rn(dbl(a), dbl(b)));
}

__device__ __noinline__ uint64_t mul_rn(uint64_t a, uint64_t b) {
  bool ok = ((a | b) >> 63) == 0;
  uint64_t r = ok ? emu_mul_pos(a, b, ok) : 0;
  if (ok) return r;
  return bits(__dmul_rn(dbl(a), dbl(b)));
}

__device__ __noinline__ uint64_t div_rn(uint64_t a, uint64_t b) {
  bool ok = ((a | b) >> 63) == 0;
  uint64_t r = ok ? emu_div_pos(a, b, ok) : 0;
  if (ok) return r;
  return bits(__ddiv_rn(dbl(a), dbl(b)));
}

// Running sum held decoded: biased exponent e and the 53-bit significand m
// with its leading bit, value m * 2^(e - 1075).  e = 0 holds the bit
// pattern itself in m (zero, or a subnormal sum), handled by the general
// path.
struct Acc {
  uint32_t e;
  uint64_t m;
};

__device__ __forceinline__ uint64_t acc_bits(const Acc &a) {
  return a.e ? (((uint64_t)a.e << 52) | (a.m & EMU_M52)) : a.m;
}

__device__ __noinline__ Acc acc_add_general(Acc a, uint64_t pb) {
  uint64_t r = add_rn(acc_bits(a), pb);
  Acc o;
  o.e = (uint32_t)(r >> 52);
  o.m = o.e ? ((r & EMU_M52) | EMU_H53) : r;
  return o;
}

// a += p (p >= 0 given as bits), correctly rounded.  Fast path: p is 1 to
// 31 binades below the sum and the sum stays in its binade -- then the sum
// is m + round(P / 2^d) in units of the sum's ulp, ties to even.
__device__ __forceinline__ void acc_add(Acc &a, uint64_t pb) {
  uint32_t phi = (uint32_t)(pb >> 32), plo = (uint32_t)pb;
  uint32_t ep = phi >> 20;
  uint32_t d = a.e - ep;
  if (d - 1u < 31u && ep != 0 && a.e < 2046u) {
    uint32_t Phi = (phi & 0xFFFFFu) | 0x100000u;
    uint32_t Qlo = __funnelshift_r(plo, Phi, d);
    uint32_t Qhi = Phi >> d;
    uint32_t R = plo & ((1u << d) - 1u);
    uint32_t half = 1u << (d - 1u);
    uint64_t M = a.m + (((uint64_t)Qhi << 32) | Qlo);
    M += (uint64_t)((R > half) | ((R == half) & (uint32_t)M));
    if (M < (1ull << 53)) {
      a.m = M;
      return;
    }
  } else if (d - 54u < 2000u && a.e != 0 && ep != 0) {
    return;  // p < half an ulp of the sum: the sum is unchanged
  }
  a = acc_add_general(a, pb);
}

// x' = a x + b (swx / sw), each operation rounded in this order
__device__ __noinline__ double finish(double pa, double pb_, double xi, uint64_t sw,
                                      uint64_t swx) {
  uint64_t m = div_rn(swx, sw);
  uint64_t l = mul_rn(bits(pa), bits(xi));
  uint64_t r = mul_rn(bits(pb_), m);
  return dbl(add_rn(l, r));
}

// ordered fold of edges [b, e) of a row into (sw, swx, cnt)
__device__ __forceinline__ void fold(const OpinionArgs &p, uint32_t b, uint32_t e, double xi,
                                     float fxi, bool xi_ok, Acc &sw, Acc &swx,
                                     uint32_t &cnt) {
  for (uint32_t k = b; k < e; k++) {
    double xj = __ldg(p.x + __ldg(p.src + k));
    if (within(xj, xi, fxi, xi_ok, p)) {
      double wk = __ldg(p.w + k);
      double pk = __dmul_rn(wk, xj);
      acc_add(sw, bits(wk));
      acc_add(swx, bits(pk));
      cnt++;
    }
  }
}

__global__ void __launch_bounds__(TPB) k_opinion(OpinionArgs p) {
  if (blockIdx.x < p.hub_blocks) {
    // one warp per hub row: lane l folds the l-th contiguous chunk in order
    const int lane = threadIdx.x & 31;
    uint64_t h = (uint64_t)blockIdx.x * (TPB / 32) + (threadIdx.x >> 5);
    if (h >= p.nhub) return;
    uint32_t r = p.hub_rows[h];
    double xi = p.x[r];
    bool xi_ok;
    float fxi = hi_float(xi, xi_ok);
    uint32_t b = p.rp[r], e = p.rp[r + 1];
    uint32_t chunk = (e - b + 31) / 32;
    uint32_t cb = min(e, b + lane * chunk), ce = min(e, cb + chunk);
    Acc asw{0, 0}, aswx{0, 0};
    uint32_t cnt = 0;
    fold(p, cb, ce, xi, fxi, xi_ok, asw, aswx, cnt);
    uint64_t sw = acc_bits(asw), swx = acc_bits(aswx);
    // fixed tree: lane l receives lane l + off
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      uint64_t osw = __shfl_down_sync(0xffffffffu, sw, off);
      uint64_t oswx = __shfl_down_sync(0xffffffffu, swx, off);
      uint32_t ocnt = __shfl_down_sync(0xffffffffu, cnt, off);
      if ((lane & (2 * off - 1)) == 0 && ocnt) {
        sw = add_rn(sw, osw);
        swx = add_rn(swx, oswx);
        cnt += ocnt;
      }
    }
    if (lane == 0) p.xo[r] = cnt ? finish(p.a, p.b, xi, sw, swx) : xi;
    return;
  }
  uint64_t i = (uint64_t)(blockIdx.x - p.hub_blocks) * TPB + threadIdx.x;
  if (i >= p.n) return;
  double xi = p.x[i];
  if (i >= p.nrows) {
    p.xo[i] = xi;
    return;
  }
  uint32_t b = p.rp[i], e = p.rp[i + 1];
  if (e - b > p.hub_thr) return;  // a hub warp writes this row
  bool xi_ok;
  float fxi = hi_float(xi, xi_ok);
  Acc sw{0, 0}, swx{0, 0};
  uint32_t cnt = 0;
  fold(p, b, e, xi, fxi, xi_ok, sw, swx, cnt);
  p.xo[i] = cnt ? finish(p.a, p.b, xi, acc_bits(sw), acc_bits(swx)) : xi;
}

}  // namespace

// apply!(sim, bounded_confidence, [T], [T, E], [T]; params = [E, eps, a, b,
// hub_thr]); defaults eps 0.3, a 0.5, b 1 - a, hub_thr 256.
void tr_bounded_confidence(ApplyCtx &c) {
  Sim &s = *c.sim;
  const AgentTypeDesc &ad = s.model->at(c.call_type);
  if (ad.fields.empty() || ad.fields[0].dtype != VG_F64)
    fail(VG_ERR_ARG, "bounded_confidence: agent field 0 must be Float64");
  if (!ad.immortal()) fail(VG_ERR_ARG, "bounded_confidence: the opinion type is :Immortal");
  if (c.nparams < 1) fail(VG_ERR_ARG, "bounded_confidence: parameter 0 is the edge type");
  int e = (int)c.params[0];
  const EdgeTypeDesc &ed = s.model->et(e);
  if (!ed.stores_payload() || ed.fields[0].dtype != VG_F64 || !ed.stores_src())
    fail(VG_ERR_ARG, "bounded_confidence: edges need a source and a Float64 weight");
  if (c.sim->check_readable && !c.in_read(VG_EDGE(e)))
    fail(VG_ERR_ASSERT, "You try to access an edge of type " + ed.name +
                            " but the type is not in the `read` argument of the apply! function.");
  if (c.sim->check_readable && !c.in_read(c.call_type))
    fail(VG_ERR_ASSERT, ad.name + " must be in the `read` argument of the transition function.");
  if (!c.writes_call()) fail(VG_ERR_ARG, "bounded_confidence: the called type must be in `write`");
  if (c.with_edge >= 0) fail(VG_ERR_ARG, "bounded_confidence: with_edge is not supported");
  double eps = c.param(1, 0.3);
  double a = c.param(2, 0.5);
  double b = c.nparams > 3 ? c.params[3] : 1.0 - a;
  double thr_d = c.param(4, 256);
  uint32_t thr = thr_d >= 4294967295.0 ? 0xffffffffu : (uint32_t)thr_d;
  EdgeStore &es = s.edges[e];
  DevCSRView v = csr_view(s, e, c.call_type);
  if (v.nedges && v.src_type_const != c.call_type)
    fail(VG_ERR_ARG, "bounded_confidence: sources must be of the called type");
  DevAgentView av = agent_view(s, c.call_type);
  if (av.n == 0) return;
  OpinionArgs p{};
  p.rp = v.row_ptr;
  p.src = v.src;
  p.w = (const double *)v.payload[0];
  p.x = (const double *)av.rd[0];
  p.xo = (double *)av.wr[0];
  p.n = av.n;
  p.nrows = v.nrows;
  p.eps = eps;
  p.a = a;
  p.b = b;
  p.eps_lo = (float)(eps - 1e-5);
  p.eps_hi = (float)(eps + 1e-5);
  p.hub_thr = 0xffffffffu;
  if (v.nedges && c.call_type < (int)es.csr.size() && thr != 0xffffffffu) {
    CSR &cs = es.csr[c.call_type];
    ensure_schedule(s, cs, thr);
    p.hub_rows = cs.hub_rows.as<uint32_t>();
    p.nhub = cs.nhub;
    p.hub_thr = thr;
    p.hub_blocks = (unsigned)((cs.nhub + (TPB / 32) - 1) / (TPB / 32));
  }
  unsigned grid = p.hub_blocks + (unsigned)((av.n + TPB - 1) / TPB);
  k_opinion<<<grid, TPB, 0, s.stream>>>(p);
  VG_CUDA(cudaGetLastError());
}

}  // namespace vg
