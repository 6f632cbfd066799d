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
// Row classes:
//   rows with in-degree <= hub_thr, and agents with no in-edge: slices of
//     32 rows of similar degree (degree-sorted windows) whose edges sit in
//     a column-major copy of the CSR (SELL-C-sigma, built once per graph by
//     ensure_schedule): lane l of a warp folds its row's edges in insertion
//     order while every load of the warp is one coalesced access --
//     bit-identical to the sequential binary64 computation.
//   rows above block_thr (an optional parameter): one block per row, the
//     row's edges staged through shared memory by bulk copies (hub_block).
//   rows above hub_thr ("hubs"): one warp per row, lane l folds the edges
//     l, l + 32, ... in order and the 32 lane sums are combined in a fixed
//     tree.  The additions are regrouped, so these rows agree with the
//     sequential fold to within 1e-12 relative; hub_thr = 2^32-1 disables
//     the split and keeps every row bit-exact.
//   The hub warps are the first blocks of the grid so that they start
//   first.
//
// Arithmetic placement on GB300 (the FP64 pipe executes 5.3e11 binary64
// operations per second, far below the integer pipes):
//   threshold test  float filter of the opinions' high words; the exact
//                   binary64 test only within 1e-5 of eps
//   w_j * x_j       exact round-to-nearest-even product from 32x32-bit
//                   multiplies (vg_fp64emu.cuh)
//   swx += p,       the hardware binary64 adds, predicated on the test: two
//   sw += w         FP64 warp instructions per slot (measured 5.3e11 lane
//                   operations per second on GB300, the same with any number
//                   of active lanes: the floor of this kernel)
//   per row         exact integer division, exponent scaling for mixing
//                   weights that are powers of two, one hardware add
// Every operation is the correctly rounded binary64 result, in the
// reference's order.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "vg_fp64emu.cuh"
#include "vg_internal.h"

namespace vg {
namespace {

constexpr int TPB = 128;

struct OpinionArgs {
  const uint32_t *__restrict__ rp;
  const uint32_t *__restrict__ src;
  const double *__restrict__ w;
  const double *__restrict__ x;
  double *__restrict__ xo;
  uint64_t n, nrows;
  const uint32_t *__restrict__ hub_rows;  // degree > hub_thr, split over a warp
  uint64_t nhub;
  uint64_t nbig;         // the first nbig hub rows take a whole block each
  int *status;           // the simulation's device error word
  const uint32_t *__restrict__ order;  // the other rows, degree-sorted windows
  const uint32_t *__restrict__ order_deg;  // their in-degrees, by position
  uint64_t norder;
  const uint64_t *__restrict__ slice_base;  // column-major slices of 32 rows
  const uint32_t *__restrict__ slice_deg;
  const uint32_t *__restrict__ sell_src;
  const double *__restrict__ sell_w;
  uint64_t nslices;
  uint32_t hub_thr;
  unsigned hub_blocks;   // blocks of the other hub rows, 4 per block
  double eps, a, b;
  int a_pow2, b_pow2, a_k, b_k;  // a = 2^a_k, b = 2^b_k (positive normal powers of two)
  float eps_lo, eps_hi;  // float filter: certainly inside / certainly outside
  int grid;              // all weights are multiples of 2^-53 in (0, 1] (exponent 970..1023)
  CSR *csr;              // host side only: the layout the arguments come from
};

__device__ __forceinline__ uint64_t bits(double v) { return (uint64_t)__double_as_longlong(v); }

// L2 policies: the edge columns stream through once per step (evict first);
// the opinions, gathered once per edge, should stay resident (evict last).
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint32_t ld_stream(const uint32_t *a, uint64_t pol) {
  uint32_t v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;"
               : "=r"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ double ld_stream(const double *a, uint64_t pol) {
  double v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;"
               : "=d"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ double ld_keep(const double *a, uint64_t pol) {
  double v;
  asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
  return v;
}
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

// |x_j - x_i| < eps, exactly as binary64 would decide it: the float
// filter decides unless |fd - eps| < 1e-5 or an opinion is outside the
// filter's range; then the exact test runs (out of line, so that its FP64
// subtraction is never issued for the lanes the filter decided)
__device__ __forceinline__ bool within(double xj, double xi, float fxi, bool xi_ok,
                                       const OpinionArgs &p) {
  bool ok;
  const float fxj = hi_float(xj, ok);
  const float fd = fabsf(fxj - fxi);
  const bool sure = ok && xi_ok && (fd < p.eps_lo || fd > p.eps_hi);
  if (__builtin_expect(sure, 1)) return fd < p.eps_lo;
  return within_exact(xj, xi, p.eps);
}

__device__ __noinline__ uint64_t add_rn(uint64_t a, uint64_t b) {
  bool ok = ((a | b) >> 63) == 0;
  uint64_t r = ok ? emu_add_pos(a, b, ok) : 0;
  if (ok) return r;
  return bits(__dadd_rn(dbl(a), dbl(b)));
}



__device__ __noinline__ double mul_hw(double a, double b) { return __dmul_rn(a, b); }


__device__ __noinline__ double div_hw(double a, double b) { return __ddiv_rn(a, b); }

// x' = a x + b (swx / sw), each operation correctly rounded, in this order.
// Once per row.  The division runs on the integer pipes (exact, with the
// hardware instruction for out-of-range operands); a and b that are powers
// of two (the model's 0.5) scale by their exponent, other values multiply on
// the FP64 pipe; the final addition is the hardware add.
__device__ __forceinline__ double finish(const OpinionArgs &p, double xi, uint64_t sw,
                                         uint64_t swx) {
  bool ok;
  const uint64_t m = emu_div_fast(swx, sw, ok);
  const double md = ok ? dbl(m) : div_hw(dbl(swx), dbl(sw));
  bool okl = false, okr = false;
  double l = 0.0, r = 0.0;
  if (p.a_pow2) l = dbl(emu_scale2(bits(xi), p.a_k, okl));
  if (!okl) l = mul_hw(p.a, xi);
  if (p.b_pow2) r = dbl(emu_scale2(bits(md), p.b_k, okr));
  if (!okr) r = mul_hw(p.b, md);
  return __dadd_rn(l, r);
}


// slots of a slice folded per pipeline step (see sell_slice)
constexpr uint32_t SELL_U = 2;

struct SellGroup {
  uint32_t j[SELL_U];
  double w[SELL_U], x[SELL_U];
};

struct SellCursor {
  const uint32_t *__restrict__ cs;
  const double *__restrict__ cw;
  uint32_t D;
  uint64_t pol;
  __device__ __forceinline__ void load(uint32_t g, SellGroup &G) const {
#pragma unroll
    for (uint32_t u = 0; u < SELL_U; u++) {
      const uint32_t q = g * SELL_U + u;
      const bool v = q < D;
      G.j[u] = v ? ld_stream(cs + 32ull * q, pol) : 0u;
      G.w[u] = v ? ld_stream(cw + 32ull * q, pol) : 0.0;
    }
  }
};

struct RowAcc {
  double sw, swx;
  uint32_t cnt;
};

template <bool GRID>
struct SliceCtx {
  const OpinionArgs &p;
  SellCursor cur;
  uint64_t pol_keep;
  double xi;
  float fxi;
  bool xi_ok;
  uint32_t d, G;

  __device__ __forceinline__ void gather(uint32_t g, SellGroup &N) const {
#pragma unroll
    for (uint32_t u = 0; u < SELL_U; u++)
      N.x[u] = g * SELL_U + u < cur.D ? ld_keep(p.x + N.j[u], pol_keep) : 0.0;
  }
  __device__ __forceinline__ void fold(uint32_t g, const SellGroup &C, RowAcc &a) const {
#pragma unroll
    for (uint32_t u = 0; u < SELL_U; u++) {
      const uint32_t q = g * SELL_U + u;
      if (q >= cur.D) break;  // warp-uniform: the slice's padding to a whole group
      const double wv = C.w[u], xj = C.x[u];
      const bool acc = q < d && within(xj, xi, fxi, xi_ok, p);
      bool ok;
      const uint64_t pk = GRID ? emu_mul_grid(bits(wv), bits(xj), ok)
                               : emu_mul_fast(bits(wv), bits(xj), ok);
      const double pkd = ok ? dbl(pk) : (acc ? mul_hw(wv, xj) : 0.0);
      if (acc) {  // predicated: a lane of a rejected edge skips both adds
        a.swx = __dadd_rn(a.swx, pkd);
        a.sw = __dadd_rn(a.sw, wv);
      }
      if (!GRID) a.cnt += acc;
    }
  }
  // one pipeline step: group g is folded while the opinions of group g + 1
  // and the sources and weights of group g + 2 are requested
  __device__ __forceinline__ void step(uint32_t g, const SellGroup &C, SellGroup &N,
                                       SellGroup &NN, RowAcc &a) const {
    gather(g + 1, N);
    cur.load(g + 2, NN);
    fold(g, C, a);
  }
};

// One slice of 32 rows of similar degree, lane l owning row order[32 s +
// l]: the lanes walk their rows' edges in insertion order in lock-step; the
// column-major slice layout makes every load of a source index or weight
// one coalesced 128 or 256-byte access.  Slots are taken in groups of
// SELL_U with a two-stage software pipeline over three rotating buffers
// (while group g is folded, the opinions of group g + 1 and the sources and
// weights of group g + 2 are in flight).  The two additions of an edge are
// predicated on its test: the FP64 pipe takes a warp instruction whatever
// its active lanes, so this costs the pipe what a branch-free +0 would and
// saves the selects.
template <bool GRID>
__device__ __forceinline__ void sell_slice(const OpinionArgs &p, uint64_t sl) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t pos = sl * 32 + lane;
  const bool live = pos < p.norder;
  // the row and its degree are independent loads (the degree is stored by
  // position, not read through the row pointers)
  const uint32_t r = live ? p.order[pos] : 0u;
  const uint32_t d = live ? p.order_deg[pos] : 0u;
  const double xi = live ? p.x[r] : 0.0;
  bool xi_ok;
  const float fxi = hi_float(xi, xi_ok);
  SellCursor cur{p.sell_src + p.slice_base[sl] + lane, p.sell_w + p.slice_base[sl] + lane,
                 p.slice_deg[sl], policy_evict_first()};
  const SliceCtx<GRID> c{p, cur, policy_evict_last(), xi, fxi, xi_ok, d,
                         (cur.D + SELL_U - 1) / SELL_U};
  RowAcc a{0.0, 0.0, 0};
  SellGroup X, Y, Z;
  cur.load(0, X);
  c.gather(0, X);
  cur.load(1, Y);
  for (uint32_t g = 0; g < c.G; g += 3) {
    c.step(g, X, Y, Z, a);
    if (g + 1 >= c.G) break;
    c.step(g + 1, Y, Z, X, a);
    if (g + 2 >= c.G) break;
    c.step(g + 2, Z, X, Y, a);
  }
  if (!live) return;
  // some neighbour qualified: grid weights are positive, so sw > 0 says it
  const bool any = GRID ? bits(a.sw) != 0 : a.cnt != 0;
  p.xo[r] = any ? finish(p, xi, bits(a.sw), bits(a.swx)) : xi;
}

// One warp per hub row (degree > hub_thr): lane l folds edges l, l + 32,
// l + 64, ... in order (coalesced loads), the 32 lane sums are combined in a
// fixed tree.
template <bool GRID>
__device__ __forceinline__ void hub_warp(const OpinionArgs &p, uint32_t r) {
  const unsigned lane = threadIdx.x & 31;
  double xi = p.x[r];
  bool xi_ok;
  float fxi = hi_float(xi, xi_ok);
  const uint32_t b = p.rp[r], e = p.rp[r + 1];
  double dsw = 0.0, dswx = 0.0;
  uint32_t cnt = 0;
  constexpr int U = 4;
  const uint64_t pol_stream = policy_evict_first(), pol_keep = policy_evict_last();
  for (uint32_t k0 = b; k0 < e; k0 += 32 * U) {
    uint32_t jv[U];
    double wv[U], xv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const uint32_t k = k0 + u * 32 + lane;
      const bool valid = k < e;
      jv[u] = valid ? ld_stream(p.src + k, pol_stream) : 0xffffffffu;
      wv[u] = valid ? ld_stream(p.w + k, pol_stream) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; u++)
      xv[u] = jv[u] != 0xffffffffu ? ld_keep(p.x + jv[u], pol_keep) : 0.0;
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (jv[u] != 0xffffffffu && within(xv[u], xi, fxi, xi_ok, p)) {
        bool ok;
        const uint64_t pk = GRID ? emu_mul_grid(bits(wv[u]), bits(xv[u]), ok)
                                 : emu_mul_fast(bits(wv[u]), bits(xv[u]), ok);
        dswx = __dadd_rn(dswx, ok ? dbl(pk) : mul_hw(wv[u], xv[u]));
        dsw = __dadd_rn(dsw, wv[u]);
        cnt++;
      }
    }
  }
  uint64_t sw = bits(dsw);
  uint64_t swx = bits(dswx);
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
  if (lane == 0) p.xo[r] = cnt ? finish(p, xi, sw, swx) : xi;
}

// One block per hub row above HUB_BLOCK_DEGREE in-edges.  The row's source
// indices and weights are staged through shared memory in chunks of
// HB_CHUNK edges by 1-D bulk copies (cp.async.bulk, completion counted in
// bytes on an mbarrier), two chunks in flight; thread t folds the chunk
// positions t, t + 128, ... and the 128 partial sums are combined in a
// fixed tree (warps as in hub_warp, then warps 0+1, 2+3, and the two
// halves), so the result is the same on every run and within 1e-12 of the
// sequential fold.  Bulk copies need 16-byte aligned starts and sizes: the
// chunks start at the row's first edge rounded down to a multiple of 4
// (edges of the previous row are skipped) and end at its last edge rounded
// down; the at most 3 edges after that are read directly.  Every wait is
// bounded: on a timeout the block records an error in the status word,
// waits (bounded) for its copies in flight and leaves the row unwritten.
constexpr uint32_t HB_CHUNK = 512;  // edges per stage, a multiple of 4
constexpr uint32_t HB_SPIN_LIMIT = 1u << 20;
constexpr int HB_ERR_WAIT = 0x5e03;

struct HubStage {
  uint32_t src[HB_CHUNK];
  double w[HB_CHUNK];
};

__device__ __forceinline__ uint32_t smem_u32(const void *q) {
  return (uint32_t)__cvta_generic_to_shared(q);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// bounded wait for the phase with the given parity; false on a timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < HB_SPIN_LIMIT; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes,
                                          uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

struct HubShared {
  HubStage stage[2];
  uint64_t bar[2];
  uint64_t part_sw[TPB / 32], part_swx[TPB / 32];
  uint32_t part_cnt[TPB / 32];
  int failed;
};
// one copy per kernel, whichever weight form its blocks instantiate
__device__ __forceinline__ HubShared &hub_shared() {
  __shared__ __align__(16) HubShared h;
  return h;
}

template <bool GRID>
__device__ __noinline__ void hub_block(const OpinionArgs &p, uint32_t r) {
  HubShared &H = hub_shared();
  HubStage *stage = H.stage;
  uint64_t *bar = H.bar;
  uint64_t *part_sw = H.part_sw, *part_swx = H.part_swx;
  uint32_t *part_cnt = H.part_cnt;
  int &failed = H.failed;
  const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const double xi = p.x[r];
  bool xi_ok;
  const float fxi = hi_float(xi, xi_ok);
  const uint32_t b = p.rp[r], e = p.rp[r + 1];
  const uint32_t a0 = b & ~3u, e_al = e & ~3u;
  const uint32_t nch = e_al > a0 ? (e_al - a0 + HB_CHUNK - 1) / HB_CHUNK : 0;
  const uint64_t pol_keep = policy_evict_last();
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](uint32_t k) {  // chunk k into stage k & 1 (thread 0)
    const uint32_t c0 = a0 + k * HB_CHUNK;
    const uint32_t c1 = c0 + HB_CHUNK < e_al ? c0 + HB_CHUNK : e_al;
    const uint32_t m = c1 - c0;  // a multiple of 4
    HubStage &S = stage[k & 1];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bar[k & 1], m * 12u);
    bulk_copy(S.src, p.src + c0, m * 4u, &bar[k & 1]);
    bulk_copy(S.w, p.w + c0, m * 8u, &bar[k & 1]);
  };
  if (tid == 0) {
    if (nch > 0) issue(0);
    if (nch > 1) issue(1);
  }
  double dsw = 0.0, dswx = 0.0;
  uint32_t cnt = 0;
  auto fold_x = [&](double xj, double wv) {
    if (within(xj, xi, fxi, xi_ok, p)) {
      bool ok;
      const uint64_t pk = GRID ? emu_mul_grid(bits(wv), bits(xj), ok)
                               : emu_mul_fast(bits(wv), bits(xj), ok);
      dswx = __dadd_rn(dswx, ok ? dbl(pk) : mul_hw(wv, xj));
      dsw = __dadd_rn(dsw, wv);
      cnt++;
    }
  };
  uint32_t k = 0;
  for (; k < nch; k++) {
    if (!mbar_wait(&bar[k & 1], (k >> 1) & 1u)) {
      atomicCAS(p.status, 0, HB_ERR_WAIT);
      failed = 1;
    }
    __syncthreads();
    if (failed) break;
    const uint32_t c0 = a0 + k * HB_CHUNK;
    const uint32_t c1 = c0 + HB_CHUNK < e_al ? c0 + HB_CHUNK : e_al;
    const HubStage &S = stage[k & 1];
    // the thread's HB_CHUNK / TPB positions: opinions requested together
    constexpr uint32_t PER = HB_CHUNK / TPB;
    uint32_t jv[PER];
    double wv[PER], xv[PER];
    bool use[PER];
#pragma unroll
    for (uint32_t u = 0; u < PER; u++) {
      const uint32_t i = tid + u * TPB;
      use[u] = i < c1 - c0 && c0 + i >= b;
      jv[u] = use[u] ? S.src[i] : 0u;
      wv[u] = use[u] ? S.w[i] : 0.0;
    }
#pragma unroll
    for (uint32_t u = 0; u < PER; u++) xv[u] = use[u] ? ld_keep(p.x + jv[u], pol_keep) : 0.0;
#pragma unroll
    for (uint32_t u = 0; u < PER; u++)
      if (use[u]) fold_x(xv[u], wv[u]);
    __syncthreads();  // stage k & 1 is read
    if (tid == 0 && k + 2 < nch) issue(k + 2);
  }
  if (failed) {  // let the copies still in flight (chunks k, k + 1) land before leaving
    for (uint32_t j = k; j < nch && j < k + 2; j++) mbar_wait(&bar[j & 1], (j >> 1) & 1u);
    return;
  }
  // the edges after the last bulk copy (fewer than 4)
  const uint32_t t0 = e_al > b ? e_al : b;
  if (t0 + tid < e) fold_x(ld_keep(p.x + p.src[t0 + tid], pol_keep), p.w[t0 + tid]);
  // fixed tree: within each warp (lane l receives lane l + off), then warps
  uint64_t sw = bits(dsw), swx = bits(dswx);
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint64_t osw = __shfl_down_sync(0xffffffffu, sw, off);
    const uint64_t oswx = __shfl_down_sync(0xffffffffu, swx, off);
    const uint32_t ocnt = __shfl_down_sync(0xffffffffu, cnt, off);
    if ((lane & (2 * off - 1)) == 0 && ocnt) {
      sw = add_rn(sw, osw);
      swx = add_rn(swx, oswx);
      cnt += ocnt;
    }
  }
  if (lane == 0) {
    part_sw[wid] = sw;
    part_swx[wid] = swx;
    part_cnt[wid] = cnt;
  }
  __syncthreads();
  if (tid == 0) {
    uint64_t s2[2], x2[2];
    uint32_t c2[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      s2[h] = part_sw[2 * h];
      x2[h] = part_swx[2 * h];
      c2[h] = part_cnt[2 * h];
      if (part_cnt[2 * h + 1]) {
        s2[h] = add_rn(s2[h], part_sw[2 * h + 1]);
        x2[h] = add_rn(x2[h], part_swx[2 * h + 1]);
        c2[h] += part_cnt[2 * h + 1];
      }
    }
    if (c2[1]) {
      s2[0] = add_rn(s2[0], s2[1]);
      x2[0] = add_rn(x2[0], x2[1]);
      c2[0] += c2[1];
    }
    p.xo[r] = c2[0] ? finish(p, xi, s2[0], x2[0]) : xi;
    mbar_inval(&bar[0]);
    mbar_inval(&bar[1]);
  }
}

// The work of one block of the gather grid: hub warps, then slices (one
// per warp).  Shared by the single-simulation kernel and the multi-job
// kernel of the serving loop.
// BIG: the block range starts with the block-wide hub rows; otherwise they
// are run by their own launch (k_opinion_big) and the range starts at the
// warp hubs, so that this kernel needs no shared memory (its L1 keeps the
// whole unified array).
template <bool GRID, bool BIG>
__device__ __forceinline__ void opinion_block(const OpinionArgs &p, unsigned blk) {
  if (BIG) {
    if (blk < p.nbig) {  // block-wide hub rows (whole blocks: the test is uniform)
      hub_block<GRID>(p, p.hub_rows[blk]);
      return;
    }
    blk -= (unsigned)p.nbig;
  }
  const uint64_t warp = (uint64_t)blk * (TPB / 32) + (threadIdx.x >> 5);
  if (blk < p.hub_blocks) {
    if (p.nbig + warp < p.nhub) hub_warp<GRID>(p, p.hub_rows[p.nbig + warp]);
    return;
  }
  const uint64_t sl = warp - (uint64_t)p.hub_blocks * (TPB / 32);
  if (sl < p.nslices) sell_slice<GRID>(p, sl);
}

template <bool GRID>
__global__ void __launch_bounds__(TPB, 9) k_opinion(OpinionArgs p) {
  opinion_block<GRID, false>(p, blockIdx.x);
}

// Completion reports of one gather launch (apply! with host exchange): the
// launch is k_opinion's (the same blocks, the same work); the hub warps'
// blocks form range `nranges`, slice blocks below end[k] (and not below
// end[k - 1]) range k.  A block reports once its rows are stored: after the
// block barrier its first thread fences (GPU scope, cumulative over the
// block's stores) and adds 1 to its range's counter; the block that
// completes a range makes the range visible system-wide and writes the
// call's generation to the range's flag in mapped host memory.
constexpr unsigned XCHG_RANGES = 16;
struct Notify {
  unsigned *count;  // device: blocks finished per range
  unsigned *flag;   // mapped host memory: generation of the finished range
  unsigned gen, nranges, hub_blocks;
  unsigned end[XCHG_RANGES];         // launch blocks: range k ends before end[k]
  unsigned expect[XCHG_RANGES + 1];  // blocks per range
};

template <bool GRID>
__global__ void __launch_bounds__(TPB, 9) k_opinion_notify(OpinionArgs p, Notify nt) {
  opinion_block<GRID, false>(p, blockIdx.x);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned b = blockIdx.x;
    unsigned r = nt.nranges;  // the hub warps
    if (b >= nt.hub_blocks) {
      r = 0;
      while (r + 1 < nt.nranges && b >= nt.end[r]) r++;
    }
    if (atomicAdd(nt.count + r, 1u) + 1 == nt.expect[r]) {
      __threadfence_system();
      *(volatile unsigned *)(nt.flag + r) = nt.gen;
    }
  }
}

// the block-wide hub rows of one simulation, one block each
template <bool GRID>
__global__ void __launch_bounds__(TPB) k_opinion_big(OpinionArgs p) {
  hub_block<GRID>(p, p.hub_rows[blockIdx.x]);
}

// Many simulations in one launch: block i runs virtual block tiles[i].blk of
// job tiles[i].job -- the same work, in the same order, as that job's own
// launch of k_opinion.  Jobs run no block-wide hub rows (the caller checks),
// so the kernel carries no shared-memory staging and every block keeps the
// whole unified L1/shared array for the opinion gathers.
struct JobTile {
  uint32_t job, blk;
};

__global__ void __launch_bounds__(TPB, 9) k_opinion_jobs(const OpinionArgs *jobs,
                                                      const JobTile *tiles) {
  __shared__ OpinionArgs sp;
  JobTile t = tiles[blockIdx.x];
  if (threadIdx.x == 0) sp = jobs[t.job];
  __syncthreads();
  if (sp.grid) opinion_block<true, false>(sp, t.blk);
  else opinion_block<false, false>(sp, t.blk);
}


// every weight a multiple of 2^-53 in (0, 1]?
__global__ void k_check_grid(const double *w, uint64_t n, int *bad) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t wb = bits(w[i]);
    uint32_t ew = (uint32_t)(wb >> 52);
    bool ok = (wb >> 63) == 0 && ew >= 970u && ew <= 1023u && (ew < 1023u || (wb & EMU_M52) == 0);
    if (ok && ew < 1022u) {
      uint64_t m = (wb & EMU_M52) | EMU_H53;
      ok = (m & ((1ull << (1022u - ew)) - 1ull)) == 0;
    }
    if (!ok) atomicExch(bad, 1);
  }
}

}  // namespace

static unsigned opinion_args(Sim &s, int e, int T, double eps, double a, double b,
                             uint32_t thr, uint32_t big_thr, OpinionArgs &p,
                             cudaStream_t launch_stream);
// a gather launch whose finished row ranges are downloaded while it runs
// (apply! with host exchange)
static void launch_notified(Sim &s, OpinionArgs &p, unsigned grid, Sim::HostExchange &hx);

// apply!(sim, bounded_confidence, [T], [T, E], [T]; params = [E, eps, a, b,
// hub_thr, block_thr]); defaults eps 0.3, a 0.5, b 1 - a, hub_thr 1536,
// block_thr none (hub rows above block_thr take a whole block each).
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
  double thr_d = c.param(4, OPINION_HUB_DEFAULT);
  uint32_t thr = thr_d >= 4294967295.0 ? 0xffffffffu : (uint32_t)thr_d;
  // rows above this many in-edges take a whole block (default: none)
  double big_d = c.param(5, 4294967295.0);
  uint32_t big_thr = big_d >= 4294967295.0 ? 0xffffffffu : (uint32_t)big_d;
  OpinionArgs p{};
  unsigned grid = opinion_args(s, e, c.call_type, eps, a, b, thr, big_thr, p, s.stream);
  if (!grid) return;
  // block-wide hubs (only with a block threshold) by their own launch, then
  // the rest: the two write disjoint rows and read only the old opinions
  const unsigned nbig = (unsigned)p.nbig;
  if (nbig) {
    if (p.grid) k_opinion_big<true><<<nbig, TPB, 0, s.stream>>>(p);
    else k_opinion_big<false><<<nbig, TPB, 0, s.stream>>>(p);
  }
  Sim::HostExchange *hx = s.host_xchg;
  if (hx && hx->type_nr == c.call_type && ad.fields.size() == 1 && hx->out && hx->out[0] &&
      nbig == 0 && grid > 0) {
    launch_notified(s, p, grid, *hx);
    return;
  }
  if (grid > nbig) {
    if (p.grid) k_opinion<true><<<grid - nbig, TPB, 0, s.stream>>>(p);
    else k_opinion<false><<<grid - nbig, TPB, 0, s.stream>>>(p);
  }
  VG_CUDA(cudaGetLastError());
}

// Row ranges of the gather: range k is the launch blocks [range_block[k],
// range_block[k + 1]) (equal shares of the slice blocks); the rows are
// sorted by window (row >> wshift) before degree, so once range k is done
// every non-hub row of the windows below the window of range k + 1's first
// row is final: range_rows[k] = that window << wshift.  hub_rows_sorted:
// the hub rows.
static void range_bounds(Sim &s, CSR &cs, uint64_t n, unsigned hub_blocks, unsigned slice_blocks) {
  if (!cs.range_block.empty() && cs.range_block.back() == hub_blocks + (uint64_t)slice_blocks)
    return;
  const unsigned K = std::max(1u, std::min(XCHG_RANGES, slice_blocks));
  cs.range_block.assign(K + 1, 0);
  cs.range_rows.assign(K, n);
  cs.range_window.assign(K, 0xFFFFFFFFu);
  cs.range_window[0] = 0;
  for (unsigned k = 0; k <= K; k++)
    cs.range_block[k] = hub_blocks + (uint64_t)slice_blocks * k / K;
  for (unsigned k = 0; k + 1 < K; k++) {
    // first position in `order` of the range's first block (TPB / 32
    // slices of 32 rows per block)
    const uint64_t pos = (cs.range_block[k + 1] - hub_blocks) * TPB;
    if (pos >= cs.norder) continue;
    uint32_t row = 0;
    VG_CUDA(cudaMemcpyAsync(&row, cs.order.as<uint32_t>() + pos, 4, cudaMemcpyDeviceToHost,
                            s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    cs.range_window[k + 1] = row >> cs.wshift;
    cs.range_rows[k] = std::min<uint64_t>(n, ((uint64_t)row >> cs.wshift) << cs.wshift);
  }
  cs.hub_rows_sorted.assign(cs.nhub, 0);
  if (cs.nhub) {
    VG_CUDA(cudaMemcpyAsync(cs.hub_rows_sorted.data(), cs.hub_rows.p, cs.nhub * 4,
                            cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    std::sort(cs.hub_rows_sorted.begin(), cs.hub_rows_sorted.end());
  }
}

// The gather as one launch (its load balance intact: the long rows start
// first and overlap the rest) that reports each finished row range to the
// host; the host issues the range's download on the copy stream as soon as
// its flag (and, for a range holding hub rows, the hub warps' flag) shows
// this call's generation.  No GPU work waits on another: the host polls,
// and if the launch ends without a report (or fails) the remaining ranges
// are downloaded after it, so the wait is bounded by the launch itself.
static void launch_notified(Sim &s, OpinionArgs &p, unsigned grid, Sim::HostExchange &hx) {
  CSR &cs = *p.csr;
  const unsigned slice_blocks = grid - p.hub_blocks;
  range_bounds(s, cs, p.n, p.hub_blocks, slice_blocks);
  const unsigned K = (unsigned)cs.range_rows.size();
  if (!s.copy_stream) VG_CUDA(cudaStreamCreateWithFlags(&s.copy_stream, cudaStreamNonBlocking));
  if (!s.xchg_flags_host) {
    void *h = nullptr, *d = nullptr;
    VG_CUDA(cudaHostAlloc(&h, (XCHG_RANGES + 1) * 4, cudaHostAllocMapped));
    std::memset(h, 0, (XCHG_RANGES + 1) * 4);
    VG_CUDA(cudaHostGetDevicePointer(&d, h, 0));
    s.xchg_flags_host = (unsigned *)h;
    s.xchg_flags_dev = (unsigned *)d;
    s.xchg_count.alloc((XCHG_RANGES + 1) * 4, &s.footprint);
  }
  if (++s.xchg_gen == 0) s.xchg_gen = 1;
  Notify nt{};
  nt.count = s.xchg_count.as<unsigned>();
  nt.flag = s.xchg_flags_dev;
  nt.gen = s.xchg_gen;
  nt.nranges = K;
  nt.hub_blocks = p.hub_blocks;
  for (unsigned k = 0; k < K; k++) {
    nt.end[k] = (unsigned)cs.range_block[k + 1];
    nt.expect[k] = (unsigned)(cs.range_block[k + 1] - cs.range_block[k]);
  }
  nt.expect[K] = p.hub_blocks;
  VG_CUDA(cudaMemsetAsync(nt.count, 0, (K + 1) * 4, s.stream));
  if (p.grid) k_opinion_notify<true><<<grid, TPB, 0, s.stream>>>(p, nt);
  else k_opinion_notify<false><<<grid, TPB, 0, s.stream>>>(p, nt);
  VG_CUDA(cudaGetLastError());

  const uint64_t n = std::min<uint64_t>(hx.n, p.n);
  double *out = (double *)hx.out[0];
  // rows [lo[k], hi[k]) are the windows from range k's first window up to
  // range k + 1's; a window's rows may also sit in earlier ranges (a window
  // can straddle a boundary), so the download waits for ranges first[k]..k,
  // first[k] being the first range that reaches range k's first window
  std::vector<uint64_t> lo(K), hi(K);
  std::vector<unsigned> first(K);
  std::vector<char> needs_hubs(K), issued(K, 0);
  uint64_t prev = 0;
  for (unsigned k = 0; k < K; k++) {
    lo[k] = prev;
    hi[k] = std::max(prev, k + 1 == K ? n : std::min(n, cs.range_rows[k]));
    auto it = std::lower_bound(cs.hub_rows_sorted.begin(), cs.hub_rows_sorted.end(),
                               (uint32_t)lo[k]);
    needs_hubs[k] = p.hub_blocks && it != cs.hub_rows_sorted.end() && *it < hi[k];
    unsigned j = 0;
    while (j < k && (j + 1 < K ? cs.range_window[j + 1] : 0xFFFFFFFFu) < cs.range_window[k]) j++;
    first[k] = j;
    prev = hi[k];
  }
  volatile unsigned *flag = s.xchg_flags_host;
  auto issue = [&](unsigned k) {
    if (hi[k] > lo[k])
      VG_CUDA(cudaMemcpyAsync(out + lo[k], p.xo + lo[k], (hi[k] - lo[k]) * 8,
                              cudaMemcpyDeviceToHost, s.copy_stream));
    issued[k] = 1;
  };
  unsigned left = K;
  for (uint64_t poll = 0; left; poll++) {
    const bool hubs_done = p.hub_blocks == 0 || flag[K] == nt.gen;
    for (unsigned k = 0; k < K; k++) {
      if (issued[k] || (needs_hubs[k] && !hubs_done)) continue;
      bool ready = true;
      for (unsigned j = first[k]; j <= k && ready; j++) ready = flag[j] == nt.gen;
      if (ready) {
        issue(k);
        left--;
      }
    }
    if (left && (poll & 255) == 255 && cudaStreamQuery(s.stream) != cudaErrorNotReady) break;
  }
  if (left) {  // the launch ended (or failed) without reporting every range
    VG_CUDA(cudaStreamSynchronize(s.stream));
    for (unsigned k = 0; k < K; k++)
      if (!issued[k]) issue(k);
  }
  hx.done = true;
}

// arguments and grid size of one simulation's gather launch; 0 when there
// is nothing to launch (no agents, or no edges: then x' = x, copied here on
// the stream the launch would use)
static unsigned opinion_args(Sim &s, int e, int T, double eps, double a, double b,
                             uint32_t thr, uint32_t big_thr, OpinionArgs &p,
                             cudaStream_t launch_stream) {
  EdgeStore &es = s.edges[e];
  DevCSRView v = csr_view(s, e, T);
  if (v.nedges && v.src_type_const != T)
    fail(VG_ERR_ARG, "bounded_confidence: sources must be of the called type");
  DevAgentView av = agent_view(s, T);
  if (av.n == 0) return 0;
  p = OpinionArgs{};
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
  auto pow2 = [](double v, int &k) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    const int ev = (int)(u >> 52);
    k = ev - 1023;
    return (u & EMU_M52) == 0 && ev >= 1 && ev <= 2046;  // positive, normal, no fraction bits
  };
  p.a_pow2 = pow2(a, p.a_k);
  p.b_pow2 = pow2(b, p.b_k);
  p.hub_thr = thr;
  if (!v.nedges || T >= (int)es.csr.size() || !v.row_ptr) {
    VG_CUDA(cudaMemcpyAsync(p.xo, p.x, av.n * 8, cudaMemcpyDeviceToDevice, launch_stream));
    return 0;
  }
  CSR &cs = es.csr[T];
  if (cs.unit_grid_weights < 0) {
    int *bad = nullptr;
    VG_CUDA(cudaMallocAsync((void **)&bad, 4, s.stream));
    VG_CUDA(cudaMemsetAsync(bad, 0, 4, s.stream));
    k_check_grid<<<1024, TPB, 0, s.stream>>>(p.w, v.nedges, bad);
    int h = 0;
    VG_CUDA(cudaMemcpyAsync(&h, bad, 4, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaFreeAsync(bad, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    cs.unit_grid_weights = h ? 0 : 1;
  }
  p.grid = cs.unit_grid_weights;
  ensure_schedule(s, cs, thr, big_thr, av.n);
  p.hub_rows = cs.hub_rows.as<uint32_t>();
  p.nhub = cs.nhub;
  p.nbig = cs.nbig;
  p.status = s.d_status.as<int>();
  p.order = cs.order.as<uint32_t>();
  p.order_deg = cs.order_deg.as<uint32_t>();
  p.norder = cs.norder;
  p.slice_base = cs.slice_base.as<uint64_t>();
  p.slice_deg = cs.slice_deg.as<uint32_t>();
  p.sell_src = cs.sell_src.as<uint32_t>();
  p.sell_w = cs.sell_w.as<double>();
  p.nslices = cs.nslices;
  p.hub_blocks = (unsigned)((cs.nhub - cs.nbig + (TPB / 32) - 1) / (TPB / 32));
  p.csr = &cs;
  return (unsigned)cs.nbig + p.hub_blocks + (unsigned)((cs.nslices + (TPB / 32) - 1) / (TPB / 32));
}

// Builds what a job's launches need ahead of its first step (the weight
// check and the gather layout), on the simulation's own stream.
void prepare_opinion_job(const OpinionJob &j) {
  OpinionArgs p{};
  DevCSRView v = csr_view(*j.sim, j.edge_type, j.type_nr);
  if (v.nedges == 0) return;  // nothing to prepare (and no copy to queue)
  opinion_args(*j.sim, j.edge_type, j.type_nr, j.eps, j.a, j.b, j.hub_thr, j.block_thr, p,
               j.sim->stream);
  VG_CUDA(cudaStreamSynchronize(j.sim->stream));
}

// One launch for the bounded-confidence step of many simulations (the
// serving loop's continuous batching).  Each job's blocks do exactly what
// its own launch would; the caller finishes each job's transition.
void launch_opinion_jobs(const std::vector<OpinionJob> &jobs, cudaStream_t st, DevBuf &args_buf,
                         DevBuf &tiles_buf, uint64_t *fp) {
  std::vector<OpinionArgs> args;
  std::vector<JobTile> tiles;
  for (size_t j = 0; j < jobs.size(); j++) {
    OpinionArgs p{};
    unsigned g = opinion_args(*jobs[j].sim, jobs[j].edge_type, jobs[j].type_nr, jobs[j].eps,
                              jobs[j].a, jobs[j].b, jobs[j].hub_thr, jobs[j].block_thr, p, st);
    if (p.nbig)
      fail(VG_ERR_ARG, "the multi-job gather runs no block-wide hub rows (block threshold)");
    args.push_back(p);
    for (unsigned k = 0; k < g; k++) tiles.push_back({(uint32_t)j, k});
  }
  if (tiles.empty()) return;
  if (args_buf.bytes < args.size() * sizeof(OpinionArgs))
    args_buf.alloc(args.size() * sizeof(OpinionArgs) * 2, fp);
  if (tiles_buf.bytes < tiles.size() * sizeof(JobTile))
    tiles_buf.alloc(tiles.size() * sizeof(JobTile) * 2, fp);
  VG_CUDA(cudaMemcpyAsync(args_buf.p, args.data(), args.size() * sizeof(OpinionArgs),
                          cudaMemcpyHostToDevice, st));
  VG_CUDA(cudaMemcpyAsync(tiles_buf.p, tiles.data(), tiles.size() * sizeof(JobTile),
                          cudaMemcpyHostToDevice, st));
  k_opinion_jobs<<<(unsigned)tiles.size(), TPB, 0, st>>>(args_buf.as<OpinionArgs>(),
                                                        tiles_buf.as<JobTile>());
  VG_CUDA(cudaGetLastError());
  // no wait: a copy from pageable host memory is staged before the call
  // returns, so the host vectors may go; the device buffers are rewritten by
  // the next call's copies in stream order, after this launch
}

}  // namespace vg
