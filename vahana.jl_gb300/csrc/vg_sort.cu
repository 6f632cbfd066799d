// Device primitives: exclusive scan and a stable LSD radix sort of
// (key, value) pairs.  Both are the building blocks of the CSR
// (re)construction that reproduces Vahana's per-target `push!` order
// (src/EdgeMethods.jl:495-496): records arrive in insertion order (or carry
// an order key), and a stable sort by target row keeps that order inside
// each row.
#include <algorithm>
#include <numeric>
#include <vector>

#include "vg_internal.h"

namespace vg {

int bits_for(uint64_t maxval) {
  int b = 0;
  while (b < 64 && (maxval >> b)) b++;
  return b;
}

namespace {

constexpr int SCAN_TPB = 256;
constexpr int SCAN_IPT = 16;
constexpr int SCAN_CHUNK = SCAN_TPB * SCAN_IPT;

template <class T>
__device__ T block_exclusive_scan(T v, T *warp_sums, T *block_total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  if (w == 0) {
    T s = lane < nw ? warp_sums[lane] : T(0);
    T incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane < nw) warp_sums[lane] = incl - s;
    if (lane == 31 && block_total) *block_total = incl;
  }
  __syncthreads();
  T r = warp_sums[w] + x - v;
  __syncthreads();
  return r;
}

// The scan of at most one tile (SCAN_CHUNK items) in a single block, plus
// an optional per-block prefix.  Each thread owns SCAN_IPT consecutive
// items; safe in place.
template <class T>
__global__ void scan_apply(const T *in, T *out, uint64_t n, const T *prefix) {
  __shared__ T ws[32];
  uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK +
                  (uint64_t)threadIdx.x * SCAN_IPT;
  T v[SCAN_IPT];
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    uint64_t i = base + k;
    v[k] = i < n ? in[i] : T(0);
    s += v[k];
  }
  T run = block_exclusive_scan<T>(s, ws, (T *)nullptr);
  if (prefix) run += prefix[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    uint64_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

// Single-pass exclusive scan over tiles of SCAN_CHUNK items with decoupled
// look-back (D. Merrill and M. Garland, NVR-2016-002): a tile publishes its
// total, then warp 0 reads the flags of the 32 preceding tiles at once and
// adds totals back to the nearest tile whose inclusive prefix is known.
// Tiles take their index from a ticket counter in start order (a tile only
// waits for running tiles); every wait is bounded and records an error in
// *err when it gives up.  In place is allowed (a tile reads all its items
// before it writes).
constexpr uint32_t SCAN_SPIN_LIMIT = 1u << 21;
constexpr int SCAN_ERR_LOOKBACK = 0x5e02;

__device__ __forceinline__ void st_release_u32(uint32_t *a, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *a) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *a) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *a) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
  return v;
}

template <class T>
struct ScanState {
  uint32_t *flag;  // per tile: 0 nothing, 1 total in agg, 2 inclusive prefix in pre
  T *agg, *pre;
  uint32_t *ticket;
};

template <class T>
__global__ void __launch_bounds__(SCAN_TPB) scan_lookback(const T *in, T *out, uint64_t n,
                                                          ScanState<T> S, int *err) {
  __shared__ T ws[32];
  __shared__ T s_tot, s_excl;
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(S.ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t base = (uint64_t)tile * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_IPT;
  T v[SCAN_IPT];
  T sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    const uint64_t i = base + k;
    v[k] = i < n ? in[i] : T(0);
    sum += v[k];
  }
  T run = block_exclusive_scan<T>(sum, ws, &s_tot);
  if (threadIdx.x < 32) {
    const uint32_t lane = threadIdx.x;
    const T total = s_tot;
    T excl = 0;
    if (tile == 0) {
      if (lane == 0) {
        S.pre[0] = total;
        st_release_u32(S.flag, 2u);
      }
    } else {
      if (lane == 0) {
        S.agg[tile] = total;
        st_release_u32(S.flag + tile, 1u);
      }
      int64_t t = (int64_t)tile - 1;
      uint32_t spins = 0;
      for (;;) {
        const int64_t tt = t - (int64_t)lane;
        const uint32_t f = tt >= 0 ? ld_acquire_u32(S.flag + tt) : 2u;
        const unsigned pm = __ballot_sync(0xffffffffu, f == 2u);
        const unsigned zm = __ballot_sync(0xffffffffu, f == 0u);
        const int P = pm ? __ffs(pm) - 1 : 32;  // nearest predecessor with a prefix
        const unsigned need = P == 32 ? 0xffffffffu : (2u << P) - 1u;
        if (zm & need) {  // a tile in between has published nothing yet
          if (++spins > SCAN_SPIN_LIMIT) {
            if (lane == 0) atomicCAS(err, 0, SCAN_ERR_LOOKBACK);
            break;
          }
          if (spins > 16) __nanosleep(64);
          continue;
        }
        T x = 0;
        if ((int)lane < P) x = ld_relaxed(S.agg + tt);
        else if ((int)lane == P && tt >= 0) x = ld_relaxed(S.pre + tt);
#pragma unroll
        for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        excl += x;
        if (P < 32) break;
        t -= 32;
        spins = 0;
      }
      if (lane == 0) {
        S.pre[tile] = excl + total;
        st_release_u32(S.flag + tile, 2u);
      }
    }
    if (lane == 0) s_excl = excl;
  }
  __syncthreads();
  run += s_excl;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    const uint64_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

template <class T>
uint64_t scan_scratch_bytes(uint64_t n) {
  const uint64_t nt = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  return 64 + nt * 4 + 2 * nt * sizeof(T) + 64;
}

// scratch: null (allocated on the stream) or scan_scratch_bytes<T>(n) bytes
template <class T>
void exclusive_scan_impl(const T *in, T *out, uint64_t n, cudaStream_t st, int *err,
                         void *scratch = nullptr) {
  if (n == 0) return;
  const uint64_t nt = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if (nt == 1) {
    scan_apply<T><<<1, SCAN_TPB, 0, st>>>(in, out, n, nullptr);
    VG_CUDA(cudaGetLastError());
    return;
  }
  if (nt >= (1ull << 31)) fail(VG_ERR_NOMEM, "scan: too many items");
  char *buf = (char *)scratch;
  const uint64_t bytes = scan_scratch_bytes<T>(n);
  if (!buf) VG_CUDA(cudaMallocAsync((void **)&buf, bytes, st));
  ScanState<T> S;
  S.ticket = (uint32_t *)buf;
  S.flag = (uint32_t *)(buf + 64);
  const uint64_t aoff = (64 + nt * 4 + 15) & ~15ull;
  S.agg = (T *)(buf + aoff);
  S.pre = S.agg + nt;
  VG_CUDA(cudaMemsetAsync(buf, 0, 64 + nt * 4, st));
  scan_lookback<T><<<(unsigned)nt, SCAN_TPB, 0, st>>>(in, out, n, S, err);
  VG_CUDA(cudaGetLastError());
  if (!scratch) VG_CUDA(cudaFreeAsync(buf, st));
}

// ------------------------------------------------------------ radix sort
// LSD radix sort with 8-bit digits in one launch per digit: the digit
// counts of every pass come from one upfront read of the keys, and each
// pass ranks its tiles locally and finds the tile's offset for every digit
// by a chained scan with decoupled look-back over the tiles' published
// counts (D. Merrill and M. Garland, "Single-pass parallel prefix scan with
// decoupled look-back", NVIDIA NVR-2016-002; A. Adinets and D. Merrill,
// "Onesweep: a faster least significant digit radix sort for GPUs",
// arXiv:2206.01784, 2022).  Tiles take their index from a counter in the
// order the blocks start, so a tile only waits for tiles that are already
// running.
constexpr int RS_TPB = 1024;                       // threads of a pass tile
constexpr int RS_WARPS = RS_TPB / 32;
constexpr int RS_IPT = 8;                          // items per lane
constexpr int RS_WARP_ITEMS = 32 * RS_IPT;         // 256
constexpr int RS_TILE = RS_WARPS * RS_WARP_ITEMS;  // 8192
constexpr int RS_UP_TPB = 256;                     // the upfront count's blocks
constexpr int RS_UP_ROUND = RS_UP_TPB * RS_IPT;    // keys per block and round
constexpr int RS_MAXPASS = 8;
// look-back polls of one tile's status before the pass gives up, records an
// error in the simulation's status word and treats the count as zero
// (every write is bounds-checked, so a failed pass stays in bounds)
constexpr uint32_t RS_SPIN_LIMIT = 1u << 21;
constexpr int RS_ERR_LOOKBACK = 0x5e01;
constexpr int RS_LOOK = 8;  // predecessor tiles read per look-back round trip

// status word of (tile, digit): count in bits 0..31, flag in bits 32..33
// (1: the tile's own count, 2: inclusive prefix over tiles 0..tile), pass
// tag (pass + 1) in bits 34..; words of an earlier pass read as not ready
__device__ __forceinline__ void st_status(unsigned long long *a, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(a), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_status(const unsigned long long *a) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
  return v;
}

template <class K>
__global__ void __launch_bounds__(RS_UP_TPB) rs_upfront(const K *keys, uint64_t n, int passes,
                                                         uint32_t *ghist) {
  __shared__ uint32_t h[RS_MAXPASS][256];
  for (int i = threadIdx.x; i < RS_MAXPASS * 256; i += RS_UP_TPB) (&h[0][0])[i] = 0;
  __syncthreads();
  // a round of RS_UP_ROUND keys: requested before any is counted
  for (uint64_t t0 = (uint64_t)blockIdx.x * RS_UP_ROUND; t0 < n;
       t0 += (uint64_t)gridDim.x * RS_UP_ROUND) {
    K k[RS_IPT];
#pragma unroll
    for (int i = 0; i < RS_IPT; i++) {
      const uint64_t idx = t0 + (uint64_t)i * RS_UP_TPB + threadIdx.x;
      k[i] = idx < n ? keys[idx] : K(0);
    }
#pragma unroll
    for (int i = 0; i < RS_IPT; i++) {
      if (t0 + (uint64_t)i * RS_UP_TPB + threadIdx.x >= n) break;
      for (int p = 0; p < passes; p++) atomicAdd(&h[p][(unsigned)(k[i] >> (8 * p)) & 255u], 1u);
    }
  }
  __syncthreads();
  for (int p = 0; p < passes; p++) {
    const uint32_t c = h[p][threadIdx.x];
    if (c) atomicAdd(&ghist[p * 256 + threadIdx.x], c);
  }
}

template <class K>
struct RsShared {
  uint32_t wcnt[RS_WARPS][256];
  uint32_t dstart[256];
  uint32_t gbase[256];
  uint32_t ws[32];
  uint32_t tile;
  int trivial;
  K key[RS_TILE];
  uint32_t val[RS_TILE];
};

// One pass: tile `tile` (from the ticket counter) is ranked stably (item
// order = warp, slot, lane = input order), published, offset by the
// look-back, staged in shared memory in digit order and written out in
// runs of consecutive positions.
template <class K>
__global__ void __launch_bounds__(RS_TPB, 1) rs_pass(const K *kin, const uint32_t *vin, K *kout,
                                                   uint32_t *vout, uint64_t n, int pass,
                                                   const uint32_t *ghist,
                                                   unsigned long long *status,
                                                   uint32_t *ticket, int *err) {
  extern __shared__ __align__(16) unsigned char rs_smem[];
  RsShared<K> &S = *reinterpret_cast<RsShared<K> *>(rs_smem);
  const bool digit_thread = threadIdx.x < 256;  // thread d owns digit d
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int shift = 8 * pass;
  const uint32_t gcount = digit_thread ? ghist[pass * 256 + threadIdx.x] : 0u;
  if (threadIdx.x == 0) {
    S.tile = atomicAdd(ticket, 1u);
    S.trivial = 0;
  }
  for (int d = threadIdx.x; d < RS_WARPS * 256; d += RS_TPB) (&S.wcnt[0][0])[d] = 0;
  __syncthreads();
  if (digit_thread && gcount == n) S.trivial = 1;  // every key has this digit: order kept
  const uint32_t tile = S.tile;
  const uint64_t t0 = (uint64_t)tile * RS_TILE;
  const uint32_t m = (uint32_t)(n - t0 < (uint64_t)RS_TILE ? n - t0 : (uint64_t)RS_TILE);
  __syncthreads();
  if (S.trivial) {
    for (uint32_t i = threadIdx.x; i < m; i += RS_TPB) {
      kout[t0 + i] = kin[t0 + i];
      vout[t0 + i] = vin[t0 + i];
    }
    return;
  }
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t wbase = (uint32_t)w * RS_WARP_ITEMS;
  K key[RS_IPT];
  uint32_t val[RS_IPT], rank[RS_IPT];
  int dig[RS_IPT];
  // every load of the tile is issued before the ranking's warp barriers
  // (loads placed between them would wait for one another)
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    const uint32_t i = wbase + (uint32_t)k * 32 + lane;
    key[k] = i < m ? kin[t0 + i] : K(0);
  }
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    const uint32_t i = wbase + (uint32_t)k * 32 + lane;
    val[k] = i < m ? vin[t0 + i] : 0u;
  }
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    const uint32_t i = wbase + (uint32_t)k * 32 + lane;
    const bool valid = i < m;
    const int d = valid ? (int)((key[k] >> shift) & 255u) : 256;
    dig[k] = d;
    rank[k] = 0;
    if (wbase + (uint32_t)k * 32 >= m) continue;  // warp-uniform: no item in this slot
    // the lanes with the same 9-bit label (digit, or 256 for no item), one
    // ballot per label bit (measured faster than match.any for full tiles)
    unsigned peers = 0xffffffffu;
#pragma unroll
    for (int bit = 0; bit < 9; bit++) {
      const bool set = (d >> bit) & 1;
      const unsigned v = __ballot_sync(0xffffffffu, set);
      peers &= set ? v : ~v;
    }
    const uint32_t b = valid ? S.wcnt[w][d] : 0u;
    rank[k] = b + __popc(peers & lt);
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) S.wcnt[w][d] = b + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // thread d < 256: exclusive counts of digit d over the warps, the tile's count
  const int d = digit_thread ? threadIdx.x : 0;
  uint32_t c = 0;
  if (digit_thread) {
#pragma unroll
    for (int w2 = 0; w2 < RS_WARPS; w2++) {
      const uint32_t t = S.wcnt[w2][d];
      S.wcnt[w2][d] = c;
      c += t;
    }
  }
  const unsigned long long tag = (unsigned long long)(pass + 1) << 34;
  unsigned long long *my = status + (uint64_t)tile * 256 + d;
  if (digit_thread) st_status(my, tag | ((tile ? 1ull : 2ull) << 32) | c);
  // all threads take part in the block scans (the others add 0)
  const uint32_t ds = block_exclusive_scan<uint32_t>(c, S.ws, (uint32_t *)nullptr);
  const uint32_t gex = block_exclusive_scan<uint32_t>(gcount, S.ws, (uint32_t *)nullptr);
  uint32_t excl = 0;
  if (digit_thread && tile) {
    // RS_LOOK predecessors per round trip: their words are loaded together
    // and consumed in order until a prefix, or a word not yet published
    int64_t t = (int64_t)tile - 1;
    uint32_t spins = 0;
    bool done = false;
    while (!done) {
      unsigned long long v[RS_LOOK];
#pragma unroll
      for (int i = 0; i < RS_LOOK; i++)
        v[i] = t - i >= 0 ? ld_status(status + (uint64_t)(t - i) * 256 + d) : 0ull;
      int used = 0;
#pragma unroll
      for (int i = 0; i < RS_LOOK; i++) {
        if (used != i || t - i < 0) break;
        const uint32_t flag =
            (v[i] >> 34) == (unsigned long long)(pass + 1) ? (uint32_t)(v[i] >> 32) & 3u : 0u;
        if (!flag) break;
        excl += (uint32_t)v[i];
        used++;
        if (flag == 2u || t - i == 0) {
          done = true;
          break;
        }
      }
      if (done) break;
      t -= used;
      if (used) {
        spins = 0;
      } else {
        if (++spins > RS_SPIN_LIMIT) {
          atomicCAS(err, 0, RS_ERR_LOOKBACK);
          break;
        }
        if (spins > 16) __nanosleep(64);
      }
    }
    st_status(my, tag | (2ull << 32) | (excl + c));
  }
  if (digit_thread) {
    S.dstart[d] = ds;
    S.gbase[d] = gex + excl;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    if (dig[k] < 256) {
      const uint32_t pos = S.dstart[dig[k]] + S.wcnt[w][dig[k]] + rank[k];
      S.key[pos] = key[k];
      S.val[pos] = val[k];
    }
  }
  __syncthreads();
  // unrolled over the RS_IPT items of a thread, so that their shared loads
  // overlap
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    const uint32_t i = threadIdx.x + (uint32_t)k * RS_TPB;
    if (i < m) {
      const K kk = S.key[i];
      const uint32_t dd = (uint32_t)(kk >> shift) & 255u;
      const uint64_t pos = (uint64_t)S.gbase[dd] + (i - S.dstart[dd]);
      if (pos < n) {
        kout[pos] = kk;
        vout[pos] = S.val[i];
      }
    }
  }
}

// scratch: digit counts [passes][256], tickets [passes], tile status
// words, then one or two alternate key/value buffers (two for an odd number
// of passes above one, so that the last pass lands in `keys`)
struct RsLayout {
  int passes, nalt;
  uint64_t ntiles, head, stat, kb, vb;
  uint64_t bytes() const { return head + stat + nalt * (kb + vb); }
};
RsLayout rs_layout(uint64_t n, int key_size, int bits) {
  RsLayout L;
  L.passes = std::min((bits + 7) / 8, key_size);
  L.ntiles = (n + RS_TILE - 1) / RS_TILE;
  L.nalt = (L.passes % 2 == 1 && L.passes > 1) ? 2 : 1;
  L.head = RS_MAXPASS * 256 * 4 + 64;
  L.stat = L.ntiles * 256 * 8;
  L.kb = (n * key_size + 255) & ~255ull;
  L.vb = (n * 4 + 255) & ~255ull;
  return L;
}

// `scratch`: null (allocated on the stream here) or at least
// radix_sort_scratch_bytes(n, sizeof(K), bits) bytes owned by the caller;
// with caller scratch the sort makes no allocation, so it can be recorded
// into a CUDA graph
// `counted`: the digit counts of every pass are already in the scratch's
// first RS_MAXPASS x 256 words (radix_sort_digit_counts), so the upfront
// count is skipped and those words are left as they are
template <class K>
void radix_sort_impl(K *keys, uint32_t *vals, uint64_t n, int bits, cudaStream_t st,
                     int *err, void *scratch = nullptr, bool counted = false) {
  if (n <= 1 || bits <= 0) return;
  if (n >= (1ull << 32)) fail(VG_ERR_NOMEM, "radix sort: more than 2^32 items");
  const RsLayout L = rs_layout(n, (int)sizeof(K), bits);
  const int passes = L.passes, nalt = L.nalt;
  const uint64_t ntiles = L.ntiles, head = L.head, stat = L.stat, kb = L.kb, vb = L.vb;
  char *buf = (char *)scratch;
  if (!buf) VG_CUDA(cudaMallocAsync((void **)&buf, L.bytes(), st));
  const uint64_t hist_bytes = RS_MAXPASS * 256 * 4;
  if (counted)
    VG_CUDA(cudaMemsetAsync(buf + hist_bytes, 0, head + stat - hist_bytes, st));
  else
    VG_CUDA(cudaMemsetAsync(buf, 0, head + stat, st));
  uint32_t *ghist = (uint32_t *)buf;
  uint32_t *tickets = (uint32_t *)(buf + RS_MAXPASS * 256 * 4);
  unsigned long long *status = (unsigned long long *)(buf + head);
  K *ka = (K *)(buf + head + stat);
  uint32_t *va = (uint32_t *)(buf + head + stat + kb);
  K *kb2 = nalt == 2 ? (K *)(buf + head + stat + kb + vb) : nullptr;
  uint32_t *vb2 = nalt == 2 ? (uint32_t *)(buf + head + stat + 2 * kb + vb) : nullptr;
  const unsigned hblocks =
      (unsigned)std::min<uint64_t>((n + RS_UP_ROUND - 1) / RS_UP_ROUND, 152 * 4);
  if (!counted) rs_upfront<K><<<hblocks, RS_UP_TPB, 0, st>>>(keys, n, passes, ghist);
  // the pass's shared memory exceeds the 48 KB of a static allocation
  static const bool smem_ok = [] {
    return cudaFuncSetAttribute(rs_pass<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(RsShared<K>)) == cudaSuccess;
  }();
  if (!smem_ok) fail(VG_ERR_CUDA, "radix sort: cannot reserve the pass's shared memory");
  VG_CUDA(cudaGetLastError());
  // buffer sequence: keys -> a -> keys ... for an even number of passes;
  // keys -> a -> b -> keys -> ... with three buffers for an odd number
  K *kbufs[3] = {keys, ka, kb2};
  uint32_t *vbufs[3] = {vals, va, vb2};
  int cur = 0;
  for (int p = 0; p < passes; p++) {
    int nxt;
    if (nalt == 1) nxt = cur == 0 ? 1 : 0;
    else if (p == passes - 1) nxt = 0;
    else nxt = cur == 0 ? 1 : (cur == 1 ? 2 : 1);
    rs_pass<K><<<(unsigned)ntiles, RS_TPB, sizeof(RsShared<K>), st>>>(kbufs[cur], vbufs[cur],
                                                                      kbufs[nxt],
                                                    vbufs[nxt], n, p, ghist, status,
                                                    tickets + p, err);
    VG_CUDA(cudaGetLastError());
    cur = nxt;
  }
  if (cur != 0) {  // one pass only
    VG_CUDA(cudaMemcpyAsync(keys, kbufs[cur], n * sizeof(K), cudaMemcpyDeviceToDevice, st));
    VG_CUDA(cudaMemcpyAsync(vals, vbufs[cur], n * 4, cudaMemcpyDeviceToDevice, st));
  }
  if (!scratch) VG_CUDA(cudaFreeAsync(buf, st));
}

}  // namespace

void exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n,
                        cudaStream_t st, Sim &s) {
  exclusive_scan_impl<uint32_t>(in, out, n, st, s.d_status.as<int>());
}
void exclusive_scan_u64(const uint64_t *in, uint64_t *out, uint64_t n,
                        cudaStream_t st, Sim &s) {
  exclusive_scan_impl<unsigned long long>((const unsigned long long *)in,
                                          (unsigned long long *)out, n, st,
                                          s.d_status.as<int>());
}
uint64_t exclusive_scan_scratch_bytes(uint64_t n) {
  return scan_scratch_bytes<uint32_t>(n);
}
void exclusive_scan_u32_in(const uint32_t *in, uint32_t *out, uint64_t n, cudaStream_t st,
                           int *err, void *scratch) {
  exclusive_scan_impl<uint32_t>(in, out, n, st, err, scratch);
}
void radix_sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint64_t n, int bits,
                          cudaStream_t st, Sim &s) {
  radix_sort_impl<uint32_t>(keys, vals, n, bits, st, s.d_status.as<int>());
}
uint64_t radix_sort_scratch_bytes(uint64_t n, int key_size, int bits) {
  if (n <= 1 || bits <= 0) return 0;
  return rs_layout(n, key_size, bits).bytes();
}
void radix_sort_pairs_u32_in(uint32_t *keys, uint32_t *vals, uint64_t n, int bits,
                             cudaStream_t st, int *err, void *scratch, bool counted) {
  radix_sort_impl<uint32_t>(keys, vals, n, bits, st, err, scratch, counted);
}
uint32_t *radix_sort_digit_counts(void *scratch) { return (uint32_t *)scratch; }
void radix_sort_pairs_u64(uint64_t *keys, uint32_t *vals, uint64_t n, int bits,
                          cudaStream_t st, Sim &s) {
  radix_sort_impl<unsigned long long>((unsigned long long *)keys, vals, n, bits, st,
                                      s.d_status.as<int>());
}

void set_last_error(const std::string &m);

}  // namespace vg

// Sorts n generated (key, index) pairs on the device and compares the result
// with a stable sort on the host.  Keys: splitmix64 of (seed, i), masked to
// key_bits, with bits [const_lo, const_hi) forced to one (a digit that all
// keys share exercises the pass that keeps the order).  Returns the number of
// mismatching positions in *mismatch_out (keys or values).
extern "C" int vg_selftest_sort(uint64_t n, int key_bits, int wide, int const_lo, int const_hi,
                                uint64_t seed, uint64_t *mismatch_out) {
  using namespace vg;
  try {
    if (key_bits < 1 || key_bits > (wide ? 64 : 32) || const_lo < 0 || const_hi > key_bits)
      fail(VG_ERR_ARG, "vg_selftest_sort: bad key bits");
    std::vector<unsigned long long> k(n);
    uint64_t cmask = 0;
    for (int b = const_lo; b < const_hi; b++) cmask |= 1ull << b;
    const uint64_t kmask = key_bits == 64 ? ~0ull : (1ull << key_bits) - 1;
    for (uint64_t i = 0; i < n; i++) {
      uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      // clustered keys: a quarter of the keys repeat a small set of values
      if ((z & 3) == 0) z = (z >> 8) % 7;
      k[i] = ((z & kmask) | cmask) & kmask;
    }
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    std::vector<uint32_t> ref = idx;
    std::stable_sort(ref.begin(), ref.end(), [&](uint32_t a, uint32_t b) { return k[a] < k[b]; });
    cudaStream_t st;
    VG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    void *dk = nullptr, *dv = nullptr;
    int *derr = nullptr;
    VG_CUDA(cudaMalloc(&dk, std::max<uint64_t>(n, 1) * 8));
    VG_CUDA(cudaMalloc(&dv, std::max<uint64_t>(n, 1) * 4));
    VG_CUDA(cudaMalloc(&derr, 4));
    VG_CUDA(cudaMemset(derr, 0, 4));
    std::vector<uint32_t> k32(wide ? 0 : n);
    for (uint64_t i = 0; i < k32.size(); i++) k32[i] = (uint32_t)k[i];
    if (wide)
      VG_CUDA(cudaMemcpy(dk, k.data(), n * 8, cudaMemcpyHostToDevice));
    else
      VG_CUDA(cudaMemcpy(dk, k32.data(), n * 4, cudaMemcpyHostToDevice));
    VG_CUDA(cudaMemcpy(dv, idx.data(), n * 4, cudaMemcpyHostToDevice));
    if (wide)
      radix_sort_impl<unsigned long long>((unsigned long long *)dk, (uint32_t *)dv, n, key_bits,
                                          st, derr);
    else
      radix_sort_impl<uint32_t>((uint32_t *)dk, (uint32_t *)dv, n, key_bits, st, derr);
    VG_CUDA(cudaStreamSynchronize(st));
    std::vector<unsigned long long> ok(n);
    std::vector<uint32_t> ok32(wide ? 0 : n), ov(n);
    int herr = 0;
    if (wide)
      VG_CUDA(cudaMemcpy(ok.data(), dk, n * 8, cudaMemcpyDeviceToHost));
    else
      VG_CUDA(cudaMemcpy(ok32.data(), dk, n * 4, cudaMemcpyDeviceToHost));
    VG_CUDA(cudaMemcpy(ov.data(), dv, n * 4, cudaMemcpyDeviceToHost));
    VG_CUDA(cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost));
    VG_CUDA(cudaFree(dk));
    VG_CUDA(cudaFree(dv));
    VG_CUDA(cudaFree(derr));
    VG_CUDA(cudaStreamDestroy(st));
    if (herr) fail(VG_ERR_DEVICE, "vg_selftest_sort: device status " + std::to_string(herr));
    uint64_t bad = 0;
    for (uint64_t i = 0; i < n; i++) {
      const unsigned long long kk = wide ? ok[i] : ok32[i];
      bad += (ov[i] != ref[i]) || (kk != k[ref[i]]);
    }
    *mismatch_out = bad;
    return VG_OK;
  } catch (const Error &e) {
    set_last_error(e.msg);
    return e.code;
  }
}

// Exclusive scan of n generated values (32-bit, or 64-bit when wide != 0)
// on the device, in place or out of place, against a host prefix sum
// (wrapping arithmetic on both sides); *mismatch_out = mismatching items.
// Failure detection without a GPU fault: a three-tile look-back scan is
// launched with two blocks and its tile counter starting at 1, so tile 0
// never runs and never publishes.  Tile 1 (and possibly tile 2) waits for
// it until the spin limit, records SCAN_ERR_LOOKBACK in the status word and
// finishes; every index stays inside the three tiles' buffers.  Reports the
// status word and the kernel's duration.
extern "C" int vg_selftest_scan_timeout(int *status_out, double *ms_out) {
  using namespace vg;
  try {
    need(status_out, "status pointer");
    const uint64_t nt = 3, n = nt * SCAN_CHUNK;
    uint32_t *din = nullptr, *dout = nullptr;
    int *derr = nullptr;
    char *buf = nullptr;
    const uint64_t bytes = scan_scratch_bytes<uint32_t>(n);
    VG_CUDA(cudaMalloc(&din, n * 4));
    VG_CUDA(cudaMalloc(&dout, n * 4));
    VG_CUDA(cudaMalloc(&derr, 4));
    VG_CUDA(cudaMalloc(&buf, bytes));
    VG_CUDA(cudaMemset(din, 0, n * 4));
    VG_CUDA(cudaMemset(dout, 0, n * 4));
    VG_CUDA(cudaMemset(derr, 0, 4));
    VG_CUDA(cudaMemset(buf, 0, bytes));
    const uint32_t first_ticket = 1;
    VG_CUDA(cudaMemcpy(buf, &first_ticket, 4, cudaMemcpyHostToDevice));
    ScanState<uint32_t> S;
    S.ticket = (uint32_t *)buf;
    S.flag = (uint32_t *)(buf + 64);
    const uint64_t aoff = (64 + nt * 4 + 15) & ~15ull;
    S.agg = (uint32_t *)(buf + aoff);
    S.pre = S.agg + nt;
    cudaStream_t st;
    cudaEvent_t e0, e1;
    VG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    VG_CUDA(cudaEventCreate(&e0));
    VG_CUDA(cudaEventCreate(&e1));
    VG_CUDA(cudaEventRecord(e0, st));
    scan_lookback<uint32_t><<<(unsigned)(nt - 1), SCAN_TPB, 0, st>>>(din, dout, n, S, derr);
    VG_CUDA(cudaGetLastError());
    VG_CUDA(cudaEventRecord(e1, st));
    VG_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    VG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    int herr = 0;
    VG_CUDA(cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost));
    VG_CUDA(cudaEventDestroy(e0));
    VG_CUDA(cudaEventDestroy(e1));
    VG_CUDA(cudaStreamDestroy(st));
    VG_CUDA(cudaFree(din));
    VG_CUDA(cudaFree(dout));
    VG_CUDA(cudaFree(derr));
    VG_CUDA(cudaFree(buf));
    *status_out = herr;
    if (ms_out) *ms_out = ms;
    return VG_OK;
  } catch (const Error &e) {
    set_last_error(e.msg);
    return e.code;
  }
}

extern "C" int vg_selftest_scan(uint64_t n, int wide, int in_place, uint64_t seed,
                                uint64_t *mismatch_out) {
  using namespace vg;
  try {
    std::vector<unsigned long long> h(n);
    for (uint64_t i = 0; i < n; i++) {
      uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      h[i] = (z & 7) == 0 ? 0 : (wide ? z >> 20 : (z >> 40) & 0xFFFFF);
    }
    const size_t es = wide ? 8 : 4;
    std::vector<uint32_t> h32(wide ? 0 : n);
    for (uint64_t i = 0; i < h32.size(); i++) h32[i] = (uint32_t)h[i];
    void *din = nullptr, *dout = nullptr;
    int *derr = nullptr;
    VG_CUDA(cudaMalloc(&din, std::max<uint64_t>(n, 1) * es));
    VG_CUDA(cudaMalloc(&dout, std::max<uint64_t>(n, 1) * es));
    VG_CUDA(cudaMalloc(&derr, 4));
    VG_CUDA(cudaMemset(derr, 0, 4));
    VG_CUDA(cudaMemcpy(din, wide ? (const void *)h.data() : (const void *)h32.data(), n * es,
                       cudaMemcpyHostToDevice));
    cudaStream_t st;
    VG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    void *o = in_place ? din : dout;
    if (wide)
      exclusive_scan_impl<unsigned long long>((const unsigned long long *)din,
                                              (unsigned long long *)o, n, st, derr);
    else
      exclusive_scan_impl<uint32_t>((const uint32_t *)din, (uint32_t *)o, n, st, derr);
    VG_CUDA(cudaStreamSynchronize(st));
    std::vector<unsigned long long> r(n);
    std::vector<uint32_t> r32(wide ? 0 : n);
    int herr = 0;
    VG_CUDA(cudaMemcpy(wide ? (void *)r.data() : (void *)r32.data(), o, n * es,
                       cudaMemcpyDeviceToHost));
    VG_CUDA(cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost));
    VG_CUDA(cudaStreamDestroy(st));
    VG_CUDA(cudaFree(din));
    VG_CUDA(cudaFree(dout));
    VG_CUDA(cudaFree(derr));
    if (herr) fail(VG_ERR_DEVICE, "vg_selftest_scan: device status " + std::to_string(herr));
    uint64_t bad = 0;
    unsigned long long acc = 0;
    for (uint64_t i = 0; i < n; i++) {
      const unsigned long long got = wide ? r[i] : r32[i];
      const unsigned long long want = wide ? acc : (uint32_t)acc;
      bad += got != want;
      acc += h[i];
    }
    *mismatch_out = bad;
    return VG_OK;
  } catch (const Error &e) {
    set_last_error(e.msg);
    return e.code;
  }
}
