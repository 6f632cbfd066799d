// Device primitives: exclusive scan and a stable LSD radix sort of
// (key, value) pairs.  Both are the building blocks of the CSR
// (re)construction that reproduces Vahana's per-target `push!` order
// (src/EdgeMethods.jl:495-496): records arrive in insertion order (or carry
// an order key), and a stable sort by target row keeps that order inside
// each row.
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

template <class T>
__global__ void scan_partials(const T *in, uint64_t n, T *partials) {
  __shared__ T ws[32];
  __shared__ T tot;
  uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK;
  T s = 0;
  for (int k = 0; k < SCAN_IPT; k++) {
    uint64_t i = base + (uint64_t)k * SCAN_TPB + threadIdx.x;
    if (i < n) s += in[i];
  }
  block_exclusive_scan<T>(s, ws, &tot);
  if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

// Each thread owns SCAN_IPT consecutive items; safe in place.
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

template <class T>
void exclusive_scan_impl(const T *in, T *out, uint64_t n, cudaStream_t st) {
  if (n == 0) return;
  uint64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if (nb == 1) {
    scan_apply<T><<<1, SCAN_TPB, 0, st>>>(in, out, n, nullptr);
    VG_CUDA(cudaGetLastError());
    return;
  }
  T *part = nullptr;
  VG_CUDA(cudaMallocAsync((void **)&part, nb * sizeof(T), st));
  scan_partials<T><<<(unsigned)nb, SCAN_TPB, 0, st>>>(in, n, part);
  VG_CUDA(cudaGetLastError());
  exclusive_scan_impl<T>(part, part, nb, st);
  scan_apply<T><<<(unsigned)nb, SCAN_TPB, 0, st>>>(in, out, n, part);
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaFreeAsync(part, st));
}

// ------------------------------------------------------------ radix sort
constexpr int RS_TPB = 256;
constexpr int RS_WARPS = RS_TPB / 32;
constexpr int RS_IPT = 8;                    // items per lane
constexpr int RS_WARP_ITEMS = 32 * RS_IPT;  // 256
constexpr int RS_TILE = RS_WARPS * RS_WARP_ITEMS;  // 2048

template <class K>
__global__ void rs_hist(const K *keys, uint64_t n, int shift, uint32_t *hist,
                        uint32_t ntiles) {
  __shared__ uint32_t s[256];
  s[threadIdx.x] = 0;
  __syncthreads();
  uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
#pragma unroll
  for (int k = 0; k < RS_TILE / RS_TPB; k++) {
    uint64_t i = base + (uint64_t)k * RS_TPB + threadIdx.x;
    if (i < n) atomicAdd(&s[(unsigned)((keys[i] >> shift) & 255u)], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = s[threadIdx.x];
}

// Stable scatter: the tile's logical item order is (warp, k, lane), and
// ranks are accumulated in that order.
template <class K>
__global__ void rs_scatter(const K *kin, const uint32_t *vin, K *kout,
                           uint32_t *vout, uint64_t n, int shift,
                           const uint32_t *offs, uint32_t ntiles) {
  __shared__ uint32_t wcnt[RS_WARPS][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < RS_WARPS * 256; d += RS_TPB)
    (&wcnt[0][0])[d] = 0;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  uint64_t base = (uint64_t)blockIdx.x * RS_TILE + (uint64_t)w * RS_WARP_ITEMS;
  K key[RS_IPT];
  uint32_t val[RS_IPT], rank[RS_IPT];
  int dig[RS_IPT];
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    uint64_t i = base + (uint64_t)k * 32 + lane;
    bool valid = i < n;
    key[k] = valid ? kin[i] : K(0);
    val[k] = valid ? vin[i] : 0u;
    int d = valid ? (int)((key[k] >> shift) & 255u) : 256;
    dig[k] = d;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t b = valid ? wcnt[w][d] : 0u;
    rank[k] = b + __popc(peers & lt);
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) wcnt[w][d] = b + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    int d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w2 = 0; w2 < RS_WARPS; w2++) {
      uint32_t t = wcnt[w2][d];
      wcnt[w2][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    if (dig[k] < 256) {
      uint64_t pos = (uint64_t)offs[(uint64_t)dig[k] * ntiles + blockIdx.x] +
                     wcnt[w][dig[k]] + rank[k];
      kout[pos] = key[k];
      vout[pos] = val[k];
    }
  }
}

template <class K>
void radix_sort_impl(K *keys, uint32_t *vals, uint64_t n, int bits,
                     cudaStream_t st) {
  if (n <= 1 || bits <= 0) return;
  if (n >= (1ull << 32)) fail(VG_ERR_NOMEM, "radix sort: more than 2^32 items");
  uint32_t ntiles = (uint32_t)((n + RS_TILE - 1) / RS_TILE);
  K *kalt = nullptr;
  uint32_t *valt = nullptr, *hist = nullptr;
  VG_CUDA(cudaMallocAsync((void **)&kalt, n * sizeof(K), st));
  VG_CUDA(cudaMallocAsync((void **)&valt, n * sizeof(uint32_t), st));
  VG_CUDA(cudaMallocAsync((void **)&hist, (uint64_t)256 * ntiles * 4, st));
  K *ki = keys, *ko = kalt;
  uint32_t *vi = vals, *vo = valt;
  int passes = (bits + 7) / 8;
  for (int p = 0; p < passes; p++) {
    int shift = 8 * p;
    rs_hist<K><<<ntiles, RS_TPB, 0, st>>>(ki, n, shift, hist, ntiles);
    VG_CUDA(cudaGetLastError());
    exclusive_scan_impl<uint32_t>(hist, hist, (uint64_t)256 * ntiles, st);
    rs_scatter<K><<<ntiles, RS_TPB, 0, st>>>(ki, vi, ko, vo, n, shift, hist,
                                             ntiles);
    VG_CUDA(cudaGetLastError());
    std::swap(ki, ko);
    std::swap(vi, vo);
  }
  if (ki != keys) {
    VG_CUDA(cudaMemcpyAsync(keys, ki, n * sizeof(K), cudaMemcpyDeviceToDevice, st));
    VG_CUDA(cudaMemcpyAsync(vals, vi, n * 4, cudaMemcpyDeviceToDevice, st));
  }
  VG_CUDA(cudaFreeAsync(kalt, st));
  VG_CUDA(cudaFreeAsync(valt, st));
  VG_CUDA(cudaFreeAsync(hist, st));
}

}  // namespace

void exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n,
                        cudaStream_t st, Sim &) {
  exclusive_scan_impl<uint32_t>(in, out, n, st);
}
void exclusive_scan_u64(const uint64_t *in, uint64_t *out, uint64_t n,
                        cudaStream_t st, Sim &) {
  exclusive_scan_impl<unsigned long long>((const unsigned long long *)in,
                                          (unsigned long long *)out, n, st);
}
void radix_sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint64_t n, int bits,
                          cudaStream_t st, Sim &) {
  radix_sort_impl<uint32_t>(keys, vals, n, bits, st);
}
void radix_sort_pairs_u64(uint64_t *keys, uint32_t *vals, uint64_t n, int bits,
                          cudaStream_t st, Sim &) {
  radix_sort_impl<unsigned long long>((unsigned long long *)keys, vals, n, bits,
                                      st);
}

}  // namespace vg
