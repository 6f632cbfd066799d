// CSR construction and maintenance.
//
// build_csr_from_records rebuilds an edge type's containers from a batch of
// edge records that are in Vahana's call order (or carry an order key):
// the per-target order that results is the one `push!` produces in
// add_edge! (src/EdgeMethods.jl:478-522).  With merge_existing the old
// edges of a row come first, as with add_existing (src/EdgeMethods.jl:
// 639-663, where the write container starts as a copy of the read one).
//
// remove_died_edges removes the edges of agents that died in a transition:
// rows of died targets (_remove_edges_agent_target!, src/EdgeMethods.jl:
// 897-920) and, for edge types that store the source, edges whose source
// died (_remove_edges_agent_source!, :606-631).
#include <algorithm>

#include "vg_internal.h"

namespace vg {

namespace {

constexpr int TPB = 256;
inline unsigned nblk(uint64_t n, int tpb = TPB) {
  uint64_t b = (n + tpb - 1) / tpb;
  return (unsigned)std::max<uint64_t>(b, 1);
}

__global__ void k_type_hist(const uint64_t *to, const uint64_t *from, uint64_t n,
                            unsigned long long *counts, unsigned *srcmask) {
  __shared__ unsigned long long sc[MAX_AGENT_TYPES];
  __shared__ unsigned sm;
  if (threadIdx.x < MAX_AGENT_TYPES) sc[threadIdx.x] = 0;
  if (threadIdx.x == 0) sm = 0;
  __syncthreads();
  // records mostly share one target type: count runs of equal types in a
  // register and flush a run to shared memory when the type changes
  unsigned mymask = 0, run_t = 0xFFFFFFFFu;
  unsigned long long run_n = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    unsigned t = (unsigned)(to[i] >> SHIFT_TYPE);
    if (t != run_t) {
      if (run_n && run_t < MAX_AGENT_TYPES) atomicAdd(&sc[run_t], run_n);
      run_t = t;
      run_n = 0;
    }
    run_n++;
    if (from) {
      unsigned f = (unsigned)(from[i] >> SHIFT_TYPE);
      if (f < 32) mymask |= 1u << f;
    }
  }
  if (run_n && run_t < MAX_AGENT_TYPES) atomicAdd(&sc[run_t], run_n);
  if (mymask) atomicOr(&sm, mymask);
  __syncthreads();
  if (threadIdx.x < MAX_AGENT_TYPES && sc[threadIdx.x])
    atomicAdd(&counts[threadIdx.x], sc[threadIdx.x]);
  if (threadIdx.x == 0 && sm) atomicOr(srcmask, sm);
}

__global__ void k_iota(uint32_t *v, uint64_t n) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}

__global__ void k_copy_u64(const uint64_t *a, uint64_t *b, uint64_t n) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

__global__ void k_flag_type(const uint64_t *to, const uint32_t *ord, uint64_t n,
                            unsigned T, uint32_t *flags) {
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) flags[j] = ((unsigned)(to[ord[j]] >> SHIFT_TYPE) == T) ? 1u : 0u;
}

__global__ void k_compact_sel(const uint32_t *ord, const uint32_t *flags,
                              const uint32_t *pos, uint64_t n, uint32_t *out) {
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n && flags[j]) out[pos[j]] = ord[j];
}

__global__ void k_row_keys(const uint64_t *to, const uint32_t *sel, uint64_t m,
                           uint64_t nrows, uint32_t *keys, uint32_t *vals,
                           int *status) {
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  uint32_t r = sel[j];
  uint64_t nr = to[r] & NR_MASK;
  if (nr == 0 || nr > nrows) {
    atomicExch(status, 101);  // edge to an agent number that does not exist
    nr = 1;
  }
  keys[j] = (uint32_t)(nr - 1);
  vals[j] = r;
}

__global__ void k_hist_rows(const uint32_t *keys, uint64_t m, uint32_t *cnt) {
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m) atomicAdd(&cnt[keys[j]], 1u);
}

__global__ void k_add_old_counts(const uint32_t *old_rp, uint64_t old_nrows,
                                 const uint32_t *newcnt, uint32_t *tot,
                                 uint32_t *oldcnt, uint64_t nrows) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  uint32_t o = 0;
  if (old_rp && r < old_nrows) o = old_rp[r + 1] - old_rp[r];
  oldcnt[r] = o;
  tot[r] = o + newcnt[r];
}

__global__ void k_clamp1(uint32_t *cnt, uint64_t nrows) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nrows && cnt[r] > 1) cnt[r] = 1;
}

__global__ void k_max_u32(const uint32_t *v, uint64_t n, unsigned *out) {
  unsigned m = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, v[i]);
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// destination of old edge k: same offset inside its row of the new CSR
__global__ void k_old_dest(const uint32_t *old_rp, uint64_t old_nrows,
                           uint64_t old_ne, const uint32_t *new_rp,
                           uint32_t *dest) {
  uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= old_ne) return;
  // binary search: last r with old_rp[r] <= k
  uint64_t lo = 0, hi = old_nrows;  // old_rp[lo] <= k < old_rp[hi]
  while (hi - lo > 1) {
    uint64_t mid = (lo + hi) >> 1;
    if (old_rp[mid] <= k) lo = mid; else hi = mid;
  }
  dest[k] = new_rp[lo] + (uint32_t)(k - old_rp[lo]);
}

__global__ void k_new_dest(const uint32_t *keys, uint64_t m,
                           const uint32_t *new_rp, const uint32_t *oldcnt,
                           const uint32_t *seg, uint32_t *dest, int dedupe) {
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  uint32_t r = keys[j];
  uint32_t within = (uint32_t)j - seg[r];
  if (dedupe && (within + oldcnt[r]) > 0) {
    dest[j] = 0xffffffffu;  // HasEdgeOnly keeps a single `true`
    return;
  }
  dest[j] = new_rp[r] + oldcnt[r] + within;
}

__global__ void k_place_src(const uint64_t *from, const uint32_t *rec,
                            const uint32_t *dest, uint64_t m, uint32_t *src,
                            uint8_t *src_type) {
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m || dest[j] == 0xffffffffu) return;
  uint64_t f = from[rec[j]];
  src[dest[j]] = (uint32_t)((f & NR_MASK) - 1);
  if (src_type) src_type[dest[j]] = (uint8_t)(f >> SHIFT_TYPE);
}

template <class E>
__global__ void k_scatter_col(const E *in, const uint32_t *rec,
                              const uint32_t *dest, uint64_t m, E *out) {
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const uint32_t dj = dest ? dest[j] : (uint32_t)j;  // no dest: a gather in place order
  if (dj == 0xffffffffu) return;
  out[dj] = rec ? in[rec[j]] : in[j];
}

__global__ void k_fill_u8(uint8_t *p, uint8_t v, const uint32_t *dest,
                          uint64_t m) {
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m) p[dest ? dest[j] : j] = v;
}

void scatter_column(int esz, const void *in, const uint32_t *rec,
                    const uint32_t *dest, uint64_t m, void *out,
                    cudaStream_t st) {
  if (m == 0) return;
  switch (esz) {
    case 1: k_scatter_col<uint8_t><<<nblk(m), TPB, 0, st>>>((const uint8_t *)in, rec, dest, m, (uint8_t *)out); break;
    case 2: k_scatter_col<uint16_t><<<nblk(m), TPB, 0, st>>>((const uint16_t *)in, rec, dest, m, (uint16_t *)out); break;
    case 4: k_scatter_col<uint32_t><<<nblk(m), TPB, 0, st>>>((const uint32_t *)in, rec, dest, m, (uint32_t *)out); break;
    case 8: k_scatter_col<uint64_t><<<nblk(m), TPB, 0, st>>>((const uint64_t *)in, rec, dest, m, (uint64_t *)out); break;
    default: fail(VG_ERR_ARG, "unsupported field size");
  }
  VG_CUDA(cudaGetLastError());
}

template <class T> struct Tmp {
  T *p = nullptr;
  cudaStream_t st;
  Tmp(uint64_t n, cudaStream_t s) : st(s) {
    VG_CUDA(cudaMallocAsync((void **)&p, std::max<uint64_t>(n, 1) * sizeof(T), st));
  }
  ~Tmp() { if (p) cudaFreeAsync(p, st); }
};

// ------------------------------------------------------ died-edge removal
__global__ void k_keep_flags(const uint32_t *rp, uint64_t nrows,
                             const uint32_t *src, const uint8_t *src_type,
                             int src_type_const, const uint8_t *died,
                             uint64_t died_n, int died_type, int target_is_died,
                             int check_src, uint32_t *keep) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  uint32_t b = rp[r], e = rp[r + 1];
  bool tdead = target_is_died && r < died_n && died[r];
  for (uint32_t k = b; k < e; k++) {
    bool kp = !tdead;
    if (kp && check_src) {
      int t = src_type ? src_type[k] : src_type_const;
      uint32_t sidx = src[k];
      if (t == died_type && sidx < died_n && died[sidx]) kp = false;
    }
    keep[k] = kp ? 1u : 0u;
  }
}

__global__ void k_new_rowptr(const uint32_t *rp, uint64_t nrows,
                             const uint32_t *keep_scan, uint32_t *out) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r <= nrows) out[r] = keep_scan[rp[r]];
}

__global__ void k_compact_dest(const uint32_t *keep, const uint32_t *scan,
                               uint64_t n, uint32_t *dest) {
  uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dest[k] = keep[k] ? scan[k] : 0xffffffffu;
}

}  // namespace

uint64_t csr_edges_total(const EdgeStore &es) {
  uint64_t t = 0;
  for (auto &c : es.csr) t += c.nedges;
  return t;
}

// ---------------------------------------- fast rebuild from typed records
namespace {
// row key of each record (target agent_nr - 1); a record of another type or
// beyond the rows sets the status word (the records come from kernels that
// declare their types)
// key: the target row; value: the source's agent_nr - 1, which the stable
// sort then carries straight into the CSR's source column.  With
// digit_counts, the kernel also counts the keys' 8-bit digits of `passes`
// sort passes (the radix sort's upfront count: per block in shared memory,
// then added to digit_counts[256 p + digit]); the grid then strides.
__global__ void k_typed_keys(const uint64_t *to, const uint64_t *from, uint64_t n,
                             uint32_t target_type, uint32_t src_type, uint64_t nrows,
                             uint32_t *keys, uint32_t *src, int *status,
                             uint32_t *digit_counts, int passes) {
  __shared__ uint32_t h[4 * 256];
  if (digit_counts) {
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
  }
  // four records per thread and round, their loads issued before the
  // shared-memory counts (which would otherwise order each load after the
  // previous record's atomics)
  constexpr int U = 4;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t k0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += U * stride) {
    uint64_t tv[U], fv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const uint64_t k = k0 + u * stride;
      tv[u] = k < n ? to[k] : 0;
      fv[u] = k < n ? from[k] : 0;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const uint64_t k = k0 + u * stride;
      if (k >= n) break;
      const uint64_t t = tv[u], f = fv[u];
      uint64_t r = (t & NR_MASK) - 1;
      const bool bad = (uint32_t)(t >> SHIFT_TYPE) != target_type || r >= nrows ||
                       (uint32_t)(f >> SHIFT_TYPE) != src_type;
      if (bad) {
        atomicCAS(status, 0, 501);
        r = 0;
      }
      keys[k] = (uint32_t)r;
      src[k] = (uint32_t)((f & NR_MASK) - 1);
      if (digit_counts)
        for (int p = 0; p < passes; p++) atomicAdd(&h[p * 256 + ((r >> (8 * p)) & 255u)], 1u);
    }
  }
  if (digit_counts) {
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
      if (h[i]) atomicAdd(digit_counts + i, h[i]);
  }
}

// row_ptr of the rows 0..nrows from the sorted row keys: rp[r] = the
// number of keys below r.  Rows are cut into spans of RP_ROWS, one block
// each; a first pass over the records finds, for every span boundary
// j * RP_ROWS, the first record at or above it (record k owns the boundaries
// in (keys[k-1], keys[k]]).  In the block, the last record of each row's run
// stores its end position (relative to the span's first record) at the
// row's slot in shared memory -- one plain store per non-empty row, however
// long the run.  Since the ends grow with the row, rp of a row is the
// largest end stored before it: an exclusive max-scan (each thread 32
// consecutive rows, then across the threads), which also gives every
// non-empty row's length for the block's largest degree.  The rows leave
// shared memory as coalesced 16-byte stores.  Shared rows are swizzled in
// 16-byte chunks (chunk q of thread t at q ^ (t & 7)) so that both the
// per-thread and the per-warp access patterns avoid bank conflicts.
constexpr uint32_t RP_ROWS = 8192;
constexpr uint32_t RP_PER_THREAD = RP_ROWS / TPB;  // 32

__global__ void k_rp_bounds(const uint32_t *keys, uint64_t n, uint64_t nbr, uint32_t *bstart) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k > n) return;
  const uint64_t jlo = k == 0 ? 0 : (uint64_t)keys[k - 1] / RP_ROWS + 1;
  const uint64_t jhi = k == n ? nbr : (uint64_t)keys[k] / RP_ROWS;
  for (uint64_t j = jlo; j <= jhi; j++) bstart[j] = (uint32_t)k;
}

// shared word of row i of the span (32 rows per thread, 8 chunks of 4)
__device__ __forceinline__ uint32_t rp_slot(uint32_t i) {
  const uint32_t t = i >> 5, q = (i >> 2) & 7u;
  return (t << 5) | ((q ^ (t & 7u)) << 2) | (i & 3u);
}

__global__ void __launch_bounds__(TPB) k_rp_fill(const uint32_t *keys, uint64_t nrows,
                                                 const uint32_t *bstart, uint32_t *rp,
                                                 unsigned *maxdeg) {
  __shared__ __align__(16) uint32_t E[RP_ROWS];
  __shared__ uint32_t ws[32];
  const uint32_t tid = threadIdx.x;
  const uint64_t R0 = (uint64_t)blockIdx.x * RP_ROWS;
  const uint64_t R1 = R0 + RP_ROWS < nrows + 1 ? R0 + RP_ROWS : nrows + 1;
  const uint32_t k0 = bstart[blockIdx.x], k1 = bstart[blockIdx.x + 1];
  uint4 *E4 = reinterpret_cast<uint4 *>(E);
  for (uint32_t i = tid; i < RP_ROWS / 4; i += TPB) E4[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  for (uint32_t k = k0 + tid; k < k1; k += TPB) {
    const uint32_t key = keys[k];
    if (k + 1 == k1 || keys[k + 1] != key) E[rp_slot(key - (uint32_t)R0)] = k + 1 - k0;
  }
  __syncthreads();
  // pass 1: the largest end in the thread's 32 rows (its last stored end)
  uint4 v[RP_PER_THREAD / 4];
  uint32_t m = 0;
#pragma unroll
  for (uint32_t q = 0; q < RP_PER_THREAD / 4; q++) {
    v[q] = E4[(tid << 3) | (q ^ (tid & 7u))];
    m = max(m, max(max(v[q].x, v[q].y), max(v[q].z, v[q].w)));
  }
  // exclusive max-scan over the threads
  const uint32_t lane = tid & 31, wid = tid >> 5;
  uint32_t incl = m;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl = max(incl, y);
  }
  if (lane == 31) ws[wid] = incl;
  __syncthreads();
  uint32_t before = 0;
  for (uint32_t w2 = 0; w2 < wid; w2++) before = max(before, ws[w2]);
  const uint32_t excl_lane = __shfl_up_sync(0xffffffffu, incl, 1);
  uint32_t run = max(before, lane ? excl_lane : 0u);
  // pass 2: rp of each row = the largest end before it; a row's length is
  // its end minus that (0 for rows without an end: max(e, run) = run);
  // rows at or beyond nrows hold no end
  unsigned dmax = 0;
#pragma unroll
  for (uint32_t q = 0; q < RP_PER_THREAD / 4; q++) {
    uint32_t o0, o1, o2, o3, t;
    t = max(v[q].x, run); dmax = max(dmax, t - run); o0 = k0 + run; run = t;
    t = max(v[q].y, run); dmax = max(dmax, t - run); o1 = k0 + run; run = t;
    t = max(v[q].z, run); dmax = max(dmax, t - run); o2 = k0 + run; run = t;
    t = max(v[q].w, run); dmax = max(dmax, t - run); o3 = k0 + run; run = t;
    v[q] = make_uint4(o0, o1, o2, o3);
  }
#pragma unroll
  for (uint32_t q = 0; q < RP_PER_THREAD / 4; q++) E4[(tid << 3) | (q ^ (tid & 7u))] = v[q];
  __syncthreads();
  const uint32_t nr = (uint32_t)(R1 - R0);
  if (nr == RP_ROWS && ((uintptr_t)(rp + R0) & 15) == 0) {
    uint4 *out = reinterpret_cast<uint4 *>(rp + R0);
    for (uint32_t c = tid; c < RP_ROWS / 4; c += TPB)
      out[c] = E4[((c >> 3) << 3) | ((c & 7u) ^ ((c >> 3) & 7u))];
  } else {
    for (uint32_t i = tid; i < nr; i += TPB) rp[R0 + i] = E[rp_slot(i)];
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) dmax = max(dmax, __shfl_xor_sync(0xffffffffu, dmax, off));
  if (lane == 0 && dmax) atomicMax(maxdeg, dmax);
}

}  // namespace

uint32_t csr_max_degree(Sim &s, CSR &c) {
  if (c.max_degree_pending) {
    VG_CUDA(cudaMemcpyAsync(&c.max_degree, c.d_max_degree.p, 4, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    c.max_degree_pending = false;
  }
  return c.max_degree;
}

bool build_csr_typed(Sim &s, int e, const EdgeAppend &ap, uint64_t n) {
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  // the form the typed emitters produce: sources kept, no payload columns
  if (!ap.ordered || ap.target_type <= 0 || !ed.stores_src() || ap.src_type <= 0 ||
      ed.stores_payload() || ed.bool_only() || ed.singleedge() || es.add_existing ||
      n >= (1ull << 31))
    return false;
  const int T = ap.target_type;
  if (T > (int)s.model->atypes.size() || (ed.singletype() && T != ed.target)) return false;
  s.csr_epoch++;
  cudaStream_t st = s.stream;
  if (es.csr.size() < (size_t)MAX_AGENT_TYPES) es.csr.resize(MAX_AGENT_TYPES);
  for (int U = 1; U < (int)es.csr.size(); U++)
    if (U != T && es.csr[U].row_ptr.p) es.csr[U] = CSR();
  CSR &c = es.csr[T];
  const uint64_t nrows = s.agents[T - 1].n;
  // buffers of the previous container are reused when large enough (the
  // stream orders every earlier reader before these writes)
  auto ensure = [&](DevBuf &b, uint64_t bytes) {
    if (b.bytes < bytes || !b.p) b.alloc(std::max<uint64_t>(bytes, 16), &s.footprint);
  };
  ensure(c.row_ptr, (nrows + 1) * 4);
  ensure(c.src, std::max<uint64_t>(n, 1) * 4);
  c.src_type.release();
  c.payload.clear();
  ensure(c.d_max_degree, 4);
  if (!c.rebuild) c.rebuild.reset(new RebuildCache());
  RebuildCache &rc = *c.rebuild;
  const int bits = bits_for(nrows ? nrows - 1 : 0);
  const uint64_t nbr = (nrows + 1 + RP_ROWS - 1) / RP_ROWS;
  const uint64_t sort_bytes = radix_sort_scratch_bytes(n, 4, bits);
  ensure(rc.keys, std::max<uint64_t>(n, 1) * 4);
  ensure(rc.bstart, (nbr + 1) * 4);
  if (sort_bytes) ensure(rc.sort, sort_bytes);
  const uint64_t *from = ap.from.as<uint64_t>();
  // the sorted values are the source column itself
  uint32_t *keys = rc.keys.as<uint32_t>(), *src = c.src.as<uint32_t>();
  // the launch sequence, a function of these arguments only
  const std::vector<uint64_t> args = {
      (uint64_t)ap.to.p,  (uint64_t)from,          n,
      nrows,              (uint64_t)T,             (uint64_t)ap.src_type,
      (uint64_t)c.row_ptr.p, (uint64_t)src,        (uint64_t)c.d_max_degree.p,
      (uint64_t)keys,     (uint64_t)rc.sort.p,     (uint64_t)rc.bstart.p,
      (uint64_t)s.d_status.p};
  auto enqueue = [&]() {
    VG_CUDA(cudaMemsetAsync(c.d_max_degree.p, 0, 4, st));
    if (n) {
      // the sort's digit counts come from the key kernel (one pass over the
      // records fewer)
      const bool counted = sort_bytes > 0;
      const int passes = std::min((bits + 7) / 8, 4);
      uint32_t *dc = counted ? radix_sort_digit_counts(rc.sort.p) : nullptr;
      if (counted) VG_CUDA(cudaMemsetAsync(dc, 0, (size_t)passes * 256 * 4, st));
      const unsigned kb = counted ? std::min<unsigned>(nblk(n), 152 * 4) : nblk(n);
      k_typed_keys<<<kb, TPB, 0, st>>>(ap.to.as<uint64_t>(), from, n, (uint32_t)T,
                                       (uint32_t)ap.src_type, nrows, keys, src,
                                       s.d_status.as<int>(), dc, passes);
      radix_sort_pairs_u32_in(keys, src, n, bits, st, s.d_status.as<int>(), rc.sort.p, counted);
    }
    k_rp_bounds<<<nblk(n + 1), TPB, 0, st>>>(keys, n, nbr, rc.bstart.as<uint32_t>());
    k_rp_fill<<<(unsigned)nbr, TPB, 0, st>>>(keys, nrows, rc.bstart.as<uint32_t>(),
                                             c.row_ptr.as<uint32_t>(),
                                             c.d_max_degree.as<unsigned>());
    VG_CUDA(cudaGetLastError());
  };
  const bool graphable = st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
  if (rc.exec && args == rc.graph_args) {
    VG_CUDA(cudaGraphLaunch(rc.exec, st));
  } else if (graphable && args == rc.last) {
    // the same rebuild twice in a row: record it once, replay from now on
    if (rc.exec) {
      cudaGraphExecDestroy(rc.exec);
      rc.exec = nullptr;
      rc.graph_args.clear();
    }
    cudaGraph_t g = nullptr;
    VG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue();
    } catch (...) {
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    VG_CUDA(cudaStreamEndCapture(st, &g));
    const cudaError_t ie = cudaGraphInstantiate(&rc.exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) rc.exec = nullptr;
    VG_CUDA(ie);
    rc.graph_args = args;
    VG_CUDA(cudaGraphLaunch(rc.exec, st));
  } else {
    enqueue();
  }
  rc.last = std::move(args);
  VG_CUDA(cudaGetLastError());
  c.nrows = nrows;
  c.nedges = n;
  c.src_type_const = ed.stores_src() ? ap.src_type : 0;
  c.max_degree_pending = true;
  c.schedule_valid = false;
  c.unit_grid_weights = -1;
  return true;
}

void build_csr_from_records(Sim &s, int e, const uint64_t *d_from,
                            const uint64_t *d_to,
                            const std::vector<const void *> &d_payload,
                            uint64_t n, bool records_sorted_by_key,
                            const uint64_t *d_key, bool merge_existing) {
  s.csr_epoch++;
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  cudaStream_t st = s.stream;
  if (n >= (1ull << 31)) fail(VG_ERR_NOMEM, "more than 2^31 edge records in one build");

  // 1. target types and source types of the records
  unsigned long long h_counts[MAX_AGENT_TYPES] = {0};
  unsigned h_srcmask = 0;
  if (n > 0) {
    Tmp<unsigned long long> counts(MAX_AGENT_TYPES + 1, st);
    VG_CUDA(cudaMemsetAsync(counts.p, 0, (MAX_AGENT_TYPES + 1) * 8, st));
    unsigned *d_mask = (unsigned *)(counts.p + MAX_AGENT_TYPES);
    k_type_hist<<<std::min<unsigned>(nblk(n), 1024), TPB, 0, st>>>(
        d_to, ed.stores_src() ? d_from : nullptr, n, counts.p, d_mask);
    VG_CUDA(cudaGetLastError());
    VG_CUDA(cudaMemcpyAsync(h_counts, counts.p, MAX_AGENT_TYPES * 8, cudaMemcpyDeviceToHost, st));
    VG_CUDA(cudaMemcpyAsync(&h_srcmask, d_mask, 4, cudaMemcpyDeviceToHost, st));
    VG_CUDA(cudaStreamSynchronize(st));
  }
  if (es.csr.size() < (size_t)MAX_AGENT_TYPES) es.csr.resize(MAX_AGENT_TYPES);
  int ntypes_present = 0;
  for (int T = 1; T < MAX_AGENT_TYPES; T++) ntypes_present += h_counts[T] > 0;
  if (h_counts[0] > 0) fail(VG_ERR_ASSERT, "edge target is not a valid agent id");
  for (int T = 1; T < MAX_AGENT_TYPES; T++) {
    if (h_counts[T] == 0) continue;
    if (T > (int)s.model->atypes.size())
      fail(VG_ERR_ASSERT, "edge target has an unknown agent type");
    if (ed.singletype() && T != ed.target)
      fail(VG_ERR_ASSERT, "The :SingleType hint is set for " + ed.name +
                              ", and the agent type is specified as " +
                              s.model->at(ed.target).name +
                              ". But the type for the given agent is " +
                              s.model->at(T).name + ".");
  }

  // 2. order permutation of the records
  Tmp<uint32_t> ord(n, st);
  if (n > 0) {
    k_iota<<<nblk(n), TPB, 0, st>>>(ord.p, n);
    if (d_key && !records_sorted_by_key) {
      Tmp<uint64_t> kk(n, st);
      k_copy_u64<<<nblk(n), TPB, 0, st>>>(d_key, kk.p, n);
      radix_sort_pairs_u64(kk.p, ord.p, n, 64, st, s);
    }
  }

  // 3. per target type
  for (int T = 1; T < MAX_AGENT_TYPES; T++) {
    CSR &old = es.csr[T];
    bool has_old = merge_existing && old.nedges + old.nrows > 0 && old.row_ptr.p;
    if (h_counts[T] == 0 && !has_old) {
      if (!merge_existing) es.csr[T] = CSR();
      continue;
    }
    if (T > (int)s.model->atypes.size()) continue;
    uint64_t nrows = s.agents[T - 1].n;
    uint64_t m = h_counts[T];
    // select the records of this target type in order
    Tmp<uint32_t> sel(m, st);
    const uint32_t *selp = ord.p;
    if (m > 0 && ntypes_present > 1) {
      Tmp<uint32_t> flags(n + 1, st), pos(n + 1, st);
      k_flag_type<<<nblk(n), TPB, 0, st>>>(d_to, ord.p, n, (unsigned)T, flags.p);
      exclusive_scan_u32(flags.p, pos.p, n, st, s);
      k_compact_sel<<<nblk(n), TPB, 0, st>>>(ord.p, flags.p, pos.p, n, sel.p);
      selp = sel.p;
    }
    Tmp<uint32_t> keys(m, st), rec(m, st);
    Tmp<int> status(1, st);
    VG_CUDA(cudaMemsetAsync(status.p, 0, 4, st));
    if (m > 0) {
      k_row_keys<<<nblk(m), TPB, 0, st>>>(d_to, selp, m, nrows, keys.p, rec.p, status.p);
      radix_sort_pairs_u32(keys.p, rec.p, m, bits_for(nrows ? nrows - 1 : 0), st, s);
    }
    int h_status = 0;
    VG_CUDA(cudaMemcpyAsync(&h_status, status.p, 4, cudaMemcpyDeviceToHost, st));
    // counts
    Tmp<uint32_t> newcnt(nrows + 1, st), oldcnt(nrows + 1, st),
        tot(nrows + 1, st), seg(nrows + 1, st);
    VG_CUDA(cudaMemsetAsync(newcnt.p, 0, (nrows + 1) * 4, st));
    if (m > 0) k_hist_rows<<<nblk(m), TPB, 0, st>>>(keys.p, m, newcnt.p);
    exclusive_scan_u32(newcnt.p, seg.p, nrows + 1, st, s);
    k_add_old_counts<<<nblk(nrows + 1), TPB, 0, st>>>(
        has_old ? old.row_ptr.as<uint32_t>() : nullptr, has_old ? old.nrows : 0,
        newcnt.p, tot.p, oldcnt.p, nrows);
    VG_CUDA(cudaMemsetAsync(tot.p + nrows, 0, 4, st));
    VG_CUDA(cudaMemsetAsync(oldcnt.p + nrows, 0, 4, st));
    bool dedupe = ed.bool_only();
    if (dedupe) k_clamp1<<<nblk(nrows + 1), TPB, 0, st>>>(tot.p, nrows);
    CSR c;
    c.nrows = nrows;
    c.row_ptr.alloc((nrows + 1) * 4, &s.footprint);
    exclusive_scan_u32(tot.p, c.row_ptr.as<uint32_t>(), nrows + 1, st, s);
    uint32_t h_total = 0;
    VG_CUDA(cudaMemcpyAsync(&h_total, c.row_ptr.as<uint32_t>() + nrows, 4, cudaMemcpyDeviceToHost, st));
    {
      Tmp<unsigned> mx(1, st);
      VG_CUDA(cudaMemsetAsync(mx.p, 0, 4, st));
      k_max_u32<<<std::min<unsigned>(nblk(nrows), 1024), TPB, 0, st>>>(tot.p, nrows, mx.p);
      VG_CUDA(cudaMemcpyAsync(&c.max_degree, mx.p, 4, cudaMemcpyDeviceToHost, st));
    }
    VG_CUDA(cudaStreamSynchronize(st));
    if (h_status) fail(VG_ERR_ASSERT, "an edge targets an agent that does not exist");
    if (ed.singleedge() && !dedupe && c.max_degree > 1)
      fail(VG_ERR_ASSERT, "An edge has already been added to an agent of edge type " +
                              ed.name + " (which has the :SingleEdge hint).");
    c.nedges = h_total;
    // source types
    unsigned mask = 0;
    if (ed.stores_src()) {
      mask = m > 0 ? h_srcmask : 0;  // conservative: mask of all records
      if (has_old) {
        if (old.src_type_const > 0) mask |= 1u << old.src_type_const;
        if (old.src_type_const < 0) mask |= 0xfffeu;  // mixed: keep mixed
      }
    }
    int npop = __builtin_popcount(mask);
    c.src_type_const = npop == 0 ? 0 : (npop == 1 ? __builtin_ctz(mask) : -1);
    uint64_t ne = c.nedges;
    if (ed.stores_src()) {
      c.src.alloc(std::max<uint64_t>(ne, 1) * 4, &s.footprint);
      if (c.src_type_const < 0) c.src_type.alloc(std::max<uint64_t>(ne, 1), &s.footprint);
    }
    int nf = ed.stores_payload() ? (int)ed.fields.size() : 0;
    c.payload.resize(nf);
    for (int f = 0; f < nf; f++)
      c.payload[f].alloc(std::max<uint64_t>(ne, 1) * ed.fields[f].size, &s.footprint);
    // old edges
    if (has_old && old.nedges > 0) {
      Tmp<uint32_t> dest(old.nedges, st);
      k_old_dest<<<nblk(old.nedges), TPB, 0, st>>>(old.row_ptr.as<uint32_t>(), old.nrows,
                                                   old.nedges, c.row_ptr.as<uint32_t>(), dest.p);
      if (dedupe) {
        // rows keep one entry; old rows already hold at most one
      }
      if (ed.stores_src()) {
        scatter_column(4, old.src.p, nullptr, dest.p, old.nedges, c.src.p, st);
        if (c.src_type_const < 0) {
          if (old.src_type.p)
            scatter_column(1, old.src_type.p, nullptr, dest.p, old.nedges, c.src_type.p, st);
          else
            k_fill_u8<<<nblk(old.nedges), TPB, 0, st>>>(c.src_type.as<uint8_t>(),
                                                        (uint8_t)old.src_type_const, dest.p, old.nedges);
        }
      }
      for (int f = 0; f < nf; f++)
        scatter_column(ed.fields[f].size, old.payload[f].p, nullptr, dest.p, old.nedges,
                       c.payload[f].p, st);
    }
    // new records
    if (m > 0) {
      Tmp<uint32_t> dest(m, st);
      k_new_dest<<<nblk(m), TPB, 0, st>>>(keys.p, m, c.row_ptr.as<uint32_t>(), oldcnt.p,
                                          seg.p, dest.p, dedupe ? 1 : 0);
      if (ed.stores_src())
        k_place_src<<<nblk(m), TPB, 0, st>>>(d_from, rec.p, dest.p, m, c.src.as<uint32_t>(),
                                             c.src_type_const < 0 ? c.src_type.as<uint8_t>() : nullptr);
      for (int f = 0; f < nf; f++)
        scatter_column(ed.fields[f].size, d_payload[f], rec.p, dest.p, m, c.payload[f].p, st);
    }
    VG_CUDA(cudaGetLastError());
    es.csr[T] = std::move(c);
  }
  VG_CUDA(cudaStreamSynchronize(st));
}

// Replace c by its edges with keep[k] = 1 (scan = exclusive scan of keep,
// newtotal = kept edges), rows and order unchanged.
static void compact_csr(Sim &s, const EdgeTypeDesc &ed, CSR &c, const uint32_t *keep,
                        const uint32_t *scan, uint32_t newtotal) {
  cudaStream_t st = s.stream;
  uint64_t ne = c.nedges;
  CSR n2;
  n2.nrows = c.nrows;
  n2.nedges = newtotal;
  n2.src_type_const = c.src_type_const;
  n2.row_ptr.alloc((c.nrows + 1) * 4, &s.footprint);
  k_new_rowptr<<<nblk(c.nrows + 1), TPB, 0, st>>>(c.row_ptr.as<uint32_t>(), c.nrows, scan,
                                                  n2.row_ptr.as<uint32_t>());
  Tmp<uint32_t> dest(ne, st);
  k_compact_dest<<<nblk(ne), TPB, 0, st>>>(keep, scan, ne, dest.p);
  uint64_t alloc_n = std::max<uint64_t>(newtotal, 1);
  if (c.src.p) {
    n2.src.alloc(alloc_n * 4, &s.footprint);
    scatter_column(4, c.src.p, nullptr, dest.p, ne, n2.src.p, st);
  }
  if (c.src_type.p) {
    n2.src_type.alloc(alloc_n, &s.footprint);
    scatter_column(1, c.src_type.p, nullptr, dest.p, ne, n2.src_type.p, st);
  }
  n2.payload.resize(c.payload.size());
  for (size_t f = 0; f < c.payload.size(); f++) {
    n2.payload[f].alloc(alloc_n * ed.fields[f].size, &s.footprint);
    scatter_column(ed.fields[f].size, c.payload[f].p, nullptr, dest.p, ne, n2.payload[f].p, st);
  }
  n2.max_degree = csr_max_degree(s, c);
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaStreamSynchronize(st));
  c = std::move(n2);
}

void remove_died_edges(Sim &s, int died_type, const uint8_t *died,
                       uint64_t died_n) {
  s.csr_epoch++;
  cudaStream_t st = s.stream;
  for (size_t e = 0; e < s.edges.size(); e++) {
    EdgeStore &es = s.edges[e];
    const EdgeTypeDesc &ed = s.model->et((int)e);
    if (es.implicit) continue;
    for (int T = 1; T < (int)es.csr.size(); T++) {
      CSR &c = es.csr[T];
      if (c.nedges == 0) continue;
      bool tgt = (T == died_type);
      bool srcchk = ed.stores_src() &&
                    (c.src_type_const == died_type || c.src_type_const < 0);
      if (!tgt && !srcchk) continue;
      uint64_t ne = c.nedges;
      Tmp<uint32_t> keep(ne + 1, st), scan(ne + 1, st);
      VG_CUDA(cudaMemsetAsync(keep.p + ne, 0, 4, st));
      k_keep_flags<<<nblk(c.nrows), TPB, 0, st>>>(
          c.row_ptr.as<uint32_t>(), c.nrows, c.src.as<uint32_t>(),
          c.src_type.as<uint8_t>(), c.src_type_const, died, died_n, died_type,
          tgt ? 1 : 0, srcchk ? 1 : 0, keep.p);
      exclusive_scan_u32(keep.p, scan.p, ne + 1, st, s);
      uint32_t newtotal = 0;
      VG_CUDA(cudaMemcpyAsync(&newtotal, scan.p + ne, 4, cudaMemcpyDeviceToHost, st));
      VG_CUDA(cudaStreamSynchronize(st));
      if (newtotal == ne) continue;
      compact_csr(s, ed, c, keep.p, scan.p, newtotal);
    }
  }
}

namespace {
// remove_edges! records sorted by (to, from); from = REMOVE_ALL sorts last
struct RemovalTable {
  const uint64_t *to, *from, *key;
  uint64_t n;
};

__device__ uint64_t removal_key(const RemovalTable &R, uint64_t to, uint64_t from) {
  uint64_t lo = 0, hi = R.n;
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (R.to[mid] < to || (R.to[mid] == to && R.from[mid] < from)) lo = mid + 1;
    else hi = mid;
  }
  uint64_t mx = 0;
  for (uint64_t k = lo; k < R.n && R.to[k] == to && R.from[k] == from; k++)
    mx = R.key[k] > mx ? R.key[k] : mx;
  return mx;
}

// an edge (to, from) added with key k is gone when a later removal hit it
__device__ __forceinline__ bool removed_edge(const RemovalTable &R, uint64_t to, uint64_t from,
                                             uint64_t k, bool has_from) {
  if (removal_key(R, to, REMOVE_ALL) > k) return true;
  return has_from && removal_key(R, to, from) > k;
}

__global__ void k_removal_keep_old(const uint32_t *rp, uint64_t nrows, const uint32_t *src,
                                   const uint8_t *src_type, int src_type_const, int target_type,
                                   RemovalTable R, uint32_t *keep) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const uint64_t to = ((uint64_t)target_type << SHIFT_TYPE) | (r + 1);
  for (uint32_t k = rp[r]; k < rp[r + 1]; k++) {
    uint64_t from = REMOVE_ALL;
    if (src) {
      int ty = src_type ? (int)src_type[k] : src_type_const;
      from = ((uint64_t)ty << SHIFT_TYPE) | ((uint64_t)src[k] + 1);
    }
    keep[k] = removed_edge(R, to, from, 0, src != nullptr) ? 0u : 1u;
  }
}

__global__ void k_removal_keep_new(const uint64_t *to, const uint64_t *from, const uint64_t *key,
                                   uint64_t n, int has_from, RemovalTable R, uint32_t *keep) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keep[i] = removed_edge(R, to[i], from[i], key[i] + 1, has_from != 0) ? 0u : 1u;
}

__global__ void k_gather_u64(const uint64_t *in, const uint32_t *perm, uint64_t n, uint64_t *out) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[perm[i]];
}
}  // namespace

void apply_edge_removals(Sim &s, int e, EdgeRemoval &rm, EdgeAppend *ap, uint64_t &n_records,
                         bool merge_existing) {
  s.csr_epoch++;
  cudaStream_t st = s.stream;
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  uint64_t r = 0;
  VG_CUDA(cudaMemcpyAsync(&r, rm.counter.p, 8, cudaMemcpyDeviceToHost, st));
  VG_CUDA(cudaStreamSynchronize(st));
  if (r > rm.cap) fail(VG_ERR_DEVICE, "remove_edges! record buffer overflow");
  if (r == 0) return;
  if (r >= (1ull << 31)) fail(VG_ERR_NOMEM, "more than 2^31 remove_edges! calls in one apply!");
  // the table sorted by (to, from): stable LSD passes, from first
  Tmp<uint32_t> perm(r, st);
  k_iota<<<nblk(r), TPB, 0, st>>>(perm.p, r);
  Tmp<uint64_t> k1(r, st), tto(r, st), tfrom(r, st), tkey(r, st);
  k_copy_u64<<<nblk(r), TPB, 0, st>>>(rm.from.as<uint64_t>(), k1.p, r);
  radix_sort_pairs_u64(k1.p, perm.p, r, 64, st, s);
  k_gather_u64<<<nblk(r), TPB, 0, st>>>(rm.to.as<uint64_t>(), perm.p, r, tto.p);
  radix_sort_pairs_u64(tto.p, perm.p, r, 64, st, s);
  k_gather_u64<<<nblk(r), TPB, 0, st>>>(rm.from.as<uint64_t>(), perm.p, r, tfrom.p);
  k_gather_u64<<<nblk(r), TPB, 0, st>>>(rm.key.as<uint64_t>(), perm.p, r, tkey.p);
  VG_CUDA(cudaGetLastError());
  RemovalTable R{tto.p, tfrom.p, tkey.p, r};
  // the old edges that add_existing carries over
  if (merge_existing) {
    for (int T = 1; T < (int)es.csr.size(); T++) {
      CSR &c = es.csr[T];
      if (c.nedges == 0 || !c.row_ptr.p) continue;
      uint64_t ne = c.nedges;
      Tmp<uint32_t> keep(ne + 1, st), scan(ne + 1, st);
      VG_CUDA(cudaMemsetAsync(keep.p + ne, 0, 4, st));
      k_removal_keep_old<<<nblk(c.nrows), TPB, 0, st>>>(
          c.row_ptr.as<uint32_t>(), c.nrows, ed.stores_src() ? c.src.as<uint32_t>() : nullptr,
          c.src_type.as<uint8_t>(), c.src_type_const, T, R, keep.p);
      exclusive_scan_u32(keep.p, scan.p, ne + 1, st, s);
      uint32_t newtotal = 0;
      VG_CUDA(cudaMemcpyAsync(&newtotal, scan.p + ne, 4, cudaMemcpyDeviceToHost, st));
      VG_CUDA(cudaStreamSynchronize(st));
      if (newtotal != ne) compact_csr(s, ed, c, keep.p, scan.p, newtotal);
    }
  }
  // the edges appended in this transition
  if (ap && n_records > 0) {
    if (ap->key.p == nullptr)
      fail(VG_ERR_ARG, "remove_edges! with edges appended in a fixed order is not supported");
    uint64_t n = n_records;
    Tmp<uint32_t> keep(n + 1, st), scan(n + 1, st);
    VG_CUDA(cudaMemsetAsync(keep.p + n, 0, 4, st));
    k_removal_keep_new<<<nblk(n), TPB, 0, st>>>(ap->to.as<uint64_t>(), ap->from.as<uint64_t>(),
                                                ap->key.as<uint64_t>(), n,
                                                ed.stores_src() ? 1 : 0, R, keep.p);
    exclusive_scan_u32(keep.p, scan.p, n + 1, st, s);
    uint32_t kept = 0;
    VG_CUDA(cudaMemcpyAsync(&kept, scan.p + n, 4, cudaMemcpyDeviceToHost, st));
    VG_CUDA(cudaStreamSynchronize(st));
    if (kept != n) {
      Tmp<uint32_t> dest(n, st);
      k_compact_dest<<<nblk(n), TPB, 0, st>>>(keep.p, scan.p, n, dest.p);
      auto squeeze = [&](DevBuf &b, int esz) {
        DevBuf nb;
        nb.alloc(std::max<uint64_t>(kept, 1) * esz, &s.footprint);
        scatter_column(esz, b.p, nullptr, dest.p, n, nb.p, st);
        b = std::move(nb);
      };
      squeeze(ap->to, 8);
      squeeze(ap->from, 8);
      squeeze(ap->key, 8);
      for (size_t f = 0; f < ap->payload.size(); f++) squeeze(ap->payload[f], ed.fields[f].size);
      ap->cap = std::max<uint64_t>(kept, 1);
      VG_CUDA(cudaGetLastError());
      VG_CUDA(cudaStreamSynchronize(st));
      n_records = kept;
    }
  }
}

namespace {
__device__ __forceinline__ uint32_t row_degree(const uint32_t *rp, uint64_t nrows, uint64_t r) {
  return r < nrows ? rp[r + 1] - rp[r] : 0u;
}

// flag rows with lo < degree <= hi
__global__ void k_flag_degree(const uint32_t *rp, uint64_t nrows, uint64_t n, uint32_t lo,
                              uint32_t hi, uint32_t *flag) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  uint32_t d = row_degree(rp, nrows, r);
  flag[r] = (d > lo && d <= hi) ? 1u : 0u;
}

__global__ void k_compact_rows(const uint32_t *flag, const uint32_t *pos, uint64_t n,
                               uint32_t *rows) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n && flag[r]) rows[pos[r]] = (uint32_t)r;
}

// sort key of a hub row: descending degree
__global__ void k_count_above(const uint32_t *rp, const uint32_t *rows, uint64_t m,
                              uint32_t thr, unsigned *cnt) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m && rp[rows[k] + 1] - rp[rows[k]] > thr) atomicAdd(cnt, 1u);
}

__global__ void k_hub_keys(const uint32_t *rp, const uint32_t *rows, uint64_t m, uint32_t *keys) {
  uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) keys[k] = 0xFFFFFFFFu - (rp[rows[k] + 1] - rp[rows[k]]);
}

// order keys: rows with degree <= cap by window, then descending degree
// (stable sort: ties by index); the others sort last
__global__ void k_order_keys(const uint32_t *rp, uint64_t nrows, uint64_t n, uint32_t cap,
                             uint32_t wshift, uint32_t *keys, uint32_t *vals) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  uint32_t d = row_degree(rp, nrows, r);
  keys[r] = d > cap ? 0xFFFFFFFFu : (((uint32_t)(r >> wshift) << 16) | (0xFFFFu - min(d, 0xFFFFu)));
  vals[r] = (uint32_t)r;
}




// largest degree of each slice of 32 order positions
__global__ void k_slice_deg(const uint32_t *rp, uint64_t nrows, const uint32_t *order, uint64_t m,
                            uint64_t nslices, uint32_t *sdeg, uint64_t *slots) {
  uint64_t sl = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (sl >= nslices) return;
  uint32_t dm = 0;
  for (uint64_t k = sl * 32; k < min(m, sl * 32 + 32); k++)
    dm = max(dm, row_degree(rp, nrows, order[k]));
  sdeg[sl] = dm;
  slots[sl] = 32ull * dm;
}

// copy each row's edges into its slice, column-major; padding source 0,
// weight 0
__global__ void k_sell_fill(const uint32_t *__restrict__ rp, uint64_t nrows,
                            const uint32_t *__restrict__ src, const double *__restrict__ w,
                            const uint32_t *__restrict__ order, uint64_t m,
                            const uint64_t *__restrict__ base, const uint32_t *__restrict__ sdeg,
                            uint32_t *__restrict__ ssrc, double *__restrict__ sw) {
  uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t nslices_pos = (m + 31) / 32 * 32;
  if (k >= nslices_pos) return;
  const uint64_t sl = k >> 5, lane = k & 31;
  uint32_t b = 0, d = 0;
  if (k < m) {
    uint32_t r = order[k];
    if (r < nrows) {
      b = rp[r];
      d = rp[r + 1] - b;
    }
  }
  const uint64_t o = base[sl] + lane;
  const uint32_t D = sdeg[sl];
  // (the columns do not overlap the CSR: each lane's loads of a round are
  // in flight together)
#pragma unroll 4
  for (uint32_t q = 0; q < D; q++) {
    ssrc[o + 32ull * q] = q < d ? src[b + q] : 0u;
    sw[o + 32ull * q] = q < d ? w[b + q] : 0.0;
  }
}

// rows with lo < degree <= hi, in index order
uint64_t select_rows(Sim &s, const CSR &c, uint64_t n, uint32_t lo, uint32_t hi, DevBuf &out) {
  cudaStream_t st = s.stream;
  Tmp<uint32_t> flag(n + 1, st), pos(n + 1, st);
  VG_CUDA(cudaMemsetAsync(flag.p + n, 0, 4, st));
  k_flag_degree<<<nblk(n), TPB, 0, st>>>(c.row_ptr.as<uint32_t>(), c.nrows, n, lo, hi, flag.p);
  exclusive_scan_u32(flag.p, pos.p, n + 1, st, s);
  uint32_t m = 0;
  VG_CUDA(cudaMemcpyAsync(&m, pos.p + n, 4, cudaMemcpyDeviceToHost, st));
  VG_CUDA(cudaStreamSynchronize(st));
  if (m) {
    out.alloc((uint64_t)m * 4, &s.footprint);
    k_compact_rows<<<nblk(n), TPB, 0, st>>>(flag.p, pos.p, n, out.as<uint32_t>());
    VG_CUDA(cudaGetLastError());
  }
  return m;
}
}  // namespace

// in-degree of the row at each position of the slice order
__global__ void k_order_deg(const uint32_t *rp, uint64_t nrows, const uint32_t *order,
                            uint64_t m, uint32_t *deg) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) deg[k] = row_degree(rp, nrows, order[k]);
}

void ensure_schedule(Sim &s, CSR &c, uint32_t thr, uint32_t big_thr, uint64_t n) {
  if (c.schedule_valid && c.hub_threshold == thr && c.block_threshold == big_thr &&
      c.sched_n == n)
    return;
  cudaStream_t st = s.stream;
  c.hub_rows.release();
  c.order.release();
  c.order_deg.release();
  c.slice_base.release();
  c.slice_deg.release();
  c.sell_src.release();
  c.sell_w.release();
  c.nhub = c.norder = c.nslices = c.nbig = 0;
  c.range_block.clear();
  c.range_rows.clear();
  c.range_window.clear();
  c.hub_rows_sorted.clear();
  if (n > 0 && c.row_ptr.p) {
    const uint32_t *rp = c.row_ptr.as<uint32_t>();
    // hub rows by descending degree
    c.nhub = select_rows(s, c, n, thr, 0xFFFFFFFFu, c.hub_rows);
    if (c.nhub > 1) {
      Tmp<uint32_t> keys(c.nhub, st);
      k_hub_keys<<<nblk(c.nhub), TPB, 0, st>>>(rp, c.hub_rows.as<uint32_t>(), c.nhub, keys.p);
      radix_sort_pairs_u32(keys.p, c.hub_rows.as<uint32_t>(), c.nhub, 32, st, s);
    }
    c.nbig = 0;
    if (c.nhub && big_thr != 0xFFFFFFFFu) {  // the leading hubs above the block threshold
      Tmp<unsigned> cnt(1, st);
      VG_CUDA(cudaMemsetAsync(cnt.p, 0, 4, st));
      k_count_above<<<nblk(c.nhub), TPB, 0, st>>>(rp, c.hub_rows.as<uint32_t>(), c.nhub,
                                                  big_thr, cnt.p);
      unsigned h = 0;
      VG_CUDA(cudaMemcpyAsync(&h, cnt.p, 4, cudaMemcpyDeviceToHost, st));
      VG_CUDA(cudaStreamSynchronize(st));
      c.nbig = h;
    }
    // the other rows by descending degree in windows of 2^13 rows (or
    // more, so that the window number stays below the sentinel)
    uint32_t wshift = 13;
    while ((n >> wshift) >= 0xFFFFull) wshift++;
    c.wshift = wshift;
    Tmp<uint32_t> keys(n, st);
    c.order.alloc(n * 4, &s.footprint);
    k_order_keys<<<nblk(n), TPB, 0, st>>>(rp, c.nrows, n, thr, wshift, keys.p,
                                          c.order.as<uint32_t>());
    radix_sort_pairs_u32(keys.p, c.order.as<uint32_t>(), n, 32, st, s);
    const uint64_t m = n - c.nhub;
    c.norder = m;
    const uint64_t ns = (m + 31) / 32;
    c.nslices = ns;
    if (ns > 0) {
      c.slice_deg.alloc(ns * 4, &s.footprint);
      c.slice_base.alloc((ns + 1) * 8, &s.footprint);
      Tmp<uint64_t> slots(ns + 1, st);
      VG_CUDA(cudaMemsetAsync(slots.p + ns, 0, 8, st));
      k_slice_deg<<<nblk(ns), TPB, 0, st>>>(rp, c.nrows, c.order.as<uint32_t>(), m, ns,
                                            c.slice_deg.as<uint32_t>(), slots.p);
      exclusive_scan_u64(slots.p, c.slice_base.as<uint64_t>(), ns + 1, st, s);
      uint64_t total = 0;
      VG_CUDA(cudaMemcpyAsync(&total, c.slice_base.as<uint64_t>() + ns, 8, cudaMemcpyDeviceToHost,
                              st));
      VG_CUDA(cudaStreamSynchronize(st));
      c.sell_src.alloc(std::max<uint64_t>(total, 1) * 4, &s.footprint);
      c.sell_w.alloc(std::max<uint64_t>(total, 1) * 8, &s.footprint);
      k_sell_fill<<<nblk(ns * 32), TPB, 0, st>>>(
          rp, c.nrows, c.src.as<uint32_t>(), c.payload[0].as<double>(), c.order.as<uint32_t>(), m,
          c.slice_base.as<uint64_t>(), c.slice_deg.as<uint32_t>(), c.sell_src.as<uint32_t>(),
          c.sell_w.as<double>());
      c.order_deg.alloc(std::max<uint64_t>(m, 1) * 4, &s.footprint);
      k_order_deg<<<nblk(m), TPB, 0, st>>>(rp, c.nrows, c.order.as<uint32_t>(), m,
                                           c.order_deg.as<uint32_t>());
    }
    VG_CUDA(cudaGetLastError());
    VG_CUDA(cudaStreamSynchronize(st));
  }
  c.sched_n = n;
  c.hub_threshold = thr;
  c.block_threshold = big_thr;
  c.schedule_valid = true;
}

}  // namespace vg
