// Batched ensemble: many independent SIR simulations stepped together.
//
// Each instance is built as an ordinary simulation (the "SIR" model:
// Person{state::UInt8, days::Int32} :Immortal, Contact :Stateless
// :SingleType), with its own seeded graph, and then packed into one device
// arena: the instances' CSRs concatenated (row pointers and source indices
// offset by the instance's first agent), states concatenated, one row of
// the infection-probability table per instance.  One kernel launch steps
// every agent of every instance (per-instance parameters looked up from the
// agent's instance), so a step costs one launch instead of one per
// instance; the step loop can be captured once in a CUDA graph and
// replayed.  Neighbour states are read from a bit mask of the infected
// agents that every step writes beside the states.  Two persistent forms run
// every step in one launch: a cooperative grid whose block tickets wait
// only for the instances they touch (no grid-wide barrier), and
// thread-block clusters that each step their own packs of
// whole instances (masks in distributed shared memory, cluster barriers).
// A small autotuner keyed on the arena's degree histogram picks the form and
// its shape (block size, agents per lane, degree buckets, cluster size) by
// timing them.
//
// The plain path of the same instances (vg_batch_step_one) runs apply! on
// the instance's own simulation; both paths produce bit-identical states.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "vg_internal.h"
#include "vg_philox.cuh"

namespace vg {
void set_last_error(const std::string &m);

namespace {

struct BatchArgs {
  const uint32_t *__restrict__ rp;      // global row pointers (agents + 1)
  const uint32_t *__restrict__ src;     // global source agent index
  const uint16_t *__restrict__ inst;    // instance of each agent
  const uint64_t *__restrict__ base;    // first global agent of each instance
  const double *__restrict__ ptab;      // [instance][k], k <= kmax
  const int32_t *__restrict__ rec;      // recovery steps per instance
  const uint64_t *__restrict__ seed;    // seed per instance
  const uint8_t *__restrict__ st_rd;
  const int32_t *__restrict__ d_rd;
  const uint32_t *__restrict__ inf_rd;  // bit i: agent i infected in st_rd
  uint8_t *__restrict__ st_wr;
  int32_t *__restrict__ d_wr;
  uint32_t *__restrict__ inf_wr;        // bit i: agent i infected in st_wr
  uint64_t n;
  uint32_t kmax1;  // table row length
  uint32_t step;   // transition number, plus *step_base when step_base is set
  const int64_t *step_base;
  int *status;
};

// The neighbour reads of a step need one bit per agent (infected or not):
// the step's kernels write, beside the states, a bit mask of the infected
// agents (one 32-bit word per 32 agents, formed by a warp ballot), and the
// next step gathers from the mask instead of the state bytes.  An
// instance's mask is at most 12.5 KB (10^5 agents), so the neighbour reads
// of the blocks stepping it stay in L1.  The count k is the same integer
// whichever form is read.
__device__ __forceinline__ uint32_t inf_bit(const uint32_t *m, uint32_t j) {
  return (m[j >> 5] >> (j & 31)) & 1u;
}

// the rule of transition "sir" for agent i with k infected in-neighbours;
// returns the new state
__device__ __forceinline__ uint8_t sir_rule(const BatchArgs &a, uint64_t i, uint32_t k, uint8_t s,
                                            int32_t d, uint32_t step, uint8_t *st_wr,
                                            int32_t *d_wr) {
  const uint32_t in = a.inst[i];
  if (s == 0) {
    if (k > 0) {
      if (k >= a.kmax1) {
        atomicCAS(a.status, 0, 402);
      } else {
        const uint64_t nr = i - a.base[in] + 1;
        if (unit_below(philox_u64(philox_draw(a.seed[in], nr, step, TAG_INFECT)),
                       a.ptab[(uint64_t)in * a.kmax1 + k])) {
          s = 1;
          d = 0;
        }
      }
    }
  } else if (s == 1) {
    d = d + 1;
    if (d >= a.rec[in]) s = 2;
  }
  st_wr[i] = s;
  d_wr[i] = d;
  return s;
}

// source loads of one row per round of a lane's row walk
constexpr int ROW_UNROLL = 2;

// One warp steps the ILP * 32 agents c0 .. c0 + 32 ILP - 1 (c0 a multiple of
// 32): lane l takes agents c0 + 32 u + l, u < ILP, and walks their rows
// together, ROW_UNROLL edges of each per round, so that ROW_UNROLL ILP
// source loads (and then as many mask loads) are in flight at once.  Agents flagged in `skip`
// are left to other warps (their bits too).  With `atomic_bits` the mask
// words are updated bit by bit (other warps own some of their bits);
// otherwise each word is stored whole.
template <int ILP>
__device__ __forceinline__ void sir_chunk(const BatchArgs &a, const uint8_t *st_rd,
                                          const int32_t *d_rd, const uint32_t *inf_rd,
                                          uint8_t *st_wr, int32_t *d_wr, uint32_t *inf_wr,
                                          uint64_t c0, uint32_t step, const uint8_t *skip,
                                          bool atomic_bits) {
  const unsigned lane = threadIdx.x & 31;
  uint8_t s[ILP];
  int32_t d[ILP];
  uint32_t q[ILP], e[ILP], k[ILP];
  bool live[ILP];
#pragma unroll
  for (int u = 0; u < ILP; u++) {
    const uint64_t i = c0 + 32u * u + lane;
    live[u] = i < a.n && !(skip && skip[i]);
    s[u] = live[u] ? st_rd[i] : (uint8_t)3;
    d[u] = live[u] ? d_rd[i] : 0;
    k[u] = 0;
    q[u] = e[u] = 0;
    if (s[u] == 0) {
      q[u] = a.rp[i];
      e[u] = a.rp[i + 1];
    }
  }
  constexpr uint32_t NONE = 0xFFFFFFFFu;
  for (;;) {
    uint32_t j[ILP][ROW_UNROLL], w[ILP][ROW_UNROLL];
    bool more = false;
#pragma unroll
    for (int u = 0; u < ILP; u++) {
#pragma unroll
      for (int r = 0; r < ROW_UNROLL; r++) j[u][r] = q[u] + r < e[u] ? a.src[q[u] + r] : NONE;
      more |= q[u] < e[u];
    }
    if (!more) break;
#pragma unroll
    for (int u = 0; u < ILP; u++)
#pragma unroll
      for (int r = 0; r < ROW_UNROLL; r++) w[u][r] = j[u][r] != NONE ? inf_rd[j[u][r] >> 5] : 0u;
#pragma unroll
    for (int u = 0; u < ILP; u++) {
#pragma unroll
      for (int r = 0; r < ROW_UNROLL; r++)
        if (j[u][r] != NONE) k[u] += (w[u][r] >> (j[u][r] & 31)) & 1u;
      q[u] = q[u] + ROW_UNROLL < e[u] ? q[u] + ROW_UNROLL : e[u];
    }
  }
#pragma unroll
  for (int u = 0; u < ILP; u++) {
    const uint64_t i0 = c0 + 32u * u;
    if (i0 >= a.n) break;  // warp-uniform
    uint8_t ns = 3;
    if (live[u]) ns = sir_rule(a, i0 + lane, k[u], s[u], d[u], step, st_wr, d_wr);
    const unsigned set = __ballot_sync(0xffffffffu, live[u] && ns == 1);
    if (atomic_bits) {
      const unsigned clr = __ballot_sync(0xffffffffu, live[u] && ns != 1);
      if (lane == 0) {
        if (set) atomicOr(inf_wr + (i0 >> 5), set);
        if (clr) atomicAnd(inf_wr + (i0 >> 5), ~clr);
      }
    } else if (lane == 0) {
      inf_wr[i0 >> 5] = set;
    }
  }
}

// per-step form: warp w steps agents [32 ILP w, 32 ILP (w + 1))
template <int ILP>
__global__ void k_batch_sir(BatchArgs a) {
  if (a.step_base) a.step += (uint32_t)*a.step_base;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t c0 = warp * 32 * ILP;
  if (c0 >= a.n) return;
  sir_chunk<ILP>(a, a.st_rd, a.d_rd, a.inf_rd, a.st_wr, a.d_wr, a.inf_wr, c0, a.step, nullptr,
                 false);
}

// the infected-agent mask of a state array
__global__ void k_inf_bits(const uint8_t *st, uint64_t n, uint32_t *m) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t i0 = i & ~31ull;
  if (i0 >= n) return;  // warp-uniform
  const unsigned b = __ballot_sync(0xffffffffu, i < n && st[i] == 1);
  if ((threadIdx.x & 31) == 0) m[i0 >> 5] = b;
}

// ---- persistent form: one cooperative launch runs every step.  Agents are
// taken in block tickets, numbered across the steps (ticket T: step T /
// tickets_per_step, agent range T % tickets_per_step); all blocks are
// resident (the launch is cooperative) and tickets are handed out in step
// order.  An agent reads only its own instance's agents, so a ticket of step
// t waits only until the instances its range touches have finished step t - 1
// (no grid-wide barrier): every block that finishes a range adds, per
// instance, the number of its agents in the range to that instance's
// counter of agent-steps (after a release fence), and a ticket of step t
// waits until the counter of each of its instances reaches t * N_i (an
// acquire load; bounded: a wait that runs out records BAR_ERR_WAIT and the
// launch winds down).  Finishing step t - 1 of an instance also ends every
// read of step t - 1's read buffer by that instance, so step t may write it.
// States and masks written by other blocks are read with ordinary loads
// after the acquire (never through the read-only path, which assumes data
// constant for the whole launch).  Agents above a degree threshold (listed
// in `heavy`, sorted) are folded by a warp each, inside the ticket of their
// range (the infected-neighbour count is an integer: any order gives the
// same k); the others in warp chunks as in the per-step form.
struct PersistArgs {
  BatchArgs a;                 // graph, tables; state pointers unused
  uint8_t *st[2];
  int32_t *dy[2];
  uint32_t *inf[2];
  int cur0;                    // buffer of the state before the first step
  uint32_t steps, step0;       // steps to run, transition number of the first
  const uint32_t *heavy;       // agents above the bucket threshold (nheavy, ascending)
  uint64_t nheavy;
  const uint8_t *is_heavy;     // per agent (null: no heavy agents)
  unsigned *ticket;            // next ticket (zero at launch)
  uint32_t *done;              // per instance: agent-steps finished in this launch (zero at launch)
  const uint32_t *inst_n;      // per instance: agents
  unsigned rounds;             // chunk rounds per block ticket
};

constexpr uint32_t BAR_SPIN_LIMIT = 1u << 22;
constexpr int BAR_ERR_WAIT = 0x5e04;

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t *a) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
  return v;
}

// bounded wait until *counter >= target; false (and the status word set)
// when it runs out or another wait already gave up
__device__ bool wait_count(const uint32_t *counter, uint32_t target, int *status,
                           uint32_t limit = BAR_SPIN_LIMIT) {
  for (uint32_t i = 0; i < limit; i++) {
    if (ld_acquire_gpu(counter) >= target) return true;
    if ((i & 1023u) == 1023u && *(volatile int *)status) return false;
    if (i > 64) __nanosleep(32);
  }
  atomicCAS(status, 0, BAR_ERR_WAIT);
  return false;
}

// failure detection without a fault: the blocks wait for an instance
// counter that nothing advances, so every wait runs out
__global__ void k_barrier_probe(const uint32_t *counter, uint32_t target, int *status,
                                uint32_t limit) {
  if (threadIdx.x == 0) wait_count(counter, target, status, limit);
}

template <int ILP>
__global__ void k_batch_persist(PersistArgs p) {
  __shared__ unsigned s_ticket;
  __shared__ int s_ok;
  const BatchArgs &a = p.a;
  const unsigned lane = threadIdx.x & 31;
  const unsigned wpb = blockDim.x / 32, wib = threadIdx.x / 32;
  const bool atomic_bits = p.is_heavy != nullptr;
  const uint64_t span = (uint64_t)wpb * 32 * ILP * p.rounds;
  const uint64_t tps = (a.n + span - 1) / span;  // tickets per step
  const uint64_t total = tps * p.steps;
  for (;;) {
    if (threadIdx.x == 0) s_ticket = atomicAdd(p.ticket, 1u);
    __syncthreads();
    const uint64_t T = s_ticket;
    __syncthreads();
    if (T >= total) break;
    const uint32_t t = (uint32_t)(T / tps);
    const uint64_t a0 = (T % tps) * span;
    const uint64_t a1 = a0 + span < a.n ? a0 + span : a.n;
    const uint32_t i0 = a.inst[a0], i1 = a.inst[a1 - 1];
    // the range's instances have finished step t - 1
    if (threadIdx.x == 0) {
      s_ok = !*(volatile int *)a.status;
      for (uint32_t i = i0; t > 0 && s_ok && i <= i1; i++)
        s_ok = wait_count(p.done + i, t * p.inst_n[i], a.status);
      asm volatile("fence.acq_rel.gpu;" ::: "memory");
    }
    __syncthreads();
    if (!s_ok) break;  // a wait gave up: the launch winds down
    const int cur = p.cur0 ^ (int)(t & 1);
    const uint8_t *st_rd = p.st[cur];
    const int32_t *d_rd = p.dy[cur];
    const uint32_t *inf_rd = p.inf[cur];
    uint8_t *st_wr = p.st[1 - cur];
    int32_t *d_wr = p.dy[1 - cur];
    uint32_t *inf_wr = p.inf[1 - cur];
    const uint32_t step = p.step0 + t;
    for (uint64_t c0 = a0 + (uint64_t)wib * 32 * ILP; c0 < a1; c0 += (uint64_t)wpb * 32 * ILP)
      sir_chunk<ILP>(a, st_rd, d_rd, inf_rd, st_wr, d_wr, inf_wr, c0, step, p.is_heavy,
                     atomic_bits);
    if (p.nheavy) {  // the range's heavy agents, a warp each
      uint64_t lo = 0, hi = p.nheavy;  // first heavy agent >= a0
      while (lo < hi) {
        const uint64_t mid = (lo + hi) / 2;
        if (p.heavy[mid] < a0) lo = mid + 1;
        else hi = mid;
      }
      for (uint64_t h = lo + wib; h < p.nheavy && p.heavy[h] < a1; h += wpb) {
        const uint64_t i = p.heavy[h];
        const uint8_t s = st_rd[i];
        const int32_t d = d_rd[i];
        uint32_t k = 0;
        if (s == 0) {
          const uint32_t e = a.rp[i + 1];
          for (uint32_t q = a.rp[i] + lane; q < e; q += 32) k += inf_bit(inf_rd, a.src[q]);
        }
        k = __reduce_add_sync(0xffffffffu, k);
        if (lane == 0) {
          const uint8_t ns = sir_rule(a, i, k, s, d, step, st_wr, d_wr);
          const unsigned bit = 1u << (i & 31);
          if (ns == 1)
            atomicOr(inf_wr + (i >> 5), bit);
          else
            atomicAnd(inf_wr + (i >> 5), ~bit);
        }
      }
    }
    __syncthreads();
    // the range's agents of each instance have finished step t
    if (threadIdx.x == 0) {
      __threadfence();
      for (uint32_t i = i0; i <= i1; i++) {
        const uint64_t b0 = a.base[i], b1 = b0 + p.inst_n[i];
        const uint64_t lo = a0 > b0 ? a0 : b0, hi = a1 < b1 ? a1 : b1;
        atomicAdd(p.done + i, (uint32_t)(hi - lo));
      }
    }
  }
}

// ---- persistent cluster form: instances never read each other's agents,
// so a pack of whole instances can run every step on its own.  The
// instances are packed (large ones alone, small ones together) and the
// packs ordered longest first (by edges and agents); each thread-block
// cluster of C CTAs takes the next pack from a counter, steps it through
// all the steps, then takes another.  Each CTA keeps the pack's
// infected-agent mask (one bit per agent, every instance padded to whole
// 32-agent words, two buffers) in its shared memory; the pack's 32-agent
// chunks are dealt statically to the cluster's warps, so an agent's
// own state and days are read and written by the same thread every step
// (plain global loads and stores, nothing crosses CTAs there).  A warp that
// has stepped a chunk forms the chunk's new mask word by a ballot and lanes
// 0..C-1 store it into the C CTAs' next buffers (distributed shared memory,
// st.shared::cluster); a hardware cluster barrier (arrive.release /
// wait.acquire) ends each step; the first one, before any such store, also
// makes sure that every CTA of the cluster has started.  No block waits on
// a flag, and no cluster waits for another.
struct ChunkDesc {
  uint32_t first;  // arena index of the chunk's first agent
  uint32_t word;   // its mask word in the pack
  uint32_t delta;  // pack bit of agent j = j + delta mod 2^32 (j in the chunk's instance)
  uint32_t n;      // agents in the chunk (32, or fewer at an instance's end)
};

// the packs of the instances for one cluster shape: G clusters launched
// (as many as fit the GPU at once), npacks packs in the order they are
// taken, their chunk lists and the mask size of the largest pack
struct ClusterPlan {
  unsigned G = 0;       // 0: the shape is not available (a pack's mask too large)
  uint32_t npacks = 0;
  uint32_t wmax = 0;
  size_t smem = 0;
  DevBuf chunks, cofs, ticket;
};

struct ClusterArgs {
  BatchArgs a;                  // graph, tables
  uint8_t *st[2];
  int32_t *dy[2];
  const ChunkDesc *chunks;      // pack k: chunks cofs[k] .. cofs[k + 1] - 1
  const uint32_t *cofs;
  uint32_t npacks;
  unsigned *ticket;             // next pack to take (zero at launch)
  uint32_t wmax;                // mask words of the largest pack
  int cur0;
  uint32_t steps, step0;
};

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
// every thread of every CTA of the cluster; shared-memory stores into other
// CTAs before it are visible to their loads after it
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// store v at the shared-memory location `local` of CTA `rank` of the cluster
__device__ __forceinline__ void st_cluster(const uint32_t *local, unsigned rank, uint32_t v) {
  const uint32_t la = (uint32_t)__cvta_generic_to_shared(local);
  uint32_t ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"(rank));
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(ra), "r"(v) : "memory");
}

template <int ILP>
__global__ void __launch_bounds__(512) k_batch_cluster(ClusterArgs p) {
  extern __shared__ uint32_t smask[];  // [2][wmax]
  __shared__ uint32_t s_pack;
  const BatchArgs &a = p.a;
  const unsigned csize = cluster_size(), crank = cluster_rank();
  const unsigned lane = threadIdx.x & 31;
  const unsigned wpc = blockDim.x / 32;
  const uint32_t cw = crank * wpc + threadIdx.x / 32, ncw = csize * wpc;
  constexpr uint32_t NONE = 0xFFFFFFFFu;
  cluster_sync();  // every CTA of the cluster runs before any stores into its shared memory
  for (;;) {
    // the next pack: taken by CTA 0, handed to every CTA of the cluster
    if (crank == 0 && threadIdx.x < csize) {
      uint32_t k = 0;
      if (threadIdx.x == 0) k = atomicAdd(p.ticket, 1u);
      k = __shfl_sync((1u << csize) - 1u, k, 0);
      st_cluster(&s_pack, threadIdx.x, k);
    }
    cluster_sync();
    const uint32_t pk = s_pack;
    if (pk >= p.npacks) break;  // the whole cluster
    const uint32_t c_lo = p.cofs[pk], c_hi = p.cofs[pk + 1];
    // the initial mask: every warp its chunks' words, into every CTA
    {
      const uint8_t *st0 = p.st[p.cur0];
      for (uint32_t c = c_lo + cw; c < c_hi; c += ncw) {
        const ChunkDesc D = p.chunks[c];
        const bool live = lane < D.n;
        const unsigned m = __ballot_sync(0xffffffffu, live && st0[D.first + lane] == 1);
        if (lane < csize) st_cluster(smask + D.word, lane, m);
      }
    }
    cluster_sync();
    for (uint32_t t = 0; t < p.steps; t++) {
      const int cur = p.cur0 ^ (int)(t & 1);
      const uint8_t *st_rd = p.st[cur];
      const int32_t *d_rd = p.dy[cur];
      uint8_t *st_wr = p.st[1 - cur];
      int32_t *d_wr = p.dy[1 - cur];
      const uint32_t *m_rd = smask + (t & 1) * p.wmax;
      uint32_t *m_wr = smask + ((t + 1) & 1) * p.wmax;
      const uint32_t step = p.step0 + t;
      for (uint32_t c0 = c_lo + cw * ILP; c0 < c_hi; c0 += ncw * ILP) {
        ChunkDesc D[ILP];
        uint8_t s[ILP];
        int32_t d[ILP];
        uint32_t q[ILP], e[ILP], k[ILP];
        bool live[ILP];
#pragma unroll
        for (int u = 0; u < ILP; u++) {
          const bool has = c0 + u < c_hi;
          D[u] = has ? p.chunks[c0 + u] : ChunkDesc{0, 0, 0, 0};
          live[u] = lane < D[u].n;
          const uint32_t i = D[u].first + lane;
          s[u] = live[u] ? st_rd[i] : (uint8_t)3;
          d[u] = live[u] ? d_rd[i] : 0;
          k[u] = 0;
          q[u] = e[u] = 0;
          if (s[u] == 0) {
            q[u] = a.rp[i];
            e[u] = a.rp[i + 1];
          }
        }
        for (;;) {
          uint32_t j[ILP][ROW_UNROLL];
          bool more = false;
#pragma unroll
          for (int u = 0; u < ILP; u++) {
#pragma unroll
            for (int r = 0; r < ROW_UNROLL; r++)
              j[u][r] = q[u] + r < e[u] ? a.src[q[u] + r] + D[u].delta : NONE;
            more |= q[u] < e[u];
          }
          if (!more) break;
#pragma unroll
          for (int u = 0; u < ILP; u++) {
#pragma unroll
            for (int r = 0; r < ROW_UNROLL; r++)
              if (j[u][r] != NONE) k[u] += (m_rd[j[u][r] >> 5] >> (j[u][r] & 31)) & 1u;
            q[u] = q[u] + ROW_UNROLL < e[u] ? q[u] + ROW_UNROLL : e[u];
          }
        }
#pragma unroll
        for (int u = 0; u < ILP; u++) {
          if (c0 + u >= c_hi) break;  // warp-uniform
          uint8_t ns = 3;
          if (live[u]) ns = sir_rule(a, D[u].first + lane, k[u], s[u], d[u], step, st_wr, d_wr);
          const unsigned m = __ballot_sync(0xffffffffu, live[u] && ns == 1);
          if (lane < csize) st_cluster(m_wr + D[u].word, lane, m);
        }
      }
      cluster_sync();
    }
  }
}

__global__ void k_offset_rp(const uint32_t *rp, uint64_t nrows, uint32_t ebase, uint32_t *out) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r <= nrows) out[r] = rp[r] + ebase;
}
__global__ void k_offset_src(const uint32_t *src, uint64_t ne, uint32_t abase, uint32_t *out) {
  uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < ne) out[k] = src[k] + abase;
}
__global__ void k_fill_u16(uint16_t *p, uint64_t n, uint16_t v) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

inline unsigned blocks(uint64_t n, int tpb) {
  return (unsigned)std::max<uint64_t>((n + tpb - 1) / tpb, 1);
}

}  // namespace

// initial state of an SIR instance: the n_inf agents with the smallest
// Philox(seed, nr, 0, TAG_INIT) draw (ties by index) start infected
void sir_initial_state(uint64_t n, uint64_t seed, uint64_t n_inf, std::vector<uint8_t> &state) {
  std::vector<std::pair<uint64_t, uint64_t>> d(n);
  for (uint64_t i = 0; i < n; i++) d[i] = {philox_u64(philox_draw(seed, i + 1, 0, TAG_INIT)), i};
  n_inf = std::min(n_inf, n);
  std::partial_sort(d.begin(), d.begin() + n_inf, d.end());
  state.assign(n, 0);
  for (uint64_t j = 0; j < n_inf; j++) state[d[j].second] = 1;
}

}  // namespace vg

using namespace vg;

struct vg_batch {
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int n = 0;
  std::vector<int64_t> N;
  std::vector<int32_t> deg, rec;
  std::vector<double> beta;
  std::vector<uint64_t> seed;
  vg_model *model = nullptr;
  std::vector<vg_sim *> sims;
  int person = 0, contact = 0;
  uint64_t total = 0, total_edges = 0;
  uint64_t footprint = 0;
  DevBuf rp, src, inst, base, ptab, rec_d, seed_d, st[2], dy[2], inf[2], status;
  uint32_t kmax1 = 0;
  int cur = 0;
  int64_t step = 1;  // transition number of the next step (as after finish_init!)
  int tpb = 256, apt = 1;
  bool tuned = false;
  struct Tuned {
    int tpb, apt, p_tpb, p_ilp, p_rounds;
    uint32_t p_thr;
    int c_ctas, c_tpb, c_ilp, form;
    float graph_ms, persistent_ms, cluster_ms;
  };
  std::map<uint64_t, Tuned> tune_cache;
  // persistent form: block size, bucket threshold (agents with more
  // in-edges take a warp each; 0xFFFFFFFF: none) and whether the autotuner
  // found it faster than the graph of per-step launches
  int p_tpb = 256, p_ilp = 2, p_rounds = 4;  // (and agents per lane, chunk rounds per ticket)
  uint32_t p_thr = 0xFFFFFFFFu;
  // cluster form: CTAs per cluster, threads per CTA, agents per lane; its
  // packings by shape
  int c_ctas = 8, c_tpb = 512, c_ilp = 1;
  std::map<int, ClusterPlan> cplans;
  std::vector<uint64_t> host_base;  // first arena agent of each instance
  int form = 1;  // mode 3 runs: 1 graph replay, 2 persistent grid, 4 persistent clusters
  float tuned_graph_ms = 0, tuned_persistent_ms = 0, tuned_cluster_ms = 0;  // best trials
  std::vector<uint32_t> host_rp;       // arena row pointers (autotuner, buckets)
  uint32_t heavy_thr = 0xFFFFFFFFu;    // threshold the heavy list was built for
  DevBuf heavy, is_heavy, bar;
  DevBuf done, inst_n;  // persistent form: agent-steps finished per instance, agents per instance
  uint64_t nheavy = 0;
  DevBuf scratch_st[2], scratch_dy[2], scratch_inf[2];  // autotuner trials run on copies
  // CUDA graphs of `graph_steps` steps, one per starting buffer parity; the
  // step number comes from step_base (device) + the node's offset
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaGraph_t graph_def[2] = {nullptr, nullptr};
  int graph_steps = 0;
  DevBuf step_base;
};

namespace {

// the two state buffers (and their infected-agent masks) a launch steps between
struct StateBufs {
  uint8_t *st[2];
  int32_t *dy[2];
  uint32_t *inf[2];
};

StateBufs arena_bufs(vg_batch *b) {
  return {{b->st[0].as<uint8_t>(), b->st[1].as<uint8_t>()},
          {b->dy[0].as<int32_t>(), b->dy[1].as<int32_t>()},
          {b->inf[0].as<uint32_t>(), b->inf[1].as<uint32_t>()}};
}

// mask words: one per 32 agents, rounded up to whole chunks of the widest
// warp chunk (4 x 32 agents)
inline uint64_t mask_words(uint64_t n) { return (n + 127) / 128 * 4; }

BatchArgs batch_args(vg_batch *b, int cur, uint32_t step, const int64_t *step_base) {
  BatchArgs a{};
  a.rp = b->rp.as<uint32_t>();
  a.src = b->src.as<uint32_t>();
  a.inst = b->inst.as<uint16_t>();
  a.base = b->base.as<uint64_t>();
  a.ptab = b->ptab.as<double>();
  a.rec = b->rec_d.as<int32_t>();
  a.seed = b->seed_d.as<uint64_t>();
  a.st_rd = b->st[cur].as<uint8_t>();
  a.d_rd = b->dy[cur].as<int32_t>();
  a.inf_rd = b->inf[cur].as<uint32_t>();
  a.st_wr = b->st[1 - cur].as<uint8_t>();
  a.d_wr = b->dy[1 - cur].as<int32_t>();
  a.inf_wr = b->inf[1 - cur].as<uint32_t>();
  a.n = b->total;
  a.kmax1 = b->kmax1;
  a.step = step;
  a.step_base = step_base;
  a.status = b->status.as<int>();
  return a;
}

void check_batch_status(vg_batch *b) {
  int h = 0;
  VG_CUDA(cudaMemcpyAsync(&h, b->status.p, 4, cudaMemcpyDeviceToHost, b->stream));
  VG_CUDA(cudaStreamSynchronize(b->stream));
  if (h) fail(VG_ERR_DEVICE, "batched SIR step: device status " + std::to_string(h));
}

// the heavy agents (in-degree > thr) of the arena, as a list and as flags
void build_buckets(vg_batch *b, uint32_t thr) {
  if (b->heavy_thr == thr && (thr == 0xFFFFFFFFu || b->is_heavy.p)) return;
  b->heavy_thr = thr;
  b->nheavy = 0;
  b->heavy.release();
  b->is_heavy.release();
  if (thr == 0xFFFFFFFFu) return;
  std::vector<uint32_t> h;
  std::vector<uint8_t> flag(b->total, 0);
  for (uint64_t i = 0; i < b->total; i++)
    if (b->host_rp[i + 1] - b->host_rp[i] > thr) {
      h.push_back((uint32_t)i);
      flag[i] = 1;
    }
  b->nheavy = h.size();
  b->is_heavy.alloc(std::max<uint64_t>(b->total, 1), &b->footprint);
  VG_CUDA(cudaMemcpyAsync(b->is_heavy.p, flag.data(), b->total, cudaMemcpyHostToDevice, b->stream));
  if (!h.empty()) {
    b->heavy.alloc(h.size() * 4, &b->footprint);
    VG_CUDA(cudaMemcpyAsync(b->heavy.p, h.data(), h.size() * 4, cudaMemcpyHostToDevice, b->stream));
  }
  VG_CUDA(cudaStreamSynchronize(b->stream));
}

// one cooperative launch of `steps` steps from buffer `cur` of `bufs`, the
// first with transition number step0, ilp agents per lane (1, 2 or 4)
template <int ILP>
void launch_persistent_ilp(vg_batch *b, const PersistArgs &p, int tpb) {
  int dev = 0, sms = 0, per_sm = 0;
  VG_CUDA(cudaGetDevice(&dev));
  VG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  VG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_persist<ILP>, tpb, 0));
  if (per_sm < 1) fail(VG_ERR_CUDA, "persistent batch kernel: no block fits an SM");
  // every block resident: a ticket may wait for blocks holding earlier tickets
  unsigned grid = (unsigned)(sms * per_sm);
  VG_CUDA(cudaMemsetAsync(b->bar.p, 0, 16, b->stream));
  VG_CUDA(cudaMemsetAsync(b->done.p, 0, (uint64_t)b->n * 4, b->stream));
  PersistArgs q = p;
  void *args[] = {&q};
  VG_CUDA(cudaLaunchCooperativeKernel((const void *)k_batch_persist<ILP>, dim3(grid), dim3(tpb),
                                      args, 0, b->stream));
}

void launch_persistent(vg_batch *b, const StateBufs &bufs, int cur, uint32_t step0,
                       uint32_t steps, int tpb, uint32_t thr, int ilp, int rounds) {
  build_buckets(b, thr);
  if (!b->bar.p) b->bar.alloc(16, &b->footprint);
  if (!b->done.p) {
    b->done.alloc((uint64_t)b->n * 4, &b->footprint);
    b->inst_n.alloc((uint64_t)b->n * 4, &b->footprint);
    std::vector<uint32_t> nn(b->N.begin(), b->N.end());
    VG_CUDA(cudaMemcpyAsync(b->inst_n.p, nn.data(), nn.size() * 4, cudaMemcpyHostToDevice,
                            b->stream));
    VG_CUDA(cudaStreamSynchronize(b->stream));
  }
  // the tickets of a launch (tickets per step x steps) and an instance's
  // agent-steps (steps x N) are counted in 32 bits: longer runs take
  // several launches, each starting from the state the last one left
  rounds = std::max(rounds, 1);
  const uint64_t span = (uint64_t)tpb * (uint64_t)ilp * (uint64_t)rounds;
  const uint64_t tps = (b->total + span - 1) / span;
  const uint64_t maxn = (uint64_t)*std::max_element(b->N.begin(), b->N.end());
  const uint64_t lim = 0xFFFFFFFFull;
  const uint64_t tlim = lim - (1ull << 20);  // room for every block's last (unused) ticket
  const uint32_t chunk =
      (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(lim / std::max<uint64_t>(maxn, 1),
                                                         tlim / std::max<uint64_t>(tps, 1)));
  for (uint32_t done = 0; done < steps;) {
    const uint32_t c = std::min(steps - done, chunk);
    PersistArgs p{};
    p.a = batch_args(b, cur, step0 + done, nullptr);
    for (int k = 0; k < 2; k++) {
      p.st[k] = bufs.st[k];
      p.dy[k] = bufs.dy[k];
      p.inf[k] = bufs.inf[k];
    }
    p.cur0 = cur;
    p.steps = c;
    p.step0 = step0 + done;
    p.heavy = b->heavy.as<uint32_t>();
    p.nheavy = b->nheavy;
    p.is_heavy = b->nheavy ? b->is_heavy.as<uint8_t>() : nullptr;
    p.ticket = b->bar.as<unsigned>();
    p.done = b->done.as<uint32_t>();
    p.inst_n = b->inst_n.as<uint32_t>();
    p.rounds = (unsigned)rounds;
    switch (ilp) {
      case 1: launch_persistent_ilp<1>(b, p, tpb); break;
      case 2: launch_persistent_ilp<2>(b, p, tpb); break;
      default: launch_persistent_ilp<4>(b, p, tpb); break;
    }
    if (c % 2) cur = 1 - cur;
    done += c;
  }
}

using ClusterKernel = void (*)(ClusterArgs);
ClusterKernel cluster_kernel(int ilp) { return ilp == 1 ? k_batch_cluster<1> : k_batch_cluster<2>; }

// clusters of `ctas` CTAs of `tpb` threads that can be resident at once with
// `smem` bytes of dynamic shared memory per CTA
unsigned resident_clusters(int ctas, int tpb, int ilp, size_t smem, cudaStream_t st) {
  const ClusterKernel k = cluster_kernel(ilp);
  if (cudaFuncSetAttribute((const void *)k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(tpb);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (const void *)k, &cfg) != cudaSuccess) {
    (void)cudaGetLastError();  // a shape the device cannot run: not available
    return 0;
  }
  return (unsigned)std::max(n, 0);
}

// Pack the instances for `clusters` clusters: instances by load (edges +
// agents) descending; one at least `target` = total / (4 clusters) forms a
// pack alone, the others fill packs in that order until a pack reaches the
// target.  Packs come out longest first; an instance's agents take whole
// 32-agent mask words at its pack's next free word.
void make_packs(vg_batch *b, unsigned clusters, std::vector<std::vector<int>> &packs,
                uint32_t &wmax) {
  const std::vector<uint32_t> &rp = b->host_rp;
  std::vector<int> order(b->n);
  std::vector<uint64_t> load(b->n);
  uint64_t total = 0;
  for (int i = 0; i < b->n; i++) {
    order[i] = i;
    const uint64_t a0 = b->host_base[i], Ni = (uint64_t)b->N[i];
    load[i] = (uint64_t)(rp[a0 + Ni] - rp[a0]) + Ni;
    total += load[i];
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return load[x] > load[y]; });
  const uint64_t target = std::max<uint64_t>(total / (4ull * std::max(clusters, 1u)), 1);
  packs.clear();
  uint64_t cur = 0, m = 0, words = 0;
  for (int i : order) {
    if (packs.empty() || cur >= target) {
      packs.push_back({});
      cur = 0;
      words = 0;
    }
    packs.back().push_back(i);
    cur += load[i];
    words += ((uint64_t)b->N[i] + 31) / 32;
    m = std::max(m, words);
  }
  wmax = (uint32_t)std::min<uint64_t>(m, 0xFFFFFFFFull);
}

// the packs for a cluster shape, and how many clusters to launch: as many
// as fit the GPU at once with the packs' mask size (at most one per pack)
ClusterPlan &cluster_plan(vg_batch *b, int ctas, int tpb, int ilp) {
  const int key = (ctas * 1024 + tpb) * 4 + ilp;
  auto it = b->cplans.find(key);
  if (it != b->cplans.end()) return it->second;
  ClusterPlan &P = b->cplans[key];
  int dev = 0, optin = 0;
  VG_CUDA(cudaGetDevice(&dev));
  VG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t fixed = 64;  // static shared memory besides the masks (the pack number)
  const unsigned R0 = resident_clusters(ctas, tpb, ilp, 0, b->stream);
  if (R0 == 0) return P;
  std::vector<std::vector<int>> packs;
  uint32_t wmax = 0;
  make_packs(b, R0, packs, wmax);
  P.smem = 2ull * 4 * std::max<uint32_t>(wmax, 1);
  if (P.smem + fixed > (size_t)optin) return P;  // a pack's masks do not fit a CTA
  const unsigned R = resident_clusters(ctas, tpb, ilp, P.smem, b->stream);
  if (R == 0) return P;
  std::vector<ChunkDesc> ch;
  std::vector<uint32_t> cofs(packs.size() + 1, 0);
  for (size_t k = 0; k < packs.size(); k++) {
    cofs[k] = (uint32_t)ch.size();
    uint64_t w0 = 0;
    for (int i : packs[k]) {
      const uint64_t a0 = b->host_base[i], Ni = (uint64_t)b->N[i];
      for (uint64_t c = 0; c * 32 < Ni; c++)
        ch.push_back({(uint32_t)(a0 + 32 * c), (uint32_t)(w0 + c),
                      (uint32_t)(32 * w0 - a0),  // modulo 2^64, then 2^32
                      (uint32_t)std::min<uint64_t>(32, Ni - 32 * c)});
      w0 += (Ni + 31) / 32;
    }
  }
  cofs[packs.size()] = (uint32_t)ch.size();
  P.chunks.alloc(std::max<size_t>(ch.size(), 1) * sizeof(ChunkDesc), &b->footprint);
  P.cofs.alloc(cofs.size() * 4, &b->footprint);
  P.ticket.alloc(4, &b->footprint);
  VG_CUDA(cudaMemcpyAsync(P.chunks.p, ch.data(), ch.size() * sizeof(ChunkDesc),
                          cudaMemcpyHostToDevice, b->stream));
  VG_CUDA(cudaMemcpyAsync(P.cofs.p, cofs.data(), cofs.size() * 4, cudaMemcpyHostToDevice,
                          b->stream));
  VG_CUDA(cudaStreamSynchronize(b->stream));
  P.npacks = (uint32_t)packs.size();
  P.wmax = wmax;
  P.G = std::min<unsigned>(R, P.npacks);
  return P;
}

// one launch of `steps` steps in the cluster form; false if the shape is
// not available for this arena
bool launch_cluster(vg_batch *b, const StateBufs &bufs, int cur, uint32_t step0, uint32_t steps,
                    int ctas, int tpb, int ilp) {
  ClusterPlan &P = cluster_plan(b, ctas, tpb, ilp);
  if (P.G == 0) return false;
  ClusterArgs ca{};
  ca.a = batch_args(b, cur, step0, nullptr);
  for (int k = 0; k < 2; k++) {
    ca.st[k] = bufs.st[k];
    ca.dy[k] = bufs.dy[k];
  }
  ca.chunks = P.chunks.as<ChunkDesc>();
  ca.cofs = P.cofs.as<uint32_t>();
  ca.npacks = P.npacks;
  ca.ticket = P.ticket.as<unsigned>();
  ca.wmax = P.wmax;
  ca.cur0 = cur;
  ca.steps = steps;
  ca.step0 = step0;
  const ClusterKernel k = cluster_kernel(ilp);
  VG_CUDA(cudaFuncSetAttribute((const void *)k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)P.smem));
  VG_CUDA(cudaMemsetAsync(P.ticket.p, 0, 4, b->stream));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(P.G * ctas);
  cfg.blockDim = dim3(tpb);
  cfg.dynamicSmemBytes = P.smem;
  cfg.stream = b->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  void *args[] = {&ca};
  VG_CUDA(cudaLaunchKernelExC(&cfg, (const void *)k, args));
  return true;
}

// one per-step launch: warps of 32 ilp agents
void launch_step(vg_batch *, const BatchArgs &a, int tpb, int ilp, cudaStream_t st) {
  const uint64_t warps = (a.n + 32ull * ilp - 1) / (32ull * ilp);
  unsigned g = blocks(warps * 32, tpb);
  switch (ilp) {
    case 1: k_batch_sir<1><<<g, tpb, 0, st>>>(a); break;
    case 2: k_batch_sir<2><<<g, tpb, 0, st>>>(a); break;
    default: k_batch_sir<4><<<g, tpb, 0, st>>>(a); break;
  }
}

// Choose the launch form by timing candidates on copies of the current
// state (the simulation state is not touched): per-step launches (block
// size 128/256/512 x agents per lane 1/2/4, replayed from a CUDA graph when
// stepping) and the persistent launch (block size 256/512 x agents per lane
// 1/2/4 x bucket threshold: none, or a warp for each agent above 64
// in-edges).  Keyed on the arena's agents, edges and in-degree histogram
// (log2 buckets).
void autotune(vg_batch *b) {
  if (b->host_rp.empty()) {
    b->host_rp.resize(b->total + 1);
    VG_CUDA(cudaMemcpyAsync(b->host_rp.data(), b->rp.p, b->host_rp.size() * 4,
                            cudaMemcpyDeviceToHost, b->stream));
    VG_CUDA(cudaStreamSynchronize(b->stream));
  }
  const std::vector<uint32_t> &rp = b->host_rp;
  uint64_t hist[16] = {0};
  for (uint64_t i = 0; i < b->total; i++) {
    uint32_t d = rp[i + 1] - rp[i];
    int bkt = 0;
    while (bkt < 15 && (1u << bkt) <= d) bkt++;
    hist[bkt]++;
  }
  uint64_t key = b->total * 1000003ull + b->total_edges;
  for (int i = 0; i < 16; i++) key = key * 31 + (hist[i] * 16 / std::max<uint64_t>(b->total, 1));
  auto it = b->tune_cache.find(key);
  if (it != b->tune_cache.end()) {
    b->tpb = it->second.tpb;
    b->apt = it->second.apt;
    b->p_tpb = it->second.p_tpb;
    b->p_ilp = it->second.p_ilp;
    b->p_rounds = it->second.p_rounds;
    b->p_thr = it->second.p_thr;
    b->c_ctas = it->second.c_ctas;
    b->c_tpb = it->second.c_tpb;
    b->c_ilp = it->second.c_ilp;
    b->form = it->second.form;
    b->tuned_graph_ms = it->second.graph_ms;
    b->tuned_persistent_ms = it->second.persistent_ms;
    b->tuned_cluster_ms = it->second.cluster_ms;
    b->tuned = true;
    return;
  }
  // trial buffers: copies of the current state
  const uint64_t words = mask_words(b->total);
  for (int k = 0; k < 2; k++) {
    if (!b->scratch_st[k].p) b->scratch_st[k].alloc(b->total, &b->footprint);
    if (!b->scratch_dy[k].p) b->scratch_dy[k].alloc(b->total * 4, &b->footprint);
    if (!b->scratch_inf[k].p) b->scratch_inf[k].alloc(words * 4, &b->footprint);
  }
  const StateBufs sb = {{b->scratch_st[0].as<uint8_t>(), b->scratch_st[1].as<uint8_t>()},
                        {b->scratch_dy[0].as<int32_t>(), b->scratch_dy[1].as<int32_t>()},
                        {b->scratch_inf[0].as<uint32_t>(), b->scratch_inf[1].as<uint32_t>()}};
  auto reset = [&]() {
    VG_CUDA(cudaMemcpyAsync(sb.st[0], b->st[b->cur].p, b->total, cudaMemcpyDeviceToDevice,
                            b->stream));
    VG_CUDA(cudaMemcpyAsync(sb.dy[0], b->dy[b->cur].p, b->total * 4, cudaMemcpyDeviceToDevice,
                            b->stream));
    VG_CUDA(cudaMemcpyAsync(sb.inf[0], b->inf[b->cur].p, words * 4, cudaMemcpyDeviceToDevice,
                            b->stream));
  };
  constexpr uint32_t TRIAL = 24;
  cudaEvent_t e0, e1;
  VG_CUDA(cudaEventCreate(&e0));
  VG_CUDA(cudaEventCreate(&e1));
  auto timed = [&](auto &&run) {
    reset();
    run();  // warm
    reset();
    VG_CUDA(cudaEventRecord(e0, b->stream));
    run();
    VG_CUDA(cudaEventRecord(e1, b->stream));
    VG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    VG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    return ms;
  };
  float best = 1e30f;
  int bt = 256, ba = 1;
  for (int tpb : {128, 256, 512})
    for (int ilp : {1, 2, 4}) {
      const float ms = timed([&] {
        for (uint32_t t = 0; t < TRIAL; t++) {
          BatchArgs a = batch_args(b, 0, (uint32_t)b->step + t, nullptr);
          const int c = (int)(t & 1);
          a.st_rd = sb.st[c];
          a.d_rd = sb.dy[c];
          a.inf_rd = sb.inf[c];
          a.st_wr = sb.st[1 - c];
          a.d_wr = sb.dy[1 - c];
          a.inf_wr = sb.inf[1 - c];
          launch_step(b, a, tpb, ilp, b->stream);
        }
      });
      if (ms < best) {
        best = ms;
        bt = tpb;
        ba = ilp;
      }
    }
  float pbest = 1e30f;
  int pt = 256, pi = 2, pr = 4;
  uint32_t pthr = 0xFFFFFFFFu;
  for (int tpb : {256, 512})
    for (int ilp : {1, 2, 4})
      for (int rounds : {2, 4, 8}) {
        const float ms = timed([&] {
          launch_persistent(b, sb, 0, (uint32_t)b->step, TRIAL, tpb, 0xFFFFFFFFu, ilp, rounds);
        });
        if (ms < pbest) {
          pbest = ms;
          pt = tpb;
          pi = ilp;
          pr = rounds;
        }
      }
  {  // the degree bucket on the best shape
    const float ms = timed([&] {
      launch_persistent(b, sb, 0, (uint32_t)b->step, TRIAL, pt, 64u, pi, pr);
    });
    if (ms < pbest) {
      pbest = ms;
      pthr = 64u;
    }
  }
  float cbest = 1e30f;
  int cc = 8, ct = 512, ci = 1;
  for (int ctas : {4, 8})
    for (int tpb : {256, 512})
      for (int ilp : {1, 2}) {
        if (cluster_plan(b, ctas, tpb, ilp).G == 0) continue;  // shape not available
        const float ms = timed([&] {
          launch_cluster(b, sb, 0, (uint32_t)b->step, TRIAL, ctas, tpb, ilp);
        });
        if (ms < cbest) {
          cbest = ms;
          cc = ctas;
          ct = tpb;
          ci = ilp;
        }
      }
  VG_CUDA(cudaEventDestroy(e0));
  VG_CUDA(cudaEventDestroy(e1));
  check_batch_status(b);
  b->tpb = bt;
  b->apt = ba;
  b->p_tpb = pt;
  b->p_ilp = pi;
  b->p_rounds = pr;
  b->p_thr = pthr;
  b->c_ctas = cc;
  b->c_tpb = ct;
  b->c_ilp = ci;
  // keep only the chosen shape's packing (another is rebuilt on request)
  const int keep = (cc * 1024 + ct) * 4 + ci;
  for (auto it2 = b->cplans.begin(); it2 != b->cplans.end();)
    it2 = it2->first == keep ? std::next(it2) : b->cplans.erase(it2);
  b->form = cbest < std::min(best, pbest) ? 4 : (pbest < best ? 2 : 1);
  b->tuned_graph_ms = best / TRIAL;
  b->tuned_persistent_ms = pbest / TRIAL;
  b->tuned_cluster_ms = cbest < 1e29f ? cbest / TRIAL : 0.0f;
  b->tuned = true;
  b->tune_cache[key] = {bt,       ba,      pt,      pi,      pr,
                        pthr,     cc,      ct,      ci,
                        b->form,  b->tuned_graph_ms, b->tuned_persistent_ms,
                        b->tuned_cluster_ms};
}


}  // namespace

#define API_BEGIN try {
#define API_END                     \
  return VG_OK;                     \
  }                                 \
  catch (const Error &e) {          \
    set_last_error(e.msg);          \
    return e.code;                  \
  }                                 \
  catch (const std::exception &e) { \
    set_last_error(e.what());       \
    return VG_ERR_ARG;              \
  }

extern "C" {

int vg_batch_create_sir(int n, const int64_t *N, const int32_t *deg, const double *beta,
                        const int32_t *rec, const uint64_t *seeds,
                        int64_t n_init_infected_per_1000, void *stream, vg_batch **out) {
  API_BEGIN
  if (n <= 0 || n > 65535) fail(VG_ERR_ARG, "batch: 1..65535 instances");
  need(N, "instance sizes");
  need(deg, "instance degrees");
  need(beta, "instance infection rates");
  need(rec, "instance recovery days");
  need(seeds, "instance seeds");
  need(out, "output pointer");
  auto b = std::make_unique<vg_batch>();
  b->n = n;
  b->N.assign(N, N + n);
  b->deg.assign(deg, deg + n);
  b->beta.assign(beta, beta + n);
  b->rec.assign(rec, rec + n);
  b->seed.assign(seeds, seeds + n);
  if (stream) {
    b->stream = (cudaStream_t)stream;
  } else {
    VG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->own_stream = true;
  }
  // the "SIR" model
  int rc = vg_model_create(&b->model);
  if (rc) fail(rc, vg_last_error());
  const char *pf[2] = {"state", "days"};
  int pd[2] = {VG_U8, VG_I32};
  if ((rc = vg_model_register_agenttype(b->model, "Person", 2, pf, pd, VG_HINT_IMMORTAL,
                                         &b->person)))
    fail(rc, vg_last_error());
  if ((rc = vg_model_register_edgetype(b->model, "Contact", 0, nullptr, nullptr,
                                        VG_HINT_STATELESS, b->person, 0, &b->contact)))
    fail(rc, vg_last_error());
  if ((rc = vg_model_finalize(b->model, "SIR"))) fail(rc, vg_last_error());
  // instances as plain simulations
  uint32_t kmax = 0;
  std::vector<uint64_t> bases(n);
  for (int i = 0; i < n; i++) {
    vg_sim *s = nullptr;
    if ((rc = vg_sim_create(b->model, "instance", b->stream, &s))) fail(rc, vg_last_error());
    b->sims.push_back(s);
    uint64_t Ni = (uint64_t)N[i];
    if (Ni < 2) fail(VG_ERR_ARG, "batch: instances need at least two agents");
    std::vector<uint8_t> state;
    uint64_t ninf = (uint64_t)std::max<double>(
        1.0, std::nearbyint((double)Ni * (double)n_init_infected_per_1000 / 1000.0));
    sir_initial_state(Ni, seeds[i], ninf, state);
    std::vector<int32_t> days(Ni, 0);
    const void *cols[2] = {state.data(), days.data()};
    if ((rc = vg_add_agents(s, b->person, Ni, cols, nullptr))) fail(rc, vg_last_error());
    if ((rc = vg_gen_uniform_out_edges(s, b->contact, b->person, (uint32_t)deg[i], seeds[i])))
      fail(rc, vg_last_error());
    if ((rc = vg_finish_init(s))) fail(rc, vg_last_error());
    bases[i] = b->total;
    b->total += Ni;
    Sim &S = *s->s;
    CSR &c = S.edges[b->contact].csr[b->person];
    b->total_edges += c.nedges;
    kmax = std::max(kmax, csr_max_degree(S, c));
  }
  if (b->total_edges >= (1ull << 32) || b->total >= (1ull << 32))
    fail(VG_ERR_NOMEM, "batch: arena indices are 32-bit");
  // arena
  cudaStream_t st = b->stream;
  uint64_t *fp = &b->footprint;
  b->rp.alloc((b->total + 1) * 4, fp);
  b->src.alloc(std::max<uint64_t>(b->total_edges, 1) * 4, fp);
  b->inst.alloc(b->total * 2, fp);
  for (int k = 0; k < 2; k++) {
    b->st[k].alloc(b->total, fp);
    b->dy[k].alloc(b->total * 4, fp);
    b->inf[k].alloc(mask_words(b->total) * 4, fp);
    VG_CUDA(cudaMemsetAsync(b->inf[k].p, 0, mask_words(b->total) * 4, st));
  }
  uint64_t ebase = 0;
  for (int i = 0; i < n; i++) {
    Sim &S = *b->sims[i]->s;
    CSR &c = S.edges[b->contact].csr[b->person];
    AgentStore &A = S.agents[b->person - 1];
    uint64_t Ni = A.n, a0 = bases[i];
    k_offset_rp<<<blocks(Ni + 1, 256), 256, 0, st>>>(c.row_ptr.as<uint32_t>(), Ni, (uint32_t)ebase,
                                                    b->rp.as<uint32_t>() + a0);
    if (c.nedges)
      k_offset_src<<<blocks(c.nedges, 256), 256, 0, st>>>(c.src.as<uint32_t>(), c.nedges,
                                                         (uint32_t)a0,
                                                         b->src.as<uint32_t>() + ebase);
    k_fill_u16<<<blocks(Ni, 256), 256, 0, st>>>(b->inst.as<uint16_t>() + a0, Ni, (uint16_t)i);
    VG_CUDA(cudaMemcpyAsync(b->st[0].as<uint8_t>() + a0, A.rd[0].p, Ni, cudaMemcpyDeviceToDevice, st));
    VG_CUDA(cudaMemcpyAsync(b->dy[0].as<int32_t>() + a0, A.rd[1].p, Ni * 4, cudaMemcpyDeviceToDevice, st));
    ebase += c.nedges;
    VG_CUDA(cudaGetLastError());
  }
  // the infected-agent mask of the initial state
  k_inf_bits<<<blocks(b->total, 256), 256, 0, st>>>(b->st[0].as<uint8_t>(), b->total,
                                                    b->inf[0].as<uint32_t>());
  VG_CUDA(cudaGetLastError());
  // per-instance tables: p_k = 1 - (1 - beta)^k by repeated multiplication
  b->kmax1 = kmax + 1;
  std::vector<double> tab((uint64_t)n * b->kmax1);
  for (int i = 0; i < n; i++) {
    double q = 1.0, om = 1.0 - beta[i];
    tab[(uint64_t)i * b->kmax1] = 0.0;
    for (uint32_t k = 1; k <= kmax; k++) {
      q = q * om;
      tab[(uint64_t)i * b->kmax1 + k] = 1.0 - q;
    }
  }
  b->host_base = bases;
  b->ptab.alloc(tab.size() * 8, fp);
  b->base.alloc(n * 8, fp);
  b->rec_d.alloc(n * 4, fp);
  b->seed_d.alloc(n * 8, fp);
  b->status.alloc(16, fp);
  VG_CUDA(cudaMemcpyAsync(b->ptab.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, st));
  VG_CUDA(cudaMemcpyAsync(b->base.p, bases.data(), n * 8, cudaMemcpyHostToDevice, st));
  VG_CUDA(cudaMemcpyAsync(b->rec_d.p, rec, n * 4, cudaMemcpyHostToDevice, st));
  VG_CUDA(cudaMemcpyAsync(b->seed_d.p, seeds, n * 8, cudaMemcpyHostToDevice, st));
  VG_CUDA(cudaMemsetAsync(b->status.p, 0, 16, st));
  VG_CUDA(cudaStreamSynchronize(st));
  *out = b.release();
  API_END
}

// mode 0: one launch per step; mode 1: the `steps` launches captured once in
// a CUDA graph (re-captured when the step count or phase changes) and
// replayed; mode 2: one persistent launch for all steps; mode 3: the faster
// of 1 and 2 as the autotuner measured them.
int vg_batch_step(vg_batch *b, int steps, int mode) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  if (mode < 0 || mode > 4) fail(VG_ERR_ARG, "batch: mode 0..4");
  if (steps <= 0) return VG_OK;
  if (!b->tuned) autotune(b);
  if (mode == 3) mode = b->form;
  if (mode == 4) {
    if (!launch_cluster(b, arena_bufs(b), b->cur, (uint32_t)b->step, (uint32_t)steps, b->c_ctas,
                        b->c_tpb, b->c_ilp))
      fail(VG_ERR_ARG, "batch: the cluster form does not fit this arena (a pack's mask "
                       "exceeds a CTA's shared memory)");
    if (steps % 2) b->cur = 1 - b->cur;
    b->step += steps;
    // the clusters keep their masks in shared memory: the arena's mask of the
    // final state, which the other forms read, is made from the states
    k_inf_bits<<<blocks(b->total, 256), 256, 0, b->stream>>>(b->st[b->cur].as<uint8_t>(), b->total,
                                                           b->inf[b->cur].as<uint32_t>());
    VG_CUDA(cudaGetLastError());
  } else if (mode == 2) {
    launch_persistent(b, arena_bufs(b), b->cur, (uint32_t)b->step, (uint32_t)steps, b->p_tpb,
                      b->p_thr, b->p_ilp, b->p_rounds);
    if (steps % 2) b->cur = 1 - b->cur;
    b->step += steps;
  } else if (mode == 0) {
    for (int k = 0; k < steps; k++) {
      BatchArgs a = batch_args(b, b->cur, (uint32_t)b->step, nullptr);
      launch_step(b, a, b->tpb, b->apt, b->stream);
      VG_CUDA(cudaGetLastError());
      b->cur = 1 - b->cur;
      b->step++;
    }
  } else {
    if (b->graph_steps != steps) {  // (re)capture for this step count
      for (int p = 0; p < 2; p++)
        if (b->graph[p]) {
          cudaGraphExecDestroy(b->graph[p]);
          cudaGraphDestroy(b->graph_def[p]);
          b->graph[p] = nullptr;
        }
      b->graph_steps = steps;
    }
    if (!b->step_base.p) b->step_base.alloc(8, &b->footprint);
    int p = b->cur;
    if (!b->graph[p]) {
      cudaStream_t cs;
      VG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        try {
          int cur = p;
          for (int k = 0; k < steps; k++) {
            BatchArgs a = batch_args(b, cur, (uint32_t)k, b->step_base.as<int64_t>());
            launch_step(b, a, b->tpb, b->apt, cs);
            cur = 1 - cur;
          }
        } catch (...) {  // end the capture and free the stream before passing the error on
          cudaStreamEndCapture(cs, &g);
          if (g) cudaGraphDestroy(g);
          cudaStreamDestroy(cs);
          throw;
        }
        e = cudaStreamEndCapture(cs, &g);
      }
      cudaStreamDestroy(cs);
      if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph[p], g, 0);
      if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        b->graph[p] = nullptr;
        VG_CUDA(e);
      }
      b->graph_def[p] = g;
    }
    int64_t s0 = b->step;
    VG_CUDA(cudaMemcpyAsync(b->step_base.p, &s0, 8, cudaMemcpyHostToDevice, b->stream));
    VG_CUDA(cudaGraphLaunch(b->graph[p], b->stream));
    if (steps % 2) b->cur = 1 - b->cur;
    b->step += steps;
  }
  check_batch_status(b);
  API_END
}

int vg_batch_step_one(vg_batch *b, int i, int steps) {
  API_BEGIN
  if (!b || i < 0 || i >= b->n) fail(VG_ERR_ARG, "batch: instance index");
  int call = b->person, read[2] = {b->person, VG_EDGE(b->contact)}, write = b->person;
  double params[4] = {(double)b->contact, b->beta[i], (double)b->rec[i], (double)b->seed[i]};
  if (b->seed[i] >= (1ull << 53)) fail(VG_ERR_ARG, "batch: seeds below 2^53");
  int rc = vg_sim_set_async(b->sims[i], 1);  // launches back to back, one check at the end
  if (rc) fail(rc, vg_last_error());
  for (int k = 0; k < steps; k++) {
    rc = vg_apply(b->sims[i], "sir", &call, 1, read, 2, &write, 1, nullptr, 0, -1, params, 4);
    if (rc) fail(rc, vg_last_error());
  }
  if ((rc = vg_sim_synchronize(b->sims[i]))) fail(rc, vg_last_error());
  API_END
}

// which = 0: the batched arena; which = 1: the instance's own simulation
int vg_batch_read_states2(vg_batch *b, int i, int which, uint8_t *state_out,
                          int32_t *days_out, uint64_t cap, uint64_t *n_out) {
  API_BEGIN
  if (!b || i < 0 || i >= b->n) fail(VG_ERR_ARG, "batch: instance index");
  if (which == 1) {
    void *cols[2] = {state_out, days_out};
    int rc = vg_read_agents(b->sims[i], b->person, cols, nullptr, cap, n_out);
    if (rc) fail(rc, vg_last_error());
    return VG_OK;
  }
  if (which != 0) fail(VG_ERR_ARG, "batch: which 0 (the arena) or 1 (the instance's simulation)");
  need(n_out, "count pointer");
  uint64_t a0 = 0;
  for (int j = 0; j < i; j++) a0 += (uint64_t)b->N[j];
  uint64_t Ni = (uint64_t)b->N[i];
  *n_out = Ni;
  uint64_t m = std::min(cap, Ni);
  VG_CUDA(cudaStreamSynchronize(b->stream));
  if (state_out) VG_CUDA(cudaMemcpy(state_out, b->st[b->cur].as<uint8_t>() + a0, m, cudaMemcpyDeviceToHost));
  if (days_out) VG_CUDA(cudaMemcpy(days_out, b->dy[b->cur].as<int32_t>() + a0, m * 4, cudaMemcpyDeviceToHost));
  API_END
}

int vg_batch_read_states(vg_batch *b, int i, uint8_t *state_out, int32_t *days_out,
                         uint64_t cap, uint64_t *n_out) {
  return vg_batch_read_states2(b, i, 0, state_out, days_out, cap, n_out);
}

int vg_batch_read_graph(vg_batch *b, int i, uint32_t *row_ptr_out, uint32_t *src_out,
                        uint64_t *nrows_out, uint64_t *nedges_out) {
  API_BEGIN
  if (!b || i < 0 || i >= b->n) fail(VG_ERR_ARG, "batch: instance index");
  need(nrows_out, "row count pointer");
  need(nedges_out, "edge count pointer");
  Sim &S = *b->sims[i]->s;
  CSR &c = S.edges[b->contact].csr[b->person];
  *nrows_out = c.nrows;
  *nedges_out = c.nedges;
  if (row_ptr_out) VG_CUDA(cudaMemcpy(row_ptr_out, c.row_ptr.p, (c.nrows + 1) * 4, cudaMemcpyDeviceToHost));
  if (src_out && c.nedges) VG_CUDA(cudaMemcpy(src_out, c.src.p, c.nedges * 4, cudaMemcpyDeviceToHost));
  API_END
}

int vg_selftest_barrier_timeout(int *status_out, double *ms_out) {
  API_BEGIN
  need(status_out, "status pointer");
  need(ms_out, "duration pointer");
  unsigned *bar = nullptr;
  int *status = nullptr;
  VG_CUDA(cudaMalloc(&bar, 8));
  VG_CUDA(cudaMalloc(&status, 4));
  VG_CUDA(cudaMemset(bar, 0, 8));
  VG_CUDA(cudaMemset(status, 0, 4));
  cudaEvent_t e0, e1;
  VG_CUDA(cudaEventCreate(&e0));
  VG_CUDA(cudaEventCreate(&e1));
  VG_CUDA(cudaEventRecord(e0));
  // two blocks wait for an instance counter (zero) to reach 1
  k_barrier_probe<<<2, 64>>>((const uint32_t *)bar, 1u, status, 1u << 16);
  VG_CUDA(cudaEventRecord(e1));
  VG_CUDA(cudaEventSynchronize(e1));
  VG_CUDA(cudaGetLastError());
  float ms = 0;
  VG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  VG_CUDA(cudaMemcpy(status_out, status, 4, cudaMemcpyDeviceToHost));
  *ms_out = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(bar);
  cudaFree(status);
  API_END
}

int vg_batch_set_launch(vg_batch *b, int persistent, int persistent_tpb,
                        uint32_t bucket_threshold) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  if (persistent < 0 || persistent > 2) fail(VG_ERR_ARG, "batch: form 0, 1 or 2");
  if (persistent_tpb != 128 && persistent_tpb != 256 && persistent_tpb != 512)
    fail(VG_ERR_ARG, "batch: persistent block size 128, 256 or 512");
  if (!b->tuned) autotune(b);
  if (persistent == 2 && cluster_plan(b, b->c_ctas, b->c_tpb, b->c_ilp).G == 0)
    fail(VG_ERR_ARG, "batch: the cluster form does not fit this arena");
  b->form = persistent == 2 ? 4 : (persistent == 1 ? 2 : 1);
  b->p_tpb = persistent_tpb;
  b->p_thr = bucket_threshold;
  API_END
}

int vg_batch_set_cluster(vg_batch *b, int ctas, int tpb, int ilp) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  if (ctas != 1 && ctas != 2 && ctas != 4 && ctas != 8)
    fail(VG_ERR_ARG, "batch: 1, 2, 4 or 8 CTAs per cluster");
  if (tpb != 128 && tpb != 256 && tpb != 512)
    fail(VG_ERR_ARG, "batch: cluster block size 128, 256 or 512");
  if (ilp != 1 && ilp != 2) fail(VG_ERR_ARG, "batch: cluster agents per lane 1 or 2");
  if (!b->tuned) autotune(b);
  if (cluster_plan(b, ctas, tpb, ilp).G == 0)
    fail(VG_ERR_ARG, "batch: this cluster shape does not fit the arena");
  b->c_ctas = ctas;
  b->c_tpb = tpb;
  b->c_ilp = ilp;
  API_END
}

int vg_batch_cluster(vg_batch *b, int *ctas, int *tpb, int *ilp, unsigned *clusters) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  if (!b->tuned) autotune(b);
  if (ctas) *ctas = b->c_ctas;
  if (tpb) *tpb = b->c_tpb;
  if (ilp) *ilp = b->c_ilp;
  if (clusters) *clusters = cluster_plan(b, b->c_ctas, b->c_tpb, b->c_ilp).G;
  API_END
}

int vg_batch_set_lanes(vg_batch *b, int per_step, int persistent) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  auto ok = [](int v) { return v == 0 || v == 1 || v == 2 || v == 4; };
  if (!ok(per_step) || !ok(persistent)) fail(VG_ERR_ARG, "batch: agents per lane 1, 2 or 4");
  if (!b->tuned) autotune(b);
  if (per_step) {
    if (per_step != b->apt) {  // the recorded graphs hold the old launch shape
      for (int p = 0; p < 2; p++)
        if (b->graph[p]) {
          cudaGraphExecDestroy(b->graph[p]);
          cudaGraphDestroy(b->graph_def[p]);
          b->graph[p] = nullptr;
        }
    }
    b->apt = per_step;
  }
  if (persistent) b->p_ilp = persistent;
  API_END
}

int vg_batch_lanes(vg_batch *b, int *per_step, int *persistent) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  if (!b->tuned) autotune(b);
  if (per_step) *per_step = b->apt;
  if (persistent) *persistent = b->p_ilp;
  API_END
}

int vg_batch_tuning(vg_batch *b, int *persistent, int *persistent_tpb,
                    uint32_t *bucket_threshold, uint64_t *heavy_agents,
                    double *step_ms_graph, double *step_ms_persistent,
                    double *step_ms_cluster) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  if (!b->tuned) autotune(b);
  if (step_ms_graph) *step_ms_graph = b->tuned_graph_ms;
  if (step_ms_persistent) *step_ms_persistent = b->tuned_persistent_ms;
  if (step_ms_cluster) *step_ms_cluster = b->tuned_cluster_ms;
  if (persistent) *persistent = b->form == 4 ? 2 : (b->form == 2 ? 1 : 0);
  if (persistent_tpb) *persistent_tpb = b->p_tpb;
  if (bucket_threshold) *bucket_threshold = b->p_thr;
  if (heavy_agents) {
    build_buckets(b, b->p_thr);
    *heavy_agents = b->nheavy;
  }
  API_END
}

int vg_batch_info(vg_batch *b, uint64_t *agents, uint64_t *edges, int *tpb, int *apt,
                  uint64_t *device_bytes) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  if (agents) *agents = b->total;
  if (edges) *edges = b->total_edges;
  if (tpb) *tpb = b->tpb;
  if (apt) *apt = b->apt;
  if (device_bytes) {
    uint64_t t = b->footprint;
    for (auto *s : b->sims) t += s->s->footprint;
    *device_bytes = t;
  }
  API_END
}

int vg_batch_destroy(vg_batch *b) {
  API_BEGIN
  if (!b) return VG_OK;
  cudaStreamSynchronize(b->stream);
  for (int p = 0; p < 2; p++)
    if (b->graph[p]) {
      cudaGraphExecDestroy(b->graph[p]);
      cudaGraphDestroy(b->graph_def[p]);
    }
  for (auto *s : b->sims) vg_sim_destroy(s);
  if (b->model) vg_model_destroy(b->model);
  cudaStream_t st = b->stream;
  bool own = b->own_stream;
  delete b;
  if (own) cudaStreamDestroy(st);
  API_END
}

}  // extern "C"
