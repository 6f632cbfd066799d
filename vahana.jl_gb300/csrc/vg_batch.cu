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
// replayed.  Launch shape (block size, agents per thread) comes from a
// small autotuner keyed on the arena's degree histogram; the persistent
// form runs every step in one cooperative launch with a grid-wide barrier
// between steps, and the autotuner picks it when it measures faster.
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
  uint8_t *__restrict__ st_wr;
  int32_t *__restrict__ d_wr;
  uint64_t n;
  uint32_t kmax1;  // table row length
  uint32_t step;   // transition number, plus *step_base when step_base is set
  const int64_t *step_base;
  int *status;
};

// the SIR rule of transition "sir" (csrc/vg_transitions.cu), per instance
template <int APT>
__global__ void k_batch_sir(BatchArgs a) {
  if (a.step_base) a.step += (uint32_t)*a.step_base;
  uint64_t first = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * APT;
#pragma unroll
  for (int r = 0; r < APT; r++) {
    uint64_t i = first + r;
    if (i >= a.n) return;
    uint32_t in = a.inst[i];
    uint8_t s = a.st_rd[i];
    int32_t d = a.d_rd[i];
    if (s == 0) {
      uint32_t k = 0;
      uint32_t e = a.rp[i + 1];
      for (uint32_t q = a.rp[i]; q < e; q++) k += (__ldg(a.st_rd + a.src[q]) == 1);
      if (k > 0) {
        if (k >= a.kmax1) {
          atomicCAS(a.status, 0, 402);
        } else {
          uint64_t nr = i - a.base[in] + 1;
          double u = u64_to_unit(philox_u64(philox_draw(a.seed[in], nr, a.step, TAG_INFECT)));
          if (u < a.ptab[(uint64_t)in * a.kmax1 + k]) {
            s = 1;
            d = 0;
          }
        }
      }
    } else if (s == 1) {
      d = d + 1;
      if (d >= a.rec[in]) s = 2;
    }
    a.st_wr[i] = s;
    a.d_wr[i] = d;
  }
}

// ---- persistent form: one cooperative launch runs every step.  Blocks
// meet at a grid-wide barrier between steps (all blocks are resident: the
// launch is cooperative).  The states a step reads were written by other
// blocks in the previous step of the same launch: they are read with
// ordinary loads after the barrier's GPU-scope acquire fence (never through
// the read-only path, which assumes data constant for the whole launch).  Agents whose
// in-degree exceeds the bucket threshold (listed in `heavy`) are folded by a
// warp each (the infected-neighbour count is an integer: any order gives the
// same k); the others by a thread each.
struct PersistArgs {
  BatchArgs a;                 // graph, tables; state pointers unused
  uint8_t *st[2];
  int32_t *dy[2];
  int cur0;                    // buffer of the state before the first step
  uint32_t steps, step0;       // steps to run, transition number of the first
  const uint32_t *heavy;       // agents above the bucket threshold (nheavy)
  uint64_t nheavy;
  const uint8_t *is_heavy;     // per agent (null: no heavy agents)
  unsigned *bar;               // [0] arrivals, [1] generation
};

constexpr uint32_t BAR_SPIN_LIMIT = 1u << 22;
constexpr int BAR_ERR_WAIT = 0x5e04;

// Sense-free grid barrier on a generation counter; a wait that runs out
// records BAR_ERR_WAIT and returns false (the launch then ends).
__device__ bool grid_barrier(unsigned *bar, unsigned nblocks, int *status,
                             uint32_t limit = BAR_SPIN_LIMIT) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      uint32_t i = 0;
      while (*gen == g) {
        if (++i >= limit) {
          atomicCAS(status, 0, BAR_ERR_WAIT);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    // acquire at GPU scope: the other blocks' writes of the step are visible
    // to this block's ordinary (L1-cached) loads after the barrier
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
  }
  __syncthreads();
  return ok != 0;
}

// failure detection without a fault: blocks meet at a barrier that expects
// one block more than the launch has, so every wait runs out
__global__ void k_barrier_probe(unsigned *bar, unsigned expect, int *status, uint32_t limit) {
  grid_barrier(bar, expect, status, limit);
}

// the rule of transition "sir" for agent i with k infected in-neighbours
__device__ __forceinline__ void sir_rule(const BatchArgs &a, uint64_t i, uint32_t k, uint8_t s,
                                         int32_t d, uint32_t step, uint8_t *st_wr,
                                         int32_t *d_wr) {
  const uint32_t in = a.inst[i];
  if (s == 0) {
    if (k > 0) {
      if (k >= a.kmax1) {
        atomicCAS(a.status, 0, 402);
      } else {
        const uint64_t nr = i - a.base[in] + 1;
        const double u = u64_to_unit(philox_u64(philox_draw(a.seed[in], nr, step, TAG_INFECT)));
        if (u < a.ptab[(uint64_t)in * a.kmax1 + k]) {
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
}

__global__ void k_batch_persist(PersistArgs p) {
  const BatchArgs &a = p.a;
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nwarps = nthreads / 32, wid = tid / 32;
  const unsigned lane = threadIdx.x & 31;
  for (uint32_t t = 0; t < p.steps; t++) {
    const int cur = p.cur0 ^ (int)(t & 1);
    const uint8_t *st_rd = p.st[cur];
    const int32_t *d_rd = p.dy[cur];
    uint8_t *st_wr = p.st[1 - cur];
    int32_t *d_wr = p.dy[1 - cur];
    const uint32_t step = p.step0 + t;
    for (uint64_t i = tid; i < a.n; i += nthreads) {  // thread per agent
      if (p.is_heavy && p.is_heavy[i]) continue;
      const uint8_t s = st_rd[i];
      const int32_t d = d_rd[i];
      uint32_t k = 0;
      if (s == 0) {
        const uint32_t e = a.rp[i + 1];
        for (uint32_t q = a.rp[i]; q < e; q++) k += (st_rd[a.src[q]] == 1);
      }
      sir_rule(a, i, k, s, d, step, st_wr, d_wr);
    }
    for (uint64_t h = wid; h < p.nheavy; h += nwarps) {  // warp per heavy agent
      const uint64_t i = p.heavy[h];
      const uint8_t s = st_rd[i];
      const int32_t d = d_rd[i];
      uint32_t k = 0;
      if (s == 0) {
        const uint32_t e = a.rp[i + 1];
        for (uint32_t q = a.rp[i] + lane; q < e; q += 32) k += (st_rd[a.src[q]] == 1);
      }
      k = __reduce_add_sync(0xffffffffu, k);
      if (lane == 0) sir_rule(a, i, k, s, d, step, st_wr, d_wr);
    }
    if (t + 1 < p.steps && !grid_barrier(p.bar, gridDim.x, a.status)) return;
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
  DevBuf rp, src, inst, base, ptab, rec_d, seed_d, st[2], dy[2], status;
  uint32_t kmax1 = 0;
  int cur = 0;
  int64_t step = 1;  // transition number of the next step (as after finish_init!)
  int tpb = 256, apt = 1;
  bool tuned = false;
  struct Tuned {
    int tpb, apt, p_tpb;
    uint32_t p_thr;
    bool persistent;
    float graph_ms, persistent_ms;
  };
  std::map<uint64_t, Tuned> tune_cache;
  // persistent form: block size, bucket threshold (agents with more
  // in-edges take a warp each; 0xFFFFFFFF: none) and whether the autotuner
  // found it faster than the graph of per-step launches
  int p_tpb = 256;
  uint32_t p_thr = 0xFFFFFFFFu;
  bool prefer_persistent = false;
  float tuned_graph_ms = 0, tuned_persistent_ms = 0;  // best trial of each form
  std::vector<uint32_t> host_rp;       // arena row pointers (autotuner, buckets)
  uint32_t heavy_thr = 0xFFFFFFFFu;    // threshold the heavy list was built for
  DevBuf heavy, is_heavy, bar;
  uint64_t nheavy = 0;
  DevBuf scratch_st[2], scratch_dy[2];  // autotuner trials run on copies of the state
  // CUDA graphs of `graph_steps` steps, one per starting buffer parity; the
  // step number comes from step_base (device) + the node's offset
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaGraph_t graph_def[2] = {nullptr, nullptr};
  int graph_steps = 0;
  DevBuf step_base;
};

namespace {

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
  a.st_wr = b->st[1 - cur].as<uint8_t>();
  a.d_wr = b->dy[1 - cur].as<int32_t>();
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

// one cooperative launch of `steps` steps from buffer `cur` (states in
// st/dy), the first with transition number step0
void launch_persistent(vg_batch *b, uint8_t *const st[2], int32_t *const dy[2], int cur,
                       uint32_t step0, uint32_t steps, int tpb, uint32_t thr) {
  build_buckets(b, thr);
  if (!b->bar.p) b->bar.alloc(8, &b->footprint);
  PersistArgs p{};
  p.a = batch_args(b, cur, step0, nullptr);
  p.st[0] = st[0];
  p.st[1] = st[1];
  p.dy[0] = dy[0];
  p.dy[1] = dy[1];
  p.cur0 = cur;
  p.steps = steps;
  p.step0 = step0;
  p.heavy = b->heavy.as<uint32_t>();
  p.nheavy = b->nheavy;
  p.is_heavy = b->nheavy ? b->is_heavy.as<uint8_t>() : nullptr;
  p.bar = b->bar.as<unsigned>();
  int dev = 0, sms = 0, per_sm = 0;
  VG_CUDA(cudaGetDevice(&dev));
  VG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  VG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_persist, tpb, 0));
  if (per_sm < 1) fail(VG_ERR_CUDA, "persistent batch kernel: no block fits an SM");
  unsigned grid = (unsigned)(sms * per_sm);  // every block resident: the barrier may wait
  VG_CUDA(cudaMemsetAsync(b->bar.p, 0, 8, b->stream));
  void *args[] = {&p};
  VG_CUDA(cudaLaunchCooperativeKernel((const void *)k_batch_persist, dim3(grid), dim3(tpb), args, 0,
                                      b->stream));
}

void launch_step(vg_batch *, const BatchArgs &a, int tpb, int apt, cudaStream_t st) {
  uint64_t threads = (a.n + apt - 1) / apt;
  unsigned g = blocks(threads, tpb);
  switch (apt) {
    case 1: k_batch_sir<1><<<g, tpb, 0, st>>>(a); break;
    case 2: k_batch_sir<2><<<g, tpb, 0, st>>>(a); break;
    default: k_batch_sir<4><<<g, tpb, 0, st>>>(a); break;
  }
}

// Choose the launch form by timing candidates on copies of the current
// state (the simulation state is not touched): per-step launches of the
// thread-per-agent kernel (block size 128/256/512 x agents per thread
// 1/2/4, replayed from a CUDA graph when stepping) and the persistent
// launch (block size 256/512 x bucket threshold: none, or warps for agents
// above 32 / 64 in-edges).  Keyed on the arena's agents, edges and in-degree
// histogram (log2 buckets).
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
    b->p_thr = it->second.p_thr;
    b->prefer_persistent = it->second.persistent;
    b->tuned_graph_ms = it->second.graph_ms;
    b->tuned_persistent_ms = it->second.persistent_ms;
    b->tuned = true;
    return;
  }
  // trial buffers: copies of the current state
  for (int k = 0; k < 2; k++) {
    if (!b->scratch_st[k].p) b->scratch_st[k].alloc(b->total, &b->footprint);
    if (!b->scratch_dy[k].p) b->scratch_dy[k].alloc(b->total * 4, &b->footprint);
  }
  uint8_t *sst[2] = {b->scratch_st[0].as<uint8_t>(), b->scratch_st[1].as<uint8_t>()};
  int32_t *sdy[2] = {b->scratch_dy[0].as<int32_t>(), b->scratch_dy[1].as<int32_t>()};
  auto reset = [&]() {
    VG_CUDA(cudaMemcpyAsync(sst[0], b->st[b->cur].p, b->total, cudaMemcpyDeviceToDevice, b->stream));
    VG_CUDA(cudaMemcpyAsync(sdy[0], b->dy[b->cur].p, b->total * 4, cudaMemcpyDeviceToDevice,
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
    for (int apt : {1, 2, 4}) {
      const float ms = timed([&] {
        for (uint32_t t = 0; t < TRIAL; t++) {
          BatchArgs a = batch_args(b, 0, (uint32_t)b->step + t, nullptr);
          a.st_rd = sst[t & 1];
          a.d_rd = sdy[t & 1];
          a.st_wr = sst[1 - (t & 1)];
          a.d_wr = sdy[1 - (t & 1)];
          launch_step(b, a, tpb, apt, b->stream);
        }
      });
      if (ms < best) {
        best = ms;
        bt = tpb;
        ba = apt;
      }
    }
  float pbest = 1e30f;
  int pt = 256;
  uint32_t pthr = 0xFFFFFFFFu;
  for (int tpb : {256, 512})
    for (uint32_t thr : {0xFFFFFFFFu, 64u, 32u}) {
      const float ms = timed([&] {
        launch_persistent(b, sst, sdy, 0, (uint32_t)b->step, TRIAL, tpb, thr);
      });
      if (ms < pbest) {
        pbest = ms;
        pt = tpb;
        pthr = thr;
      }
    }
  VG_CUDA(cudaEventDestroy(e0));
  VG_CUDA(cudaEventDestroy(e1));
  check_batch_status(b);
  b->tpb = bt;
  b->apt = ba;
  b->p_tpb = pt;
  b->p_thr = pthr;
  b->prefer_persistent = pbest < best;
  b->tuned_graph_ms = best / TRIAL;
  b->tuned_persistent_ms = pbest / TRIAL;
  b->tuned = true;
  b->tune_cache[key] = {bt, ba, pt, pthr, b->prefer_persistent, b->tuned_graph_ms,
                        b->tuned_persistent_ms};
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
  if (mode < 0 || mode > 3) fail(VG_ERR_ARG, "batch: mode 0..3");
  if (steps <= 0) return VG_OK;
  if (!b->tuned) autotune(b);
  if (mode == 3) mode = b->prefer_persistent ? 2 : 1;
  if (mode == 2) {
    uint8_t *st[2] = {b->st[0].as<uint8_t>(), b->st[1].as<uint8_t>()};
    int32_t *dy[2] = {b->dy[0].as<int32_t>(), b->dy[1].as<int32_t>()};
    launch_persistent(b, st, dy, b->cur, (uint32_t)b->step, (uint32_t)steps, b->p_tpb, b->p_thr);
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
      VG_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      int cur = p;
      for (int k = 0; k < steps; k++) {
        BatchArgs a = batch_args(b, cur, (uint32_t)k, b->step_base.as<int64_t>());
        launch_step(b, a, b->tpb, b->apt, cs);
        cur = 1 - cur;
      }
      VG_CUDA(cudaStreamEndCapture(cs, &b->graph_def[p]));
      VG_CUDA(cudaGraphInstantiate(&b->graph[p], b->graph_def[p], 0));
      VG_CUDA(cudaStreamDestroy(cs));
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
  k_barrier_probe<<<2, 64>>>(bar, 3, status, 1u << 16);  // two blocks, three expected
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
  if (persistent_tpb != 128 && persistent_tpb != 256 && persistent_tpb != 512)
    fail(VG_ERR_ARG, "batch: persistent block size 128, 256 or 512");
  if (!b->tuned) autotune(b);
  b->prefer_persistent = persistent != 0;
  b->p_tpb = persistent_tpb;
  b->p_thr = bucket_threshold;
  API_END
}

int vg_batch_tuning(vg_batch *b, int *persistent, int *persistent_tpb,
                    uint32_t *bucket_threshold, uint64_t *heavy_agents,
                    double *step_ms_graph, double *step_ms_persistent) {
  API_BEGIN
  if (!b) fail(VG_ERR_ARG, "null batch");
  if (!b->tuned) autotune(b);
  if (step_ms_graph) *step_ms_graph = b->tuned_graph_ms;
  if (step_ms_persistent) *step_ms_persistent = b->tuned_persistent_ms;
  if (persistent) *persistent = b->prefer_persistent;
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
