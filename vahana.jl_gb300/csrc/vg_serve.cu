// Serving loop: simulation jobs arrive over time, are admitted while their
// device footprint fits a budget, are stepped together (continuous
// batching: every tick advances every resident job by one transition in one
// launch per model), and are retired when their step count is reached.
//
// A job is an ordinary simulation (the "SIR" or the opinion model of the
// test models), built on the server's stream when admitted.  A tick runs
// the same per-job work as the job's own apply! (the SIR rule with the
// job's table; the bounded-confidence blocks through launch_opinion_jobs)
// and then the job's finish of the transition (buffer swap,
// num_transitions += 1), so each job's state after k ticks equals the
// state after k apply! calls on that job alone.
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "vg_internal.h"
#include "vg_philox.cuh"

namespace vg {
void set_last_error(const std::string &m);
}  // namespace vg

using namespace vg;


namespace {

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

uint64_t fnv1a(const void *p, size_t n, uint64_t h = 1469598103934665603ull) {
  const uint8_t *b = (const uint8_t *)p;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

struct Job {
  int64_t id;
  vg_job_spec spec;
  double arrival = 0, admit = 0, finish = 0;
  vg_sim *sim = nullptr;
  int done_steps = 0;
  DevBuf ptab;  // SIR: p_k table
  uint32_t ptab_n = 0;
  uint64_t est_bytes = 0;
  std::vector<uint8_t> final_state;
  vg_job_result result{};
  cudaEvent_t done_ev = nullptr;  // recorded after the job's last tick
};

struct SirJobDesc {
  const uint32_t *rp;
  const uint32_t *src;
  const uint8_t *st_rd;
  const int32_t *d_rd;
  uint8_t *st_wr;
  int32_t *d_wr;
  uint64_t n, nrows;
  const double *ptab;
  uint32_t ptab_n;
  uint32_t step;
  uint64_t seed;
  int32_t recovery;
};

struct SirTile {
  uint32_t job;
  uint32_t start;
};

// the SIR rule of transition "sir" for the agents of one tile of one job
__global__ void k_sir_jobs(const SirJobDesc *jobs, const SirTile *tiles, int *status) {
  SirTile t = tiles[blockIdx.x];
  const SirJobDesc &j = jobs[t.job];
  uint64_t i = (uint64_t)t.start + threadIdx.x;
  if (i >= j.n) return;
  uint8_t s = j.st_rd[i];
  int32_t d = j.d_rd[i];
  if (s == 0) {
    uint32_t k = 0;
    if (i < j.nrows) {
      uint32_t e = j.rp[i + 1];
      for (uint32_t q = j.rp[i]; q < e; q++) k += (__ldg(j.st_rd + j.src[q]) == 1);
    }
    if (k > 0) {
      if (k >= j.ptab_n) {
        atomicCAS(status, 0, 401);
      } else {
        if (unit_below(philox_u64(philox_draw(j.seed, i + 1, j.step, TAG_INFECT)), j.ptab[k])) {
          s = 1;
          d = 0;
        }
      }
    }
  } else if (s == 1) {
    d = d + 1;
    if (d >= j.recovery) s = 2;
  }
  j.st_wr[i] = s;
  j.d_wr[i] = d;
}

}  // namespace

// Threads: one worker admits jobs and ticks the resident ones on the
// server's stream; BUILDERS builder threads (each with its own stream) build
// admitted jobs -- graph generation, CSR and gather layout -- while the
// worker keeps ticking, and hand them over through `ready`.
//
// The worker does not wait for a tick before issuing the next: up to
// MAX_INFLIGHT ticks are queued on the stream (a tick's launches only read
// descriptors that the stream's own copies wrote before them).  A job that
// reaches its step count leaves the resident set at once; an event recorded
// after its last tick tells when its final state may be read, which a copy on
// a separate stream then does.  Freeing device memory waits for the whole
// device, so finished jobs' simulations are destroyed in batches
// (GRAVE_BATCH at a time, when admission needs their budget, or when nothing
// is resident); their budget is returned then.
constexpr int BUILDERS = 4;
constexpr size_t MAX_INFLIGHT = 2;
constexpr size_t GRAVE_BATCH = 16;

struct vg_server {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  int device = 0;  // the device current at vg_serve_create: every thread runs there
  uint64_t budget = 0, used = 0;
  int max_active = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t build_stream[BUILDERS] = {};
  vg_model *sir_model = nullptr, *op_model = nullptr;
  int sir_person = 0, sir_contact = 0, op_agent = 0, op_edge = 0;
  std::thread worker;
  std::thread builders[BUILDERS];
  std::mutex mu;
  std::condition_variable cv;        // worker: submissions, finished builds
  std::condition_variable build_cv;  // builders: admitted jobs
  bool stop = false;           // no more submissions: finish every job, then exit
  bool builders_stop = false;  // set once the worker has exited
  std::string error;
  int64_t next_id = 1;
  std::deque<Job *> queue;      // submitted, not admitted
  std::deque<Job *> to_build;   // admitted, not yet picked by a builder
  int building = 0;             // picked by a builder
  std::vector<Job *> ready;     // built, not yet resident
  std::vector<Job *> active;    // resident: stepped every tick
  std::vector<Job *> done;
  uint64_t ticks = 0, sim_steps = 0;
  uint64_t footprint = 0;
  DevBuf sir_jobs_buf, sir_tiles_buf, op_args_buf, op_tiles_buf, status;
  // pipelining (worker thread only)
  cudaStream_t retire_stream = nullptr;  // final-state copies of finished jobs
  int *status_host = nullptr;            // pinned: the status word after a tick
  std::deque<cudaEvent_t> inflight;      // one per queued tick, oldest first
  std::vector<cudaEvent_t> ev_pool;
  std::deque<Job *> retiring;            // finished, final state not read yet
  std::vector<Job *> graveyard;          // read back (in `done`), simulation not freed
};

namespace {

uint64_t estimate_bytes(const vg_job_spec &s) {
  double n = (double)s.n, e = s.mean_degree * n;
  if (s.model == 0) {  // state 2x5 B, rows, sources, build staging (16 B/edge + sort)
    return (uint64_t)(10 * n + 4 * n + 4 * e + 32 * e + 8 * n) + (1 << 20);
  }
  // opinion: 2x8 B state, rows + order, 12 B/edge, build staging 24 B/edge + sort
  return (uint64_t)(16 * n + 12 * n + 12 * e + 40 * e) + (1 << 20);
}

void build_job(vg_server *S, Job *J, cudaStream_t bst) {
  int rc;
  const vg_job_spec &sp = J->spec;
  if (sp.model == 0) {
    if ((rc = vg_sim_create(S->sir_model, "job", bst, &J->sim))) fail(rc, vg_last_error());
    std::vector<uint8_t> st;
    uint64_t ninf = (uint64_t)std::max<double>(1.0, std::nearbyint((double)sp.n / 1000.0));
    sir_initial_state(sp.n, sp.seed, ninf, st);
    std::vector<int32_t> days(sp.n, 0);
    const void *cols[2] = {st.data(), days.data()};
    if ((rc = vg_add_agents(J->sim, S->sir_person, sp.n, cols, nullptr))) fail(rc, vg_last_error());
    if (sp.fail_build) fail(VG_ERR_STATE, "job build failed (injected after its agents were added)");
    if ((rc = vg_gen_uniform_out_edges(J->sim, S->sir_contact, S->sir_person,
                                       (uint32_t)std::lround(sp.mean_degree), sp.seed)))
      fail(rc, vg_last_error());
    if ((rc = vg_finish_init(J->sim))) fail(rc, vg_last_error());
    Sim &s = *J->sim->s;
    uint32_t maxdeg = csr_max_degree(s, s.edges[S->sir_contact].csr[S->sir_person]);
    std::vector<double> tab(maxdeg + 1);
    double q = 1.0, om = 1.0 - sp.beta;
    tab[0] = 0.0;
    for (uint32_t k = 1; k <= maxdeg; k++) {  // p_k = 1 - (1 - beta)^k, as the "sir" kernel
      q = q * om;
      tab[k] = 1.0 - q;
    }
    J->ptab.alloc(tab.size() * 8, &s.footprint);
    VG_CUDA(cudaMemcpyAsync(J->ptab.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, bst));
    VG_CUDA(cudaStreamSynchronize(bst));
    J->ptab_n = (uint32_t)tab.size();
  } else {
    if ((rc = vg_sim_create(S->op_model, "job", bst, &J->sim))) fail(rc, vg_last_error());
    std::vector<double> x(sp.n);
    for (uint64_t i = 0; i < sp.n; i++)
      x[i] = u64_to_unit(philox_u64(philox_draw(sp.seed, i + 1, 0, TAG_INIT)));
    const void *cols[1] = {x.data()};
    if ((rc = vg_add_agents(J->sim, S->op_agent, sp.n, cols, nullptr))) fail(rc, vg_last_error());
    if (sp.fail_build) fail(VG_ERR_STATE, "job build failed (injected after its agents were added)");
    uint64_t ne = (uint64_t)std::nearbyint(sp.mean_degree * (double)sp.n);
    if ((rc = vg_gen_chung_lu_edges(J->sim, S->op_edge, S->op_agent, ne, sp.mean_degree, 2.5,
                                    sp.wmax, sp.seed, 0)))
      fail(rc, vg_last_error());
    if ((rc = vg_finish_init(J->sim))) fail(rc, vg_last_error());
    prepare_opinion_job({J->sim->s.get(), S->op_edge, S->op_agent, J->spec.eps, 0.5, 0.5,
                         OPINION_HUB_DEFAULT});
  }
}

// the final state of a finished job whose last tick has completed: read
// back (on the retire stream: the job is no longer touched by the ticks
// queued after it), hashed and summarised; the simulation stays allocated
void read_back(vg_server *S, Job *J) {
  Sim &s = *J->sim->s;
  vg_job_result &r = J->result;
  r.id = J->id;
  r.model = J->spec.model;
  r.n = J->spec.n;
  r.steps = J->spec.steps;
  r.arrival_s = J->arrival;
  r.admit_s = J->admit;
  r.device_bytes = s.footprint;
  int T = J->spec.model == 0 ? S->sir_person : S->op_agent;
  AgentStore &A = s.agents[T - 1];
  std::vector<uint8_t> bytes;
  cudaStream_t rs = S->retire_stream;
  if (J->spec.model == 0) {
    bytes.resize(A.n * 5);
    VG_CUDA(cudaMemcpyAsync(bytes.data(), A.rd[0].p, A.n, cudaMemcpyDeviceToHost, rs));
    VG_CUDA(cudaMemcpyAsync(bytes.data() + A.n, A.rd[1].p, A.n * 4, cudaMemcpyDeviceToHost, rs));
    VG_CUDA(cudaStreamSynchronize(rs));
    uint64_t rcount = 0;
    for (uint64_t i = 0; i < A.n; i++) rcount += bytes[i] == 2;
    r.summary = A.n ? (double)rcount / (double)A.n : 0.0;
  } else {
    bytes.resize(A.n * 8);
    VG_CUDA(cudaMemcpyAsync(bytes.data(), A.rd[0].p, A.n * 8, cudaMemcpyDeviceToHost, rs));
    VG_CUDA(cudaStreamSynchronize(rs));
    double m = 0;
    const double *x = (const double *)bytes.data();
    for (uint64_t i = 0; i < A.n; i++) m += x[i];
    r.summary = A.n ? m / (double)A.n : 0.0;
  }
  r.checksum = fnv1a(bytes.data(), bytes.size());
  if (J->spec.keep_state) J->final_state = std::move(bytes);
  r.finish_s = now_s(S->t0);
  J->finish = r.finish_s;
}

void free_job_sim(Job *J) {
  J->ptab.release();  // before the simulation whose byte counter it updates
  if (J->sim) vg_sim_destroy(J->sim);
  J->sim = nullptr;
}

void check_status(vg_server *S) {
  if (*(volatile int *)S->status_host)
    fail(VG_ERR_DEVICE, "serving tick: device status " + std::to_string(*S->status_host));
}

// drop the events of completed ticks; with `keep`, wait until at most that
// many ticks are queued
void settle_ticks(vg_server *S, size_t keep) {
  while (!S->inflight.empty()) {
    cudaEvent_t ev = S->inflight.front();
    if (S->inflight.size() > keep) {
      VG_CUDA(cudaEventSynchronize(ev));
    } else {
      const cudaError_t q = cudaEventQuery(ev);
      if (q == cudaErrorNotReady) break;
      VG_CUDA(q);
    }
    S->inflight.pop_front();
    S->ev_pool.push_back(ev);
    check_status(S);
  }
}

// finished jobs whose last tick has completed (all of them with `wait`):
// results to `done`, simulations to the graveyard
void reap_finished(vg_server *S, bool wait) {
  while (!S->retiring.empty()) {
    Job *J = S->retiring.front();
    if (wait) {
      VG_CUDA(cudaEventSynchronize(J->done_ev));
    } else {
      const cudaError_t q = cudaEventQuery(J->done_ev);
      if (q == cudaErrorNotReady) break;
      VG_CUDA(q);
    }
    check_status(S);
    read_back(S, J);
    VG_CUDA(cudaEventDestroy(J->done_ev));
    J->done_ev = nullptr;
    S->retiring.pop_front();
    S->graveyard.push_back(J);
    std::lock_guard<std::mutex> lk(S->mu);
    S->done.push_back(J);
  }
}

// free the graveyard's simulations (each free waits for the device) and
// return their budget
void flush_graveyard(vg_server *S) {
  if (S->graveyard.empty()) return;
  uint64_t bytes = 0;
  for (Job *J : S->graveyard) {
    free_job_sim(J);
    bytes += J->est_bytes;
  }
  S->graveyard.clear();
  std::lock_guard<std::mutex> lk(S->mu);
  S->used -= bytes;
}

// one transition of every resident job
void tick(vg_server *S) {
  cudaStream_t st = S->stream;
  std::vector<SirJobDesc> sj;
  std::vector<SirTile> stiles;
  std::vector<OpinionJob> oj;
  std::vector<Job *> sir_jobs, op_jobs;
  std::vector<Job *> stepping;
  for (Job *J : S->active)
    if (J->done_steps < J->spec.steps) stepping.push_back(J);
  for (Job *J : stepping) {
    Sim &s = *J->sim->s;
    if (J->spec.model == 0) {
      int T = S->sir_person;
      AgentStore &A = s.agents[T - 1];
      CSR &c = s.edges[S->sir_contact].csr[T];
      SirJobDesc d{};
      d.rp = c.row_ptr.as<uint32_t>();
      d.src = c.src.as<uint32_t>();
      d.st_rd = A.rd[0].as<uint8_t>();
      d.d_rd = A.rd[1].as<int32_t>();
      d.st_wr = A.wr[0].as<uint8_t>();
      d.d_wr = A.wr[1].as<int32_t>();
      d.n = A.n;
      d.nrows = c.nrows;
      d.ptab = J->ptab.as<double>();
      d.ptab_n = J->ptab_n;
      d.step = (uint32_t)s.num_transitions;
      d.seed = J->spec.seed;
      d.recovery = J->spec.recovery;
      uint32_t ji = (uint32_t)sj.size();
      sj.push_back(d);
      for (uint64_t a = 0; a < A.n; a += 256) stiles.push_back({ji, (uint32_t)a});
      sir_jobs.push_back(J);
    } else {
      oj.push_back({&s, S->op_edge, S->op_agent, J->spec.eps, 0.5, 0.5, OPINION_HUB_DEFAULT});
      op_jobs.push_back(J);
    }
  }
  if (!stiles.empty()) {
    if (S->sir_jobs_buf.bytes < sj.size() * sizeof(SirJobDesc))
      S->sir_jobs_buf.alloc(sj.size() * sizeof(SirJobDesc) * 2, &S->footprint);
    if (S->sir_tiles_buf.bytes < stiles.size() * sizeof(SirTile))
      S->sir_tiles_buf.alloc(stiles.size() * sizeof(SirTile) * 2, &S->footprint);
    VG_CUDA(cudaMemcpyAsync(S->sir_jobs_buf.p, sj.data(), sj.size() * sizeof(SirJobDesc),
                            cudaMemcpyHostToDevice, st));
    VG_CUDA(cudaMemcpyAsync(S->sir_tiles_buf.p, stiles.data(), stiles.size() * sizeof(SirTile),
                            cudaMemcpyHostToDevice, st));
    k_sir_jobs<<<(unsigned)stiles.size(), 256, 0, st>>>(
        S->sir_jobs_buf.as<SirJobDesc>(), S->sir_tiles_buf.as<SirTile>(), S->status.as<int>());
    VG_CUDA(cudaGetLastError());
  }
  if (!oj.empty()) launch_opinion_jobs(oj, st, S->op_args_buf, S->op_tiles_buf, &S->footprint);
  // the status word as of this tick, read once the tick's event has completed
  VG_CUDA(cudaMemcpyAsync(S->status_host, S->status.p, 4, cudaMemcpyDeviceToHost, st));
  cudaEvent_t ev;
  if (S->ev_pool.empty()) {
    VG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  } else {
    ev = S->ev_pool.back();
    S->ev_pool.pop_back();
  }
  VG_CUDA(cudaEventRecord(ev, st));
  S->inflight.push_back(ev);
  // finish of the transition of every job (as apply! for its immortal type)
  for (Job *J : stepping) {
    Sim &s = *J->sim->s;
    int T = J->spec.model == 0 ? S->sir_person : S->op_agent;
    std::swap(s.agents[T - 1].rd, s.agents[T - 1].wr);
    s.num_transitions++;
    J->done_steps++;
  }
  S->ticks++;
  S->sim_steps += stepping.size();
}

void fail_server(vg_server *S, const std::string &msg) {
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->error.empty()) S->error = msg;
  S->stop = true;
  S->builders_stop = true;
  S->cv.notify_all();
  S->build_cv.notify_all();
}

// A job whose build fails is retired at once with the error (its partial
// simulation released); the server and the other jobs go on.
void retire_failed_build(vg_server *S, Job *J, int code, const std::string &msg) {
  J->ptab.release();
  if (J->sim) vg_sim_destroy(J->sim);
  J->sim = nullptr;
  vg_job_result &r = J->result;
  r = vg_job_result{};
  r.id = J->id;
  r.model = J->spec.model;
  r.n = J->spec.n;
  r.steps = J->spec.steps;
  r.arrival_s = J->arrival;
  r.admit_s = J->admit;
  r.status = code ? code : VG_ERR_STATE;
  std::snprintf(r.error, sizeof(r.error), "%s", msg.c_str());
  r.finish_s = now_s(S->t0);
  J->finish = r.finish_s;
}

void builder_loop(vg_server *S, int b) {
  try {
    VG_CUDA(cudaSetDevice(S->device));
    while (true) {
      Job *J = nullptr;
      {
        std::unique_lock<std::mutex> lk(S->mu);
        // builders outlive the worker's admissions: they leave only after the
        // worker has exited (or on an error)
        S->build_cv.wait(lk, [&] { return !S->to_build.empty() || S->builders_stop; });
        if (S->to_build.empty()) return;
        J = S->to_build.front();
        S->to_build.pop_front();
        S->building++;
      }
      bool built = true;
      try {
        build_job(S, J, S->build_stream[b]);
      } catch (const Error &e) {
        retire_failed_build(S, J, e.code, e.msg);
        built = false;
      }
      {
        std::lock_guard<std::mutex> lk(S->mu);
        S->building--;
        if (built) {
          S->ready.push_back(J);
        } else {
          S->used -= J->est_bytes;
          S->done.push_back(J);
        }
      }
      S->cv.notify_one();
    }
  } catch (const Error &e) {
    fail_server(S, e.msg);
  }
}

void worker_loop(vg_server *S) {
  try {
    VG_CUDA(cudaSetDevice(S->device));
    while (true) {
      settle_ticks(S, MAX_INFLIGHT);
      reap_finished(S, false);
      bool need_budget = false, idle = false;
      {
        std::lock_guard<std::mutex> lk(S->mu);
        need_budget = !S->queue.empty() && S->used + S->queue.front()->est_bytes > S->budget;
        idle = S->active.empty() && S->ready.empty();
      }
      if (S->graveyard.size() >= GRAVE_BATCH || (need_budget && !S->graveyard.empty()) || idle)
        flush_graveyard(S);
      std::vector<Job *> arrived;
      {
        std::unique_lock<std::mutex> lk(S->mu);
        if (!S->error.empty()) return;
        // admission, first come first served, by estimated footprint
        bool admitted = false;
        while (!S->queue.empty()) {
          Job *J = S->queue.front();
          const size_t inflight = S->active.size() + S->ready.size() + S->to_build.size() +
                                  (size_t)S->building;
          bool fits = S->used + J->est_bytes <= S->budget && (int)inflight < S->max_active;
          bool alone = inflight == 0 && S->graveyard.empty() && S->retiring.empty();
          if (!fits && !alone) break;
          S->queue.pop_front();
          S->used += J->est_bytes;
          J->admit = now_s(S->t0);
          S->to_build.push_back(J);
          admitted = true;
        }
        if (admitted) S->build_cv.notify_all();
        arrived.swap(S->ready);
        if (arrived.empty() && S->active.empty()) {
          if (!S->retiring.empty() || !S->graveyard.empty() || !S->inflight.empty()) {
            lk.unlock();  // nothing to tick: finish the queued work first
            settle_ticks(S, 0);
            reap_finished(S, true);
            flush_graveyard(S);
            continue;
          }
          if (S->stop && S->queue.empty() && S->to_build.empty() && S->building == 0) break;
          S->cv.wait_for(lk, std::chrono::milliseconds(2));
          continue;
        }
      }
      for (Job *J : arrived) S->active.push_back(J);
      tick(S);
      std::vector<Job *> still;
      for (Job *J : S->active) {
        if (J->done_steps >= J->spec.steps) {
          VG_CUDA(cudaEventCreateWithFlags(&J->done_ev, cudaEventDisableTiming));
          VG_CUDA(cudaEventRecord(J->done_ev, S->stream));
          S->retiring.push_back(J);
        } else {
          still.push_back(J);
        }
      }
      std::lock_guard<std::mutex> lk(S->mu);
      S->active.swap(still);
    }
  } catch (const Error &e) {
    fail_server(S, e.msg);
  }
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

int vg_serve_create(uint64_t budget_bytes, int max_active, vg_server **out) {
  API_BEGIN
  need(out, "output pointer");
  auto S = std::make_unique<vg_server>();
  S->budget = budget_bytes;
  S->max_active = max_active > 0 ? max_active : 1 << 20;
  VG_CUDA(cudaGetDevice(&S->device));
  VG_CUDA(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
  int rc;
  if ((rc = vg_model_create(&S->sir_model))) fail(rc, vg_last_error());
  const char *pf[2] = {"state", "days"};
  int pd[2] = {VG_U8, VG_I32};
  if ((rc = vg_model_register_agenttype(S->sir_model, "Person", 2, pf, pd, VG_HINT_IMMORTAL,
                                         &S->sir_person)) ||
      (rc = vg_model_register_edgetype(S->sir_model, "Contact", 0, nullptr, nullptr,
                                        VG_HINT_STATELESS, S->sir_person, 0, &S->sir_contact)) ||
      (rc = vg_model_finalize(S->sir_model, "SIR")))
    fail(rc, vg_last_error());
  if ((rc = vg_model_create(&S->op_model))) fail(rc, vg_last_error());
  const char *of[1] = {"x"};
  int od[1] = {VG_F64};
  const char *wf[1] = {"w"};
  if ((rc = vg_model_register_agenttype(S->op_model, "Opinion", 1, of, od, VG_HINT_IMMORTAL,
                                         &S->op_agent)) ||
      (rc = vg_model_register_edgetype(S->op_model, "Weight", 1, wf, od, 0, S->op_agent, 0,
                                        &S->op_edge)) ||
      (rc = vg_model_finalize(S->op_model, "Opinion")))
    fail(rc, vg_last_error());
  S->status.alloc(16, &S->footprint);
  VG_CUDA(cudaMemset(S->status.p, 0, 16));
  VG_CUDA(cudaHostAlloc((void **)&S->status_host, 4, cudaHostAllocDefault));
  *S->status_host = 0;
  VG_CUDA(cudaStreamCreateWithFlags(&S->retire_stream, cudaStreamNonBlocking));
  for (int b = 0; b < BUILDERS; b++)
    VG_CUDA(cudaStreamCreateWithFlags(&S->build_stream[b], cudaStreamNonBlocking));
  vg_server *raw = S.release();
  raw->worker = std::thread(worker_loop, raw);
  for (int b = 0; b < BUILDERS; b++) raw->builders[b] = std::thread(builder_loop, raw, b);
  *out = raw;
  API_END
}

int vg_serve_submit(vg_server *S, const vg_job_spec *spec, int64_t *id_out) {
  API_BEGIN
  if (!S) fail(VG_ERR_ARG, "null server");
  need(spec, "job spec");
  if (spec->model != 0 && spec->model != 1) fail(VG_ERR_ARG, "job model 0 (SIR) or 1 (opinion)");
  if (spec->n < 2 || spec->steps < 0) fail(VG_ERR_ARG, "job size");
  Job *J = new Job();
  J->spec = *spec;
  if (J->spec.model == 1 && J->spec.wmax <= 0) J->spec.wmax = 1e4;
  J->est_bytes = estimate_bytes(J->spec);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->error.empty()) {
      delete J;
      fail(VG_ERR_STATE, "server stopped: " + S->error);
    }
    J->id = S->next_id++;
    J->arrival = now_s(S->t0);
    S->queue.push_back(J);
  }
  S->cv.notify_one();
  if (id_out) *id_out = J->id;
  API_END
}

// finished jobs since the last poll (at most cap); *n_out = number written
int vg_serve_poll(vg_server *S, vg_job_result *out, uint64_t cap, uint64_t *n_out) {
  API_BEGIN
  if (!S) fail(VG_ERR_ARG, "null server");
  need(n_out, "count pointer");
  if (cap) need(out, "result array");
  std::lock_guard<std::mutex> lk(S->mu);
  if (!S->error.empty()) fail(VG_ERR_DEVICE, "server stopped: " + S->error);
  uint64_t k = 0;
  for (Job *J : S->done) {
    if (J->result.id == 0) continue;  // already reported
    if (k >= cap) break;
    out[k++] = J->result;
    J->result.id = 0;
  }
  *n_out = k;
  API_END
}

// the final state bytes of a finished job submitted with keep_state
int vg_serve_job_state(vg_server *S, int64_t id, void *out, uint64_t cap, uint64_t *n_out) {
  API_BEGIN
  if (!S) fail(VG_ERR_ARG, "null server");
  need(n_out, "count pointer");
  std::lock_guard<std::mutex> lk(S->mu);
  for (Job *J : S->done)
    if (J->id == id) {
      *n_out = J->final_state.size();
      if (out) std::memcpy(out, J->final_state.data(), std::min<uint64_t>(cap, J->final_state.size()));
      return VG_OK;
    }
  fail(VG_ERR_ARG, "no finished job with this id");
  API_END
}

int vg_serve_stats(vg_server *S, uint64_t *queued, uint64_t *active, uint64_t *done,
                   uint64_t *ticks, uint64_t *sim_steps, uint64_t *bytes_in_use) {
  API_BEGIN
  if (!S) fail(VG_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(S->mu);
  if (queued) *queued = S->queue.size();
  if (active) *active = S->active.size();
  if (done) *done = S->done.size();
  if (ticks) *ticks = S->ticks;
  if (sim_steps) *sim_steps = S->sim_steps;
  if (bytes_in_use) *bytes_in_use = S->used;
  API_END
}

// stop accepting, finish every queued and resident job, join the worker
static void stop_threads(vg_server *S) {
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  if (S->worker.joinable()) S->worker.join();  // every admitted job built, stepped, retired
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->builders_stop = true;
  }
  S->build_cv.notify_all();
  for (auto &t : S->builders)
    if (t.joinable()) t.join();
}

int vg_serve_drain(vg_server *S) {
  API_BEGIN
  if (!S) fail(VG_ERR_ARG, "null server");
  stop_threads(S);
  if (!S->error.empty()) fail(VG_ERR_DEVICE, "server stopped: " + S->error);
  API_END
}

int vg_serve_destroy(vg_server *S) {
  API_BEGIN
  if (!S) return VG_OK;
  stop_threads(S);
  for (auto *q : {&S->queue, &S->to_build})
    for (Job *J : *q) delete J;
  for (auto *v : {&S->ready, &S->active})
    for (Job *J : *v) {
      free_job_sim(J);
      delete J;
    }
  cudaStreamSynchronize(S->stream);  // (after an error: queued ticks end before their jobs go)
  for (Job *J : S->retiring) {
    if (J->done_ev) cudaEventDestroy(J->done_ev);
    free_job_sim(J);
    delete J;
  }
  for (Job *J : S->graveyard) free_job_sim(J);  // (also in done)
  for (Job *J : S->done) delete J;
  for (cudaEvent_t e : S->inflight) cudaEventDestroy(e);
  for (cudaEvent_t e : S->ev_pool) cudaEventDestroy(e);
  if (S->status_host) cudaFreeHost(S->status_host);
  if (S->retire_stream) cudaStreamDestroy(S->retire_stream);
  vg_model_destroy(S->sir_model);
  vg_model_destroy(S->op_model);
  cudaStream_t st = S->stream;
  cudaStream_t bst[BUILDERS];
  for (int b = 0; b < BUILDERS; b++) bst[b] = S->build_stream[b];
  delete S;
  cudaStreamDestroy(st);
  for (int b = 0; b < BUILDERS; b++) cudaStreamDestroy(bst[b]);
  API_END
}

}  // extern "C"
