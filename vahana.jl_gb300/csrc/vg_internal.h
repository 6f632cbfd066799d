// Internal runtime structures of libvahana_gb300.
//
// Layout in HBM (one simulation):
//   agent type T  : n slots (nextid-1); per field a read and a write column
//                   (SoA, dtype-sized); died_rd/died_wr byte columns for
//                   mortal types; a device stack of reusable agent numbers.
//   edge type E   : per target agent type one CSR: row_ptr u32[n_T+1] over
//                   target slots, src u32[E] (agent_nr-1 of the source),
//                   src_type u8[E] only when sources have several types,
//                   one column per payload field.  Edges of a row are in the
//                   reference's insertion order.
//   implicit raster edges keep no CSR: a stencil descriptor answers rows.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/vahana_gb300.h"

namespace vg {

constexpr int MAX_FIELDS = 8;
constexpr int MAX_AGENT_TYPES = 16;  // type numbers 1..15
constexpr int MAX_EDGE_TYPES = 64;
constexpr int MAX_DIMS = 4;
constexpr int SHIFT_TYPE = 56;   // src/Agent.jl:64 (BITS_PROCESS + BITS_AGENTNR)
constexpr int SHIFT_RANK = 36;   // src/Agent.jl:65
constexpr uint64_t NR_MASK = (1ull << 36) - 1;

inline uint64_t make_id(int type_nr, uint64_t nr) {
  return ((uint64_t)type_nr << SHIFT_TYPE) | nr;  // process bits stay 0
}
inline int id_type(uint64_t id) { return (int)(id >> SHIFT_TYPE); }
inline uint64_t id_nr(uint64_t id) { return id & NR_MASK; }
inline int id_process(uint64_t id) { return (int)((id >> SHIFT_RANK) & 0xFFFFF); }

int dtype_size(int dt);

struct Error {
  int code;
  std::string msg;
};
[[noreturn]] void fail(int code, const std::string &msg);

// A pointer argument a C-ABI entry cannot do without: null fails with
// VG_ERR_ARG instead of being dereferenced.
template <class T>
inline T *need(T *p, const char *what) {
  if (!p) fail(VG_ERR_ARG, std::string("null ") + what);
  return p;
}
void cuda_check(cudaError_t e, const char *what);
#define VG_CUDA(x) ::vg::cuda_check((x), #x)
#define VG_REQUIRE(cond, msg) \
  do {                        \
    if (!(cond)) ::vg::fail(VG_ERR_ASSERT, (msg)); \
  } while (0)

// ---------------------------------------------------------------- buffers
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  uint64_t *footprint = nullptr;  // owning simulation's byte counter
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept { *this = std::move(o); }
  DevBuf &operator=(DevBuf &&o) noexcept;
  ~DevBuf() { release(); }
  void alloc(size_t b, uint64_t *fp);
  void release();
  template <class T> T *as() const { return (T *)p; }
};

// ---------------------------------------------------------------- model
struct FieldDesc {
  std::string name;
  int dtype;
  int size;
};

struct AgentTypeDesc {
  std::string name;
  std::vector<FieldDesc> fields;
  unsigned hints = 0;
  int nr = 0;
  bool immortal() const { return hints & VG_HINT_IMMORTAL; }
  bool independent() const { return hints & VG_HINT_INDEPENDENT; }
  int field_index(const std::string &n) const;
};

struct EdgeTypeDesc {
  std::string name;
  std::vector<FieldDesc> fields;
  unsigned hints = 0;  // normalised (NumEdgesOnly / HasEdgeOnly expanded)
  int target = 0;      // :SingleType target type number
  int64_t size = 0;
  int idx = 0;
  bool stateless() const { return hints & VG_HINT_STATELESS; }
  bool ignorefrom() const { return hints & VG_HINT_IGNOREFROM; }
  bool singletype() const { return hints & VG_HINT_SINGLETYPE; }
  bool singleedge() const { return hints & VG_HINT_SINGLEEDGE; }
  bool stores_src() const { return !ignorefrom(); }
  bool stores_payload() const { return !stateless() && !fields.empty(); }
  bool count_only() const { return stateless() && ignorefrom() && !singleedge(); }
  bool bool_only() const { return stateless() && ignorefrom() && singleedge(); }
  int field_index(const std::string &n) const;
};

struct Model {
  std::string name;
  std::vector<AgentTypeDesc> atypes;  // index = nr - 1
  std::vector<EdgeTypeDesc> etypes;   // index = edge type index
  std::vector<std::pair<std::string, double>> params, globals;
  bool finalized = false;
  bool all_immortal() const {
    for (auto &a : atypes)
      if (!a.immortal()) return false;
    return true;
  }
  const AgentTypeDesc &at(int nr) const;
  const EdgeTypeDesc &et(int e) const;
};

// ---------------------------------------------------------------- state
struct AgentStore {
  uint64_t n = 0;    // slots in use = nextid - 1 (src/AgentMethods.jl:37-63)
  uint64_t cap = 0;  // allocated slots
  std::vector<DevBuf> rd, wr;
  DevBuf died_rd, died_wr;  // mortal types only
  DevBuf reuse;             // u64 agent numbers, LIFO (readreuseable)
  uint64_t nreuse = 0, reuse_cap = 0;
  uint64_t nliving = 0;     // cached count of living agents
  // staging before finish_init!
  std::vector<std::vector<uint8_t>> h_fields;
  uint64_t h_n = 0;
  bool readable = false, writeable = false;
};

// Persistent scratch of the typed rebuild (the per-step edge rebuild from
// records whose types the emitting kernel declares) and a CUDA graph of its
// launch sequence: recorded when the same arguments (sizes and buffers)
// repeat on consecutive rebuilds, replayed while they stay the same.
struct RebuildCache {
  DevBuf keys, sort, bstart;
  std::vector<uint64_t> last, graph_args;
  cudaGraphExec_t exec = nullptr;
  RebuildCache() = default;
  RebuildCache(const RebuildCache &) = delete;
  RebuildCache &operator=(const RebuildCache &) = delete;
  ~RebuildCache() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

struct CSR {
  uint64_t nrows = 0, nedges = 0;
  std::unique_ptr<RebuildCache> rebuild;
  DevBuf row_ptr;  // u32[nrows + 1]
  DevBuf src;      // u32[nedges] source agent_nr - 1
  DevBuf src_type; // u8[nedges] when src_type_const < 0
  int src_type_const = 0;  // >0 all sources of that type, 0 none, -1 mixed
  std::vector<DevBuf> payload;
  uint32_t max_degree = 0;  // read through csr_max_degree()
  DevBuf d_max_degree;      // device value while max_degree_pending
  bool max_degree_pending = false;
  // derived gather layout of the Float64 payload column 0 (built on first
  // use by the gather kernels, cached until the CSR changes):
  // hub rows (degree > hub threshold) by descending degree; the other rows
  // (agents beyond the CSR's rows included) in `order`, by descending
  // degree inside windows of 2^13 consecutive rows, cut into slices of 32;
  // the edges of a slice stored column-major (SELL-C-sigma): edge k of the
  // slice's lane l at slice_base + 32 k + l, padded to the slice's largest
  // degree (padding: source 0, weight 0)
  DevBuf hub_rows;  // u32
  uint64_t nhub = 0;
  // the first nbig hub rows have more than block_threshold in-edges: one
  // block each, staged through shared memory by bulk copies
  uint64_t nbig = 0;
  uint32_t block_threshold = 0xFFFFFFFFu;
  DevBuf order;     // u32 rows, position = 32 slice + lane
  DevBuf order_deg; // u32 in-degree of the row at each position of `order`
  uint64_t norder = 0;
  DevBuf slice_base;  // u64 [nslices + 1]: first column-major slot of each slice
  DevBuf slice_deg;   // u32 [nslices]: the slice's largest degree
  uint64_t nslices = 0;
  DevBuf sell_src;  // u32 [slots]
  DevBuf sell_w;    // f64 [slots]
  uint64_t sched_n = 0;  // agent count the layout covers
  uint32_t hub_threshold = 0;
  uint32_t wshift = 13;   // window = row >> wshift
  bool schedule_valid = false;
  // row ranges of the gather whose completion the launch reports (apply!
  // with host exchange): range k is the slice blocks before range_block[k]
  // (from the previous boundary) and holds the non-hub rows below
  // range_rows[k]; derived from the layout, cached with it
  std::vector<uint64_t> range_block, range_rows;
  std::vector<uint32_t> range_window;  // window of each range's first row
  std::vector<uint32_t> hub_rows_sorted;  // host copy of the hub rows, ascending
  // payload field 0 (Float64) holds only multiples of 2^-53 in (0, 1]:
  // -1 not checked yet, 0 no, 1 yes (decides the gather kernels' sum path)
  int unit_grid_weights = -1;
};

struct StencilDesc {
  int raster = -1;         // index into Sim::rasters
  int ndims = 0;
  int64_t dims[MAX_DIMS] = {0, 0, 0, 0};
  int noff = 0;
  std::vector<int> offsets;  // noff * ndims, in the reference's order
  int periodic = 1;
  int target_type = 0;
  std::vector<uint8_t> payload;  // constant payload of every stencil edge
};

// A contiguous run of staged edges (before finish_init!, or added between
// transitions with the checks disabled).  Either host or device resident.
struct EdgeSegment {
  bool device = false;
  uint64_t n = 0;
  std::vector<uint64_t> h_from, h_to;
  std::vector<std::vector<uint8_t>> h_payload;
  DevBuf d_from, d_to;
  std::vector<DevBuf> d_payload;
};

struct EdgeStore {
  std::vector<CSR> csr;  // index = target type number (0 unused)
  bool implicit = false;
  StencilDesc st;
  std::vector<EdgeSegment> staged;  // pending adds in call order
  uint64_t nstaged = 0;
  // single-edge bookkeeping of staged host adds (target -> slot)
  std::map<uint64_t, uint64_t> single_seen;
  bool readable = false, writeable = false, add_existing = false;
};

struct Raster {
  std::string name;
  int ndims = 0;
  int64_t dims[MAX_DIMS] = {0, 0, 0, 0};
  int type_nr = 0;
  uint64_t first_nr = 0;  // agent_nr of the cell at linear index 0
  uint64_t ncells = 0;
};

struct EdgeAppend;

// stencil(metric, n, distance) -- src/Raster.jl:82-110: offsets in the
// reference's order, n per entry (vg_api.cu)
std::vector<int> make_stencil(int metric, int n, double distance);

struct Sim {
  std::shared_ptr<Model> model;
  std::string name;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool initialized = false;
  bool intransition = false;
  bool check_readable = true;
  int64_t num_transitions = 0;
  // Incremented whenever work that writes an edge container (CSR) is
  // enqueued.  A SIR step launched with programmatic dependent launch reads
  // its contact rows before waiting for the preceding kernel; it does so
  // only while no CSR write was enqueued since the previous SIR step
  // (sir_epoch: csr_epoch at that step), so the preceding kernel cannot be
  // writing them.
  uint64_t csr_epoch = 1, sir_epoch = 0;
  uint64_t footprint = 0;
  std::vector<AgentStore> agents;  // index = nr - 1
  std::vector<EdgeStore> edges;    // index = edge type index
  std::vector<Raster> rasters;
  std::map<std::string, double> params, globals;
  std::map<std::string, std::vector<double>> global_series;
  // scratch
  DevBuf d_status;  // int32 device error word
  DevBuf d_scratch;
  size_t scratch_bytes = 0;
  void *scratch(size_t bytes);
  // constant tables of the transitions (e.g. infection probabilities per
  // infected-neighbour count), uploaded once per distinct content; the key
  // names the table, the bytes decide whether the copy is current
  struct ConstTable {
    DevBuf dev;
    std::vector<uint8_t> host;
  };
  std::map<std::string, ConstTable> const_tables;
  const void *const_table(const std::string &key, const void *host, size_t bytes);
  int raster_index(const std::string &n) const;
  // stream and status word are created on first device use, so that the
  // init phase (registry, staging) runs without a GPU
  bool device_ready = false;
  void ensure_device();
  // asynchronous mode: apply! does not wait for the device; the kernels'
  // status word is checked at the next synchronizing call
  bool async = false;
  // edge-append buffers of earlier transitions, by edge type, reused by the
  // next apply! that appends to the same type (no allocation per step)
  std::map<int, std::unique_ptr<EdgeAppend>> append_spare;
  // apply! with host exchange (vg_apply_host): while set, a transition that
  // finishes its rows range by range may download each finished range of the
  // called type's new state to `out` on copy_stream while it runs (and sets
  // `done`)
  struct HostExchange {
    int type_nr = 0;
    void *const *out = nullptr;
    uint64_t n = 0;
    bool done = false;
  };
  HostExchange *host_xchg = nullptr;
  // parameter slots of a transition bound to a param (kind 0) or global
  // (kind 1) of this simulation: every apply! of the transition passes the
  // current value in that slot (param / get_global read inside the
  // transition, src/Simulation.jl:587, src/Global.jl:10)
  struct ParamBinding {
    int slot, kind;
    std::string name;
  };
  std::map<std::string, std::vector<ParamBinding>> bindings;
  cudaStream_t copy_stream = nullptr;  // created on first use, destroyed with the sim
  // completion reports of a gather launch: per-range block counters on the
  // device, per-range flags in mapped pinned host memory (the last block of
  // a range writes the call's generation), created on first use
  DevBuf xchg_count;
  unsigned *xchg_flags_host = nullptr, *xchg_flags_dev = nullptr;
  unsigned xchg_gen = 0;
  ~Sim();
};

// ---------------------------------------------------------------- kernels
// Views passed to kernels by value.
struct DevAgentView {
  uint64_t n;
  void *rd[MAX_FIELDS];
  void *wr[MAX_FIELDS];
  uint8_t *died_rd;
  uint8_t *died_wr;
};
struct DevCSRView {
  uint64_t nrows, nedges;
  const uint32_t *row_ptr;
  const uint32_t *src;
  const uint8_t *src_type;
  int src_type_const;
  const void *payload[MAX_FIELDS];
};

DevAgentView agent_view(Sim &s, int type_nr);
DevCSRView csr_view(Sim &s, int edge_type, int target_type_nr);

struct EdgeAppend {
  int edge_type = -1;
  uint64_t cap = 0;
  DevBuf to, from, key;  // u64 target id, u64 source id, u64 order key
  std::vector<DevBuf> payload;
  DevBuf counter;  // u64 device counter
  bool ordered = false;  // records already in order-key order
  uint64_t fixed_count = 0;  // when the count is known on the host
  // declared by kernels whose records are typed by construction: every
  // target of agent type target_type, every source of type src_type
  // (0: unknown) -- allows the typed fast rebuild (build_csr_typed)
  int target_type = 0, src_type = 0;
};

// remove_edges! calls recorded by a transition (src/EdgeMethods.jl:527-599):
// (to, from, key); from = REMOVE_ALL for remove_edges!(sim, to, T).  At the
// end of apply! a record of the written container (old edges kept by
// add_existing: key 0; appended edges: order key + 1) is dropped when a
// removal of its target (all sources, or its source) carries a larger key,
// i.e. was called after the edge was added in the sequential sweep.
constexpr uint64_t REMOVE_ALL = ~0ull;
struct EdgeRemoval {
  int edge_type = -1;
  uint64_t cap = 0;
  DevBuf to, from, key;
  DevBuf counter;  // u64 device counter
};
void apply_edge_removals(Sim &s, int edge_type, EdgeRemoval &rm, EdgeAppend *ap,
                         uint64_t &n_records, bool merge_existing);

// Apply context handed to a transition launcher.
struct ApplyCtx {
  Sim *sim;
  int call_type;  // agent type number being swept
  int call_pos;   // position in `call`
  std::vector<int> read, write, add_existing;
  int with_edge;
  const double *params;
  int nparams;
  int64_t step;  // num_transitions at the start of apply!
  bool in_read(int ref) const;
  bool in_write(int ref) const;
  bool writes_call() const;
  double param(int i, double dflt) const {
    return i < nparams ? params[i] : dflt;
  }
  // edge records appended by the launchers, per written edge type
  std::vector<std::unique_ptr<EdgeAppend>> appends;
  EdgeAppend *append_for(int edge_type, uint64_t capacity, bool ordered);
  std::vector<std::unique_ptr<EdgeRemoval>> removals;
  EdgeRemoval *removal_for(int edge_type, uint64_t capacity);
};


typedef void (*TransitionLauncher)(ApplyCtx &ctx);
struct TransitionDef {
  const char *name;
  TransitionLauncher launch;
};
const std::vector<TransitionDef> &transitions();
// launchers that live in their own translation units
void tr_bounded_confidence(ApplyCtx &ctx);  // vg_opinion.cu

// one bounded-confidence launch over many simulations (vg_opinion.cu)
// default hub threshold of the bounded-confidence gather: rows above it are
// split across a warp (1e-12 relative), rows at or below it fold in order
// (bit-exact); 1536 measured fastest on the benchmark graph
constexpr uint32_t OPINION_HUB_DEFAULT = 1536;

struct OpinionJob {
  Sim *sim;
  int edge_type, type_nr;
  double eps, a, b;
  uint32_t hub_thr;
  uint32_t block_thr = 0xFFFFFFFFu;
};
void launch_opinion_jobs(const std::vector<OpinionJob> &jobs, cudaStream_t st, DevBuf &args_buf,
                         DevBuf &tiles_buf, uint64_t *footprint);
void prepare_opinion_job(const OpinionJob &job);
// initial SIR state: the n_inf agents with the smallest Philox init draw
void sir_initial_state(uint64_t n, uint64_t seed, uint64_t n_inf, std::vector<uint8_t> &state);

// primitives (vg_sort.cu)
void exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n,
                        cudaStream_t st, Sim &s);
void exclusive_scan_u64(const uint64_t *in, uint64_t *out, uint64_t n,
                        cudaStream_t st, Sim &s);
// stable LSD radix sort of (key, value) pairs over key bits [0, bits)
void radix_sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint64_t n,
                          int bits, cudaStream_t st, Sim &s);
void radix_sort_pairs_u64(uint64_t *keys, uint32_t *vals, uint64_t n,
                          int bits, cudaStream_t st, Sim &s);
// caller-owned scratch of exclusive_scan_scratch_bytes(n) bytes: no allocation
uint64_t exclusive_scan_scratch_bytes(uint64_t n);
void exclusive_scan_u32_in(const uint32_t *in, uint32_t *out, uint64_t n, cudaStream_t st,
                           int *err, void *scratch);
// caller-owned scratch of radix_sort_scratch_bytes() bytes: no allocation
uint64_t radix_sort_scratch_bytes(uint64_t n, int key_size, int bits);
// counted: the caller has accumulated the digit counts of every pass (8-bit
// digit p of each key, at word 256 p + digit) into radix_sort_digit_counts
// of the same scratch, zeroed before; the sort then skips its own count
void radix_sort_pairs_u32_in(uint32_t *keys, uint32_t *vals, uint64_t n, int bits,
                             cudaStream_t st, int *err, void *scratch, bool counted = false);
uint32_t *radix_sort_digit_counts(void *scratch);
int bits_for(uint64_t maxval);

// graph building (vg_graph.cu)
void build_csr_from_records(Sim &s, int edge_type, const uint64_t *d_from,
                            const uint64_t *d_to,
                            const std::vector<const void *> &d_payload,
                            uint64_t n, bool records_sorted_by_key,
                            const uint64_t *d_key, bool merge_existing);
void remove_died_edges(Sim &s, int died_type, const uint8_t *died_now,
                       uint64_t n_died);
// hub list and degree-sorted row order over n agent slots (n >= nrows)
// block_threshold: hub rows above it take a whole block (UINT32_MAX: none)
void ensure_schedule(Sim &s, CSR &c, uint32_t hub_threshold, uint32_t block_threshold,
                     uint64_t n);
// largest row length (synchronises when the value is still on the device)
uint32_t csr_max_degree(Sim &s, CSR &c);
// rebuild of an edge type's container from typed, ordered records without
// host synchronisation; false when the generic build must run
bool build_csr_typed(Sim &s, int edge_type, const EdgeAppend &ap, uint64_t n);
uint64_t csr_edges_total(const EdgeStore &es);

// agents (vg_api.cu)
void agent_reserve(Sim &s, int type_nr, uint64_t slots);
void apply_finish_agents(Sim &s, int type_nr, bool swapped);

// misc
void check_device_status(Sim &s, const char *what);

}  // namespace vg

struct vg_model {
  std::shared_ptr<vg::Model> m;
};
struct vg_sim {
  std::unique_ptr<vg::Sim> s;
};
