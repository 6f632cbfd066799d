// apply! (src/Simulation.jl:720-821) and mapreduce
// (src/AgentMethods.jl:533-565, src/EdgeMethods.jl:972-1001).
//
// apply! runs, in the reference's order: the argument checks, prepare_read!
// (readable flags), prepare_write! (reset of written agent types that are
// neither called nor in add_existing; new or kept edge containers), the
// sweep of every called type by the named kernel, then finish_write! of the
// agent types (swap of the double buffers, collection of the agents that
// died into the reuse stack, removal of their edges) and of the edge types
// (the new CSR replaces the read container).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

#include "vg_internal.h"

namespace vg {

bool ApplyCtx::in_read(int ref) const {
  return std::find(read.begin(), read.end(), ref) != read.end();
}
bool ApplyCtx::in_write(int ref) const {
  return std::find(write.begin(), write.end(), ref) != write.end();
}
bool ApplyCtx::writes_call() const { return in_write(call_type); }

EdgeAppend *ApplyCtx::append_for(int e, uint64_t capacity, bool ordered) {
  for (auto &a : appends)
    if (a->edge_type == e) {
      if (a->ordered != ordered || ordered)
        fail(VG_ERR_ARG, "one transition call appends to an edge type once");
      return a.get();
    }
  Sim &s = *sim;
  const EdgeTypeDesc &ed = s.model->et(e);
  auto it = s.append_spare.find(e);
  if (it != s.append_spare.end() && it->second->cap >= capacity &&
      it->second->ordered == ordered) {
    std::unique_ptr<EdgeAppend> a = std::move(it->second);
    s.append_spare.erase(it);
    a->fixed_count = 0;
    a->target_type = a->src_type = 0;
    VG_CUDA(cudaMemsetAsync(a->counter.p, 0, 8, s.stream));
    appends.push_back(std::move(a));
    return appends.back().get();
  }
  auto a = std::make_unique<EdgeAppend>();
  a->edge_type = e;
  a->cap = std::max<uint64_t>(capacity, 1);
  a->ordered = ordered;
  a->to.alloc(a->cap * 8, &s.footprint);
  a->from.alloc(a->cap * 8, &s.footprint);
  if (!ordered) a->key.alloc(a->cap * 8, &s.footprint);
  int nf = ed.stores_payload() ? (int)ed.fields.size() : 0;
  a->payload.resize(nf);
  for (int f = 0; f < nf; f++) a->payload[f].alloc(a->cap * ed.fields[f].size, &s.footprint);
  a->counter.alloc(8, &s.footprint);
  VG_CUDA(cudaMemsetAsync(a->counter.p, 0, 8, s.stream));
  appends.push_back(std::move(a));
  return appends.back().get();
}

EdgeRemoval *ApplyCtx::removal_for(int e, uint64_t capacity) {
  for (auto &r : removals)
    if (r->edge_type == e) {
      if (r->cap < capacity) fail(VG_ERR_ARG, "removal buffer sized by the first call type");
      return r.get();
    }
  Sim &s = *sim;
  auto r = std::make_unique<EdgeRemoval>();
  r->edge_type = e;
  r->cap = std::max<uint64_t>(capacity, 1);
  r->to.alloc(r->cap * 8, &s.footprint);
  r->from.alloc(r->cap * 8, &s.footprint);
  r->key.alloc(r->cap * 8, &s.footprint);
  r->counter.alloc(8, &s.footprint);
  VG_CUDA(cudaMemsetAsync(r->counter.p, 0, 8, s.stream));
  removals.push_back(std::move(r));
  return removals.back().get();
}

namespace {

constexpr int TPB = 256;
inline unsigned nblk(uint64_t n, int tpb = TPB) {
  uint64_t b = (n + tpb - 1) / tpb;
  return (unsigned)std::max<uint64_t>(b, 1);
}

__global__ void k_new_deaths(const uint8_t *died_new, const uint8_t *died_old,
                             uint64_t n, uint32_t *flag) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (died_new[i] && !died_old[i]) ? 1u : 0u;
}

__global__ void k_push_reuse(const uint32_t *flag, const uint32_t *pos, uint64_t n,
                             uint64_t *stack, uint64_t base) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) stack[base + pos[i]] = i + 1;  // agent numbers, in index order
}

bool is_edge_ref(int r) { return (r & 0x10000) != 0; }
int edge_of(int r) { return r & 0xFFFF; }

std::string ref_name(Sim &s, int r) {
  return is_edge_ref(r) ? s.model->et(edge_of(r)).name : s.model->at(r).name;
}

void validate_refs(Sim &s, const int *v, int n) {
  for (int i = 0; i < n; i++) {
    if (is_edge_ref(v[i])) s.model->et(edge_of(v[i]));
    else s.model->at(v[i]);
  }
}

// ------------------------------------------------------------- mapreduce
// val4empty (src/Helpers.jl:44-81): identity of op for datatype MT; MT is
// Bool for & and | and Int64 otherwise unless `datatype` says else.
struct RedAcc {
  int64_t i;
  double f;
};

__device__ __forceinline__ int64_t red_i(int op, int64_t a, int64_t b) {
  switch (op) {
    case VG_OP_ADD: return (int64_t)((uint64_t)a + (uint64_t)b);
    case VG_OP_MUL: return (int64_t)((uint64_t)a * (uint64_t)b);
    case VG_OP_MAX: return a > b ? a : b;
    case VG_OP_MIN: return a < b ? a : b;
    case VG_OP_AND: return a & b;
    case VG_OP_OR: return a | b;
  }
  return 0;
}
// Julia's max/min of two floats: a NaN operand gives NaN, +0.0 is larger
// than -0.0 (the difference's sign decides); order-independent, so the
// tree and the sequential fold agree
__device__ __forceinline__ double jl_max(double x, double y) {
  const double d = __dsub_rn(x, y);
  const double m = signbit(d) ? y : x;
  return (isnan(x) || isnan(y)) ? d : m;
}
__device__ __forceinline__ double jl_min(double x, double y) {
  const double d = __dsub_rn(x, y);
  const double m = signbit(d) ? x : y;
  return (isnan(x) || isnan(y)) ? d : m;
}
__device__ __forceinline__ double red_f(int op, double a, double b) {
  switch (op) {
    case VG_OP_ADD: return __dadd_rn(a, b);
    case VG_OP_MUL: return __dmul_rn(a, b);
    case VG_OP_MAX: return jl_max(a, b);
    case VG_OP_MIN: return jl_min(a, b);
  }
  return 0;
}

__device__ __forceinline__ double load_val(const void *p, int dt, uint64_t i, bool *isf,
                                           int64_t *iv) {
  switch (dt) {
    case VG_BOOL: case VG_U8: *iv = ((const uint8_t *)p)[i]; break;
    case VG_I8: *iv = ((const int8_t *)p)[i]; break;
    case VG_U16: *iv = ((const uint16_t *)p)[i]; break;
    case VG_I16: *iv = ((const int16_t *)p)[i]; break;
    case VG_U32: *iv = ((const uint32_t *)p)[i]; break;
    case VG_I32: *iv = ((const int32_t *)p)[i]; break;
    case VG_U64: case VG_I64: *iv = ((const int64_t *)p)[i]; break;
    case VG_F32: *isf = true; return ((const float *)p)[i];
    case VG_F64: *isf = true; return ((const double *)p)[i];
  }
  *isf = false;
  return (double)*iv;
}

// map f: field, or field compared with a constant (result Bool)
__device__ __forceinline__ void map_val(int kind, double arg, const void *p, int dt, uint64_t i,
                                        bool float_acc, int64_t *vi, double *vf) {
  bool isf = false;
  int64_t iv = 0;
  double fv = load_val(p, dt, i, &isf, &iv);
  if (kind != VG_MAP_FIELD) {
    bool r = false;
    double x = isf ? fv : (double)iv;
    switch (kind) {
      case VG_MAP_EQ: r = x == arg; break;
      case VG_MAP_NE: r = x != arg; break;
      case VG_MAP_LT: r = x < arg; break;
      case VG_MAP_GT: r = x > arg; break;
    }
    *vi = r;
    *vf = r;
    return;
  }
  *vi = isf ? (int64_t)fv : iv;
  *vf = isf ? fv : (double)iv;
  (void)float_acc;
}

struct RedArgs {
  const void *p;
  int dt;
  uint64_t n;
  const uint8_t *died;  // agents: skip died; null for edges
  int kind;
  double arg;
  int op;
  int float_acc;
  int64_t init_i;   // the reduction's init (val4empty or the `init` keyword)
  double init_f;
  int64_t neut_i;   // neutral element of op for the partial reductions
  double neut_f;
};

// pass 1: per-block partial (deterministic block order): each thread folds
// its strided elements, each warp combines its 32 lanes by shuffles in a
// fixed tree, warp 0 combines the warps' results the same way
__device__ __forceinline__ void warp_combine(int op, int64_t &vi, double &vf) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const int64_t oi = __shfl_down_sync(0xffffffffu, vi, off);
    const double of = __shfl_down_sync(0xffffffffu, vf, off);
    vi = red_i(op, oi, vi);
    vf = red_f(op, of, vf);
  }
}

__global__ void k_reduce_partial(RedArgs a, int64_t *pi, double *pf) {
  __shared__ int64_t si[TPB / 32];
  __shared__ double sf[TPB / 32];
  int64_t acc_i = a.neut_i;
  double acc_f = a.neut_f;
  bool have = false;
  uint64_t chunk = (a.n + gridDim.x - 1) / gridDim.x;
  uint64_t b = (uint64_t)blockIdx.x * chunk, e = min(a.n, b + chunk);
  for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    if (a.died && a.died[i]) continue;
    int64_t vi;
    double vf;
    map_val(a.kind, a.arg, a.p, a.dt, i, a.float_acc, &vi, &vf);
    if (!have) {
      acc_i = vi;
      acc_f = vf;
      have = true;
    } else {
      acc_i = red_i(a.op, vi, acc_i);
      acc_f = red_f(a.op, vf, acc_f);
    }
  }
  // empty threads contribute the neutral element
  if (!have) {
    acc_i = a.neut_i;
    acc_f = a.neut_f;
  }
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  warp_combine(a.op, acc_i, acc_f);
  if (lane == 0) {
    si[wid] = acc_i;
    sf[wid] = acc_f;
  }
  __syncthreads();
  if (wid == 0) {
    acc_i = lane < TPB / 32 ? si[lane] : a.neut_i;
    acc_f = lane < TPB / 32 ? sf[lane] : a.neut_f;
    warp_combine(a.op, acc_i, acc_f);
    if (lane == 0) {
      pi[blockIdx.x] = acc_i;
      pf[blockIdx.x] = acc_f;
    }
  }
}

__global__ void k_reduce_final(const int64_t *pi, const double *pf, int nb, int op,
                               int64_t init_i, double init_f, int64_t *oi, double *of) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t ai = init_i;
  double af = init_f;
  for (int b = 0; b < nb; b++) {
    ai = red_i(op, pi[b], ai);
    af = red_f(op, pf[b], af);
  }
  *oi = ai;
  *of = af;
}

// Sequential left fold in index order, reduced = op(f(x), reduced), the
// reference's loop: one chain of dependent operations on thread 0.  The
// block's other warps map the next tile of elements into shared memory
// (value bits and whether the element counts) while thread 0 folds the
// current tile, so the chain never waits for global memory.
constexpr int ORD_TILE = 2048;
constexpr int ORD_TPB = 256;

__global__ void __launch_bounds__(ORD_TPB) k_reduce_ordered(RedArgs a, int64_t *oi, double *of) {
  __shared__ int64_t vbuf[2][ORD_TILE];
  __shared__ uint8_t live[2][ORD_TILE];
  const uint64_t ntiles = (a.n + ORD_TILE - 1) / ORD_TILE;
  auto stage = [&](uint64_t t, int b) {  // warps 1.. map tile t into buffer b
    const uint64_t base = t * ORD_TILE;
    for (uint32_t k = threadIdx.x - 32; k < (uint32_t)ORD_TILE; k += blockDim.x - 32) {
      const uint64_t i = base + k;
      const bool use = i < a.n && !(a.died && a.died[i]);
      int64_t vi = 0;
      double vf = 0.0;
      if (use) map_val(a.kind, a.arg, a.p, a.dt, i, a.float_acc, &vi, &vf);
      vbuf[b][k] = a.float_acc ? __double_as_longlong(vf) : vi;
      live[b][k] = use;
    }
  };
  if (ntiles && threadIdx.x >= 32) stage(0, 0);
  __syncthreads();
  int64_t ai = a.init_i;
  double af = a.init_f;
  for (uint64_t t = 0; t < ntiles; t++) {
    const int b = (int)(t & 1);
    if (threadIdx.x >= 32) {
      if (t + 1 < ntiles) stage(t + 1, b ^ 1);
    } else if (threadIdx.x == 0) {
      const uint32_t m = (uint32_t)min((uint64_t)ORD_TILE, a.n - t * ORD_TILE);
      if (a.float_acc && a.op == VG_OP_ADD) {
        for (uint32_t k = 0; k < m; k++)
          if (live[b][k]) af = __dadd_rn(__longlong_as_double(vbuf[b][k]), af);
      } else if (a.float_acc) {
        for (uint32_t k = 0; k < m; k++)
          if (live[b][k]) af = red_f(a.op, __longlong_as_double(vbuf[b][k]), af);
      } else {
        for (uint32_t k = 0; k < m; k++)
          if (live[b][k]) ai = red_i(a.op, vbuf[b][k], ai);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *oi = ai;
    *of = af;
  }
}

void identity_for(int op, int out_dtype, int has_init, double init, int64_t *ii,
                  double *fi) {
  if (has_init) {
    *ii = (int64_t)init;
    *fi = init;
    return;
  }
  bool boolean = out_dtype == VG_BOOL;
  switch (op) {
    case VG_OP_ADD: *ii = 0; *fi = 0; break;
    case VG_OP_MUL: *ii = 1; *fi = 1; break;
    case VG_OP_MAX:
      *ii = boolean ? -1 : -std::numeric_limits<int64_t>::max();
      *fi = (double)*ii;
      break;
    case VG_OP_MIN:
      *ii = boolean ? 1 : std::numeric_limits<int64_t>::max();
      *fi = (double)*ii;
      break;
    case VG_OP_AND:
      *ii = boolean ? 1 : std::numeric_limits<int64_t>::max();
      *fi = (double)*ii;
      break;
    case VG_OP_OR: *ii = 0; *fi = 0; break;
    default: fail(VG_ERR_ASSERT, "Can not derive the init value for the operator. You must "
                                 "add this information via the `init` keyword.");
  }
}

void neutral_for(int op, int64_t *ni, double *nf) {
  switch (op) {
    case VG_OP_ADD: *ni = 0; *nf = 0.0; break;
    case VG_OP_MUL: *ni = 1; *nf = 1.0; break;
    case VG_OP_MAX: *ni = std::numeric_limits<int64_t>::min(); *nf = -INFINITY; break;
    case VG_OP_MIN: *ni = std::numeric_limits<int64_t>::max(); *nf = INFINITY; break;
    case VG_OP_AND: *ni = -1; *nf = 0.0; break;
    default: *ni = 0; *nf = 0.0;
  }
}

// The reference folds sequentially (reduced = op(f(x), reduced)).  Integer
// and Bool results, and Float max/min, do not depend on the order, so they
// take the two-pass tree; Float + and * fold in order unless the caller
// asks for the tree (VG_REDUCE_TREE), whose result may differ in the last
// bits.
double host_jl_max(double x, double y) {
  const double d = x - y;
  return (std::isnan(x) || std::isnan(y)) ? d : (std::signbit(d) ? y : x);
}
double host_jl_min(double x, double y) {
  const double d = x - y;
  return (std::isnan(x) || std::isnan(y)) ? d : (std::signbit(d) ? x : y);
}

bool fold_in_order(int flags, bool float_acc, int op) {
  if (flags & VG_REDUCE_ORDERED) return true;
  if (flags & VG_REDUCE_TREE) return false;
  return float_acc && (op == VG_OP_ADD || op == VG_OP_MUL);
}

void run_reduce(Sim &s, RedArgs a, int out_dtype, bool ordered, void *out) {
  neutral_for(a.op, &a.neut_i, &a.neut_f);
  int64_t ri = a.init_i;
  double rf = a.init_f;
  if (a.n > 0) {
    int64_t *d = nullptr;
    VG_CUDA(cudaMallocAsync((void **)&d, 16 + 2 * 8 * 1024, s.stream));
    int64_t *oi = d;
    double *of = (double *)(d + 1);
    if (ordered) {
      k_reduce_ordered<<<1, ORD_TPB, 0, s.stream>>>(a, oi, of);
    } else {
      int nb = (int)std::min<uint64_t>(1024, (a.n + TPB - 1) / TPB);
      int64_t *pi = d + 2;
      double *pf = (double *)(d + 2 + 1024);
      k_reduce_partial<<<nb, TPB, 0, s.stream>>>(a, pi, pf);
      k_reduce_final<<<1, 32, 0, s.stream>>>(pi, pf, nb, a.op, a.init_i, a.init_f, oi, of);
    }
    VG_CUDA(cudaGetLastError());
    VG_CUDA(cudaMemcpyAsync(&ri, oi, 8, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaMemcpyAsync(&rf, of, 8, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaFreeAsync(d, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
  }
  if (out_dtype == VG_F64) *(double *)out = a.float_acc ? rf : (double)ri;
  else if (out_dtype == VG_BOOL) *(uint8_t *)out = (a.float_acc ? rf : (double)ri) != 0;
  else *(int64_t *)out = a.float_acc ? (int64_t)rf : ri;
}

}  // namespace
}  // namespace vg

using namespace vg;

#define API_BEGIN try {
#define API_END                       \
  return VG_OK;                       \
  }                                   \
  catch (const Error &e) {            \
    set_last_error(e.msg);            \
    return e.code;                    \
  }                                   \
  catch (const std::exception &e) {   \
    set_last_error(e.what());         \
    return VG_ERR_ARG;                \
  }

namespace vg {
void set_last_error(const std::string &m);
}

static Sim &S(vg_sim *s) {
  if (!s || !s->s) fail(VG_ERR_ARG, "null simulation handle");
  return *s->s;
}

extern "C" {

const char *vg_transition_names(void) {
  static std::string names;
  if (names.empty())
    for (auto &t : transitions()) {
      if (!names.empty()) names += ",";
      names += t.name;
    }
  return names.c_str();
}

int vg_apply(vg_sim *h, const char *tname, const int *call, int ncall, const int *read,
             int nread, const int *write, int nwrite, const int *ae, int nae, int with_edge,
             const double *params, int nparams) {
  API_BEGIN
  Sim &s = S(h);
  if (!s.initialized) fail(VG_ERR_ASSERT, "You must call finish_init! before apply!");
  const TransitionDef *def = nullptr;
  for (auto &t : transitions())
    if (std::strcmp(t.name, tname) == 0) def = &t;
  if (!def) fail(VG_ERR_ARG, std::string("unknown transition ") + tname);
  validate_refs(s, call, ncall);
  validate_refs(s, read, nread);
  validate_refs(s, write, nwrite);
  validate_refs(s, ae, nae);
  if (with_edge >= 0 && s.model->et(with_edge).singletype())
    fail(VG_ERR_ASSERT, "The `with_edge` keyword can only be used for edgetypes without the "
                        ":SingleType hint.");
  ApplyCtx ctx;
  ctx.sim = &s;
  ctx.read.assign(read, read + nread);
  ctx.write.assign(write, write + nwrite);
  ctx.add_existing.assign(ae, ae + nae);
  ctx.with_edge = with_edge;
  ctx.params = params;
  ctx.nparams = nparams;
  // slots bound to a param or global take its current value
  std::vector<double> bound;
  auto bit = s.bindings.find(tname);
  if (bit != s.bindings.end() && !bit->second.empty()) {
    bound.assign(params, params + std::max(nparams, 0));
    for (auto &b : bit->second) {
      if (b.slot >= (int)bound.size())
        fail(VG_ERR_ARG, "parameter slot " + std::to_string(b.slot) + " of " + tname +
                             " is bound to " + b.name + " but apply! passes " +
                             std::to_string(nparams) + " parameters");
      const auto &m = b.kind == 0 ? s.params : s.globals;
      auto it = m.find(b.name);
      if (it == m.end()) fail(VG_ERR_ARG, "unknown " + std::string(b.kind ? "global " : "param ") + b.name);
      bound[b.slot] = it->second;
    }
    ctx.params = bound.data();
  }
  ctx.step = s.num_transitions;
  auto in = [](const std::vector<int> &v, int r) {
    return std::find(v.begin(), v.end(), r) != v.end();
  };
  std::vector<int> C(call, call + ncall);
  for (int c : C) {
    if (is_edge_ref(c)) fail(VG_ERR_ARG, "call holds agent types only");
    if (in(ctx.add_existing, c))
      fail(VG_ERR_ASSERT, ref_name(s, c) + " can not be element of `add_existing`");
  }
  for (int a : ctx.add_existing)
    if (!in(ctx.write, a))
      fail(VG_ERR_ASSERT, ref_name(s, a) + " is in `add_existing` but not in `write`");

  struct Flags {
    Sim &s;
    ~Flags() {
      s.intransition = false;
      for (auto &a : s.agents) a.readable = a.writeable = false;
      for (auto &e : s.edges) e.readable = e.writeable = e.add_existing = false;
    }
  } flags{s};
  s.intransition = true;
  for (int r : ctx.read) {
    if (is_edge_ref(r)) s.edges[edge_of(r)].readable = true;
    else s.agents[r - 1].readable = true;
  }
  // prepare_write! (src/AgentMethods.jl:271-298, src/EdgeMethods.jl:639-663)
  for (int w : ctx.write) {
    if (is_edge_ref(w)) {
      EdgeStore &es = s.edges[edge_of(w)];
      if (es.implicit) fail(VG_ERR_ARG, "implicit raster edges are not written by transitions");
      es.writeable = true;
      es.add_existing = in(ctx.add_existing, w);
      continue;
    }
    const AgentTypeDesc &ad = s.model->at(w);
    bool aex = in(C, w) || in(ctx.add_existing, w);
    if (ad.immortal() && !aex)
      fail(VG_ERR_ASSERT, "You can add " + ad.name + " to the `write` argument only when " +
                              ad.name + " is also included in the `add_existing` argument, as " +
                              ad.name + " has the hint :Immortal.");
    AgentStore &a = s.agents[w - 1];
    if (!aex) {
      a.n = 0;
      a.nreuse = 0;
      a.nliving = 0;
    }
    a.writeable = true;
  }
  // the sweep
  for (int pos = 0; pos < (int)C.size(); pos++) {
    ctx.call_type = C[pos];
    ctx.call_pos = pos;
    def->launch(ctx);
  }
  if (!s.async) check_device_status(s, tname);

  // finish_write! of the agent types (src/AgentMethods.jl:300-439)
  std::vector<int> died_types;
  for (int T : C) {
    if (!in(ctx.write, T)) continue;
    AgentStore &a = s.agents[T - 1];
    const AgentTypeDesc &ad = s.model->at(T);
    std::swap(a.rd, a.wr);
    if (ad.immortal() || a.n == 0) continue;
    std::swap(a.died_rd, a.died_wr);
    // agents that died in this transition, in index order (writereuseable)
    uint32_t *flag = nullptr, *pos = nullptr;
    VG_CUDA(cudaMallocAsync((void **)&flag, (a.n + 1) * 4, s.stream));
    VG_CUDA(cudaMallocAsync((void **)&pos, (a.n + 1) * 4, s.stream));
    k_new_deaths<<<nblk(a.n), TPB, 0, s.stream>>>(a.died_rd.as<uint8_t>(),
                                                   a.died_wr.as<uint8_t>(), a.n, flag);
    VG_CUDA(cudaMemsetAsync(flag + a.n, 0, 4, s.stream));
    exclusive_scan_u32(flag, pos, a.n + 1, s.stream, s);
    uint32_t k = 0;
    VG_CUDA(cudaMemcpyAsync(&k, pos + a.n, 4, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    if (k) {
      if (a.nreuse + k > a.reuse_cap) {
        uint64_t nc = std::max<uint64_t>(a.nreuse + k, 2 * a.reuse_cap);
        DevBuf nb;
        nb.alloc(nc * 8, &s.footprint);
        if (a.nreuse)
          VG_CUDA(cudaMemcpyAsync(nb.p, a.reuse.p, a.nreuse * 8, cudaMemcpyDeviceToDevice, s.stream));
        a.reuse = std::move(nb);
        a.reuse_cap = nc;
      }
      // readreuseable = [readreuseable; writereuseable]
      k_push_reuse<<<nblk(a.n), TPB, 0, s.stream>>>(flag, pos, a.n, a.reuse.as<uint64_t>(), a.nreuse);
      a.nreuse += k;
      a.nliving -= std::min<uint64_t>(a.nliving, k);
      died_types.push_back(T);
    }
    VG_CUDA(cudaFreeAsync(flag, s.stream));
    VG_CUDA(cudaFreeAsync(pos, s.stream));
  }
  // edges of the written edge types: new container from the appended
  // records (and the old edges with add_existing)
  for (int w : ctx.write) {
    if (!is_edge_ref(w)) continue;
    int e = edge_of(w);
    EdgeAppend *ap = nullptr;
    for (auto &x : ctx.appends)
      if (x->edge_type == e) ap = x.get();
    uint64_t n = 0;
    if (ap) {
      if (ap->ordered) {
        n = ap->fixed_count;
      } else {
        VG_CUDA(cudaMemcpyAsync(&n, ap->counter.p, 8, cudaMemcpyDeviceToHost, s.stream));
        VG_CUDA(cudaStreamSynchronize(s.stream));
      }
      if (n > ap->cap) fail(VG_ERR_DEVICE, "edge append buffer overflow");
    }
    bool merge = s.edges[e].add_existing;
    bool removals = false;
    for (auto &r : ctx.removals)
      if (r->edge_type == e) {
        apply_edge_removals(s, e, *r, ap, n, merge);
        removals = true;
      }
    if (ap && !removals && build_csr_typed(s, e, *ap, n)) continue;
    std::vector<const void *> pl;
    if (ap)
      for (auto &b : ap->payload) pl.push_back(b.p);
    build_csr_from_records(s, e, ap ? ap->from.as<uint64_t>() : nullptr,
                           ap ? ap->to.as<uint64_t>() : nullptr, pl, n,
                           ap ? ap->ordered : true, ap ? ap->key.as<uint64_t>() : nullptr,
                           merge);
  }
  // remove the edges of agents that died (src/AgentMethods.jl:314-345)
  for (int T : died_types) {
    AgentStore &a = s.agents[T - 1];
    remove_died_edges(s, T, a.died_rd.as<uint8_t>(), a.n);
  }
  for (auto &a : ctx.appends) s.append_spare[a->edge_type] = std::move(a);
  ctx.appends.clear();
  ctx.removals.clear();
  s.num_transitions++;
  API_END
}

// apply! with the called type's state exchanged with host memory: upload,
// the transition, download.  The upload runs on the simulation's stream
// ahead of the kernels; a transition whose launch reports finished row
// ranges (bounded_confidence) has each range downloaded on a second stream
// while the launch goes on; otherwise the new state is downloaded after the
// transition.  Returns when the new state is in out_fields.
int vg_apply_host(vg_sim *h, const char *tname, const int *call, int ncall, const int *read,
                  int nread, const int *write, int nwrite, const int *ae, int nae, int with_edge,
                  const double *params, int nparams, int type_nr, const void *const *in_fields,
                  void *const *out_fields, uint64_t n) {
  API_BEGIN
  Sim &s = S(h);
  if (!s.initialized) fail(VG_ERR_ASSERT, "You must call finish_init! before apply!");
  const AgentTypeDesc &ad = s.model->at(type_nr);
  AgentStore &a = s.agents[type_nr - 1];
  if (n > a.n) fail(VG_ERR_ARG, "more values than agent slots");
  if (s.async) check_device_status(s, "asynchronous transition");
  for (size_t f = 0; f < ad.fields.size(); f++) {
    if (!in_fields || !in_fields[f]) continue;
    VG_CUDA(cudaMemcpyAsync(a.rd[f].p, in_fields[f], n * ad.fields[f].size,
                            cudaMemcpyHostToDevice, s.stream));
  }
  Sim::HostExchange hx;
  hx.type_nr = type_nr;
  hx.out = out_fields;
  hx.n = n;
  struct Reset {
    Sim &s;
    ~Reset() { s.host_xchg = nullptr; }
  } reset{s};
  s.host_xchg = &hx;
  const bool was_async = s.async;
  s.async = true;  // the transition's errors are read below, after the downloads
  int rc = vg_apply(h, tname, call, ncall, read, nread, write, nwrite, ae, nae, with_edge, params,
                    nparams);
  s.async = was_async;
  s.host_xchg = nullptr;
  if (rc != VG_OK) {
    if (s.copy_stream) cudaStreamSynchronize(s.copy_stream);
    return rc;
  }
  AgentStore &b = s.agents[type_nr - 1];  // after the buffer swap: the new state
  if (!hx.done && out_fields)
    for (size_t f = 0; f < ad.fields.size(); f++) {
      if (!out_fields[f]) continue;
      VG_CUDA(cudaMemcpyAsync(out_fields[f], b.rd[f].p, n * ad.fields[f].size,
                              cudaMemcpyDeviceToHost, s.stream));
    }
  if (hx.done) VG_CUDA(cudaStreamSynchronize(s.copy_stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
  check_device_status(s, tname);
  API_END
}

int vg_mapreduce_agents(vg_sim *h, int nr, int field, int map_kind, double map_arg, int op,
                        int out_dtype, int has_init, double init, void *out) {
  API_BEGIN
  Sim &s = S(h);
  const AgentTypeDesc &ad = s.model->at(nr);
  if (s.intransition && s.check_readable)
    fail(VG_ERR_ASSERT, "You can not call mapreduce inside of a transition function.");
  if (field < 0 || field >= (int)ad.fields.size()) fail(VG_ERR_ARG, "bad field");
  const int order_flags = op & (VG_REDUCE_ORDERED | VG_REDUCE_TREE);
  op &= 0xff;
  if ((op == VG_OP_AND || op == VG_OP_OR) && (ad.fields[field].dtype == VG_F32 ||
                                              ad.fields[field].dtype == VG_F64) &&
      map_kind == VG_MAP_FIELD)
    fail(VG_ERR_ASSERT, "The & operator is only supported for integer and boolean types");
  AgentStore &a = s.agents[nr - 1];
  RedArgs r{};
  identity_for(op, out_dtype, has_init, init, &r.init_i, &r.init_f);
  int dt = ad.fields[field].dtype;
  r.float_acc = (map_kind == VG_MAP_FIELD && (dt == VG_F32 || dt == VG_F64)) || out_dtype == VG_F64;
  if (!s.initialized) {
    // staged agents on the host
    uint64_t n = a.h_n;
    int64_t ai = r.init_i;
    double af = r.init_f;
    size_t sz = ad.fields[field].size;
    for (uint64_t i = 0; i < n; i++) {
      double v;
      int64_t iv;
      const uint8_t *p = a.h_fields[field].data() + i * sz;
      switch (dt) {
        case VG_F64: v = *(const double *)p; iv = (int64_t)v; break;
        case VG_F32: v = *(const float *)p; iv = (int64_t)v; break;
        case VG_BOOL: case VG_U8: iv = *p; v = iv; break;
        case VG_I32: iv = *(const int32_t *)p; v = iv; break;
        case VG_U32: iv = *(const uint32_t *)p; v = iv; break;
        case VG_I16: iv = *(const int16_t *)p; v = iv; break;
        case VG_U16: iv = *(const uint16_t *)p; v = iv; break;
        case VG_I8: iv = *(const int8_t *)p; v = iv; break;
        default: iv = *(const int64_t *)p; v = (double)iv;
      }
      if (map_kind != VG_MAP_FIELD) {
        bool b = false;
        switch (map_kind) {
          case VG_MAP_EQ: b = v == map_arg; break;
          case VG_MAP_NE: b = v != map_arg; break;
          case VG_MAP_LT: b = v < map_arg; break;
          case VG_MAP_GT: b = v > map_arg; break;
        }
        iv = b;
        v = b;
      }
      switch (op) {
        case VG_OP_ADD: ai = (int64_t)((uint64_t)iv + (uint64_t)ai); af = v + af; break;
        case VG_OP_MUL: ai = (int64_t)((uint64_t)iv * (uint64_t)ai); af = v * af; break;
        case VG_OP_MAX: ai = std::max(iv, ai); af = host_jl_max(v, af); break;
        case VG_OP_MIN: ai = std::min(iv, ai); af = host_jl_min(v, af); break;
        case VG_OP_AND: ai = iv & ai; break;
        case VG_OP_OR: ai = iv | ai; break;
      }
    }
    if (out_dtype == VG_F64) *(double *)out = r.float_acc ? af : (double)ai;
    else if (out_dtype == VG_BOOL) *(uint8_t *)out = (r.float_acc ? af : (double)ai) != 0;
    else *(int64_t *)out = r.float_acc ? (int64_t)af : ai;
    return VG_OK;
  }
  r.p = a.rd[field].p;
  r.dt = dt;
  r.n = a.n;
  r.died = ad.immortal() ? nullptr : a.died_rd.as<uint8_t>();
  r.kind = map_kind;
  r.arg = map_arg;
  r.op = op;
  run_reduce(s, r, out_dtype, fold_in_order(order_flags, r.float_acc, op), out);
  API_END
}

int vg_mapreduce_edges(vg_sim *h, int e, int field, int map_kind, double map_arg, int op,
                       int out_dtype, int has_init, double init, void *out) {
  API_BEGIN
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (ed.stateless())
    fail(VG_ERR_ASSERT, "mapreduce is not defined for the hint combination of " + ed.name);
  if (field < 0 || field >= (int)ed.fields.size()) fail(VG_ERR_ARG, "bad field");
  const int order_flags = op & (VG_REDUCE_ORDERED | VG_REDUCE_TREE);
  op &= 0xff;
  RedArgs r{};
  identity_for(op, out_dtype, has_init, init, &r.init_i, &r.init_f);
  int dt = ed.fields[field].dtype;
  r.float_acc = (map_kind == VG_MAP_FIELD && (dt == VG_F32 || dt == VG_F64)) || out_dtype == VG_F64;
  const bool ordered = fold_in_order(order_flags, r.float_acc, op);
  if (!s.initialized) {
    // Before finish_init! the reference reduces over the (empty) read
    // container: the identity.
    if (out_dtype == VG_F64) *(double *)out = r.float_acc ? r.init_f : (double)r.init_i;
    else if (out_dtype == VG_BOOL) *(uint8_t *)out = r.init_i != 0;
    else *(int64_t *)out = r.init_i;
    return VG_OK;
  }
  EdgeStore &es = s.edges[e];
  // fold over the CSR of every target type in (type, row, insertion) order
  int64_t ai = r.init_i;
  double af = r.init_f;
  for (int T = 1; T < (int)es.csr.size(); T++) {
    CSR &c = es.csr[T];
    if (!c.nedges) continue;
    RedArgs q = r;
    q.p = c.payload[field].p;
    q.dt = dt;
    q.n = c.nedges;
    q.died = nullptr;
    q.kind = map_kind;
    q.arg = map_arg;
    q.op = op;
    q.init_i = ai;
    q.init_f = af;
    if (r.float_acc) {
      double v;
      run_reduce(s, q, VG_F64, ordered, &v);
      af = v;
    } else {
      int64_t v;
      run_reduce(s, q, VG_I64, ordered, &v);
      ai = v;
    }
  }
  if (out_dtype == VG_F64) *(double *)out = r.float_acc ? af : (double)ai;
  else if (out_dtype == VG_BOOL) *(uint8_t *)out = (r.float_acc ? af : (double)ai) != 0;
  else *(int64_t *)out = r.float_acc ? (int64_t)af : ai;
  API_END
}

}  // extern "C"

// A prepared apply!: the arguments of one vg_apply call, copied once.  Each
// run is that vg_apply call (the same checks, the same transition, params or
// globals bound to parameter slots read at each run); the handle only spares
// a caller whose calls are expensive (a foreign-function layer converting
// thirteen arguments) the per-step conversion.
struct vg_apply_call {
  vg_sim *sim = nullptr;
  std::string name;
  std::vector<int> call, read, write, ae;  // (each at least one entry long)
  int ncall = 0, nread = 0, nwrite = 0, nae = 0, with_edge = -1, nparams = 0;
  std::vector<double> params;
};

extern "C" {

int vg_apply_prepare(vg_sim *h, const char *tname, const int *call, int ncall, const int *read,
                     int nread, const int *write, int nwrite, const int *ae, int nae,
                     int with_edge, const double *params, int nparams, vg_apply_call **out) {
  API_BEGIN
  S(h);
  if (!tname) fail(VG_ERR_ARG, "null transition name");
  if (!out) fail(VG_ERR_ARG, "null output pointer");
  bool known = false;
  for (auto &t : transitions()) known |= std::strcmp(t.name, tname) == 0;
  if (!known) fail(VG_ERR_ARG, std::string("unknown transition ") + tname);
  auto list = [](const int *v, int n, const char *what) {
    if (n < 0 || (n > 0 && !v)) fail(VG_ERR_ARG, std::string("bad ") + what + " list");
    std::vector<int> r(v, v + n);
    if (r.empty()) r.push_back(0);
    return r;
  };
  auto c = std::make_unique<vg_apply_call>();
  c->sim = h;
  c->name = tname;
  c->call = list(call, ncall, "call");
  c->read = list(read, nread, "read");
  c->write = list(write, nwrite, "write");
  c->ae = list(ae, nae, "add_existing");
  c->ncall = ncall;
  c->nread = nread;
  c->nwrite = nwrite;
  c->nae = nae;
  c->with_edge = with_edge;
  if (nparams < 0 || (nparams > 0 && !params)) fail(VG_ERR_ARG, "bad parameter list");
  c->params.assign(params, params + nparams);
  c->params.push_back(0.0);
  c->nparams = nparams;
  *out = c.release();
  API_END
}

int vg_apply_call_run(vg_apply_call *c) {
  if (!c) {
    set_last_error("null prepared apply! call");
    return VG_ERR_ARG;
  }
  return vg_apply(c->sim, c->name.c_str(), c->call.data(), c->ncall, c->read.data(), c->nread,
                  c->write.data(), c->nwrite, c->ae.data(), c->nae, c->with_edge,
                  c->params.data(), c->nparams);
}

int vg_apply_call_destroy(vg_apply_call *c) {
  delete c;
  return VG_OK;
}

}  // extern "C"
