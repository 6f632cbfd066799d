// C-ABI entry points: model registry, simulation lifecycle, agent and edge
// staging, finish_init!, host-side accessors, params/globals and rasters.
// The transition engine (apply!) and mapreduce live in vg_apply.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <unordered_set>

#include "vg_internal.h"

namespace vg {

static thread_local std::string g_last_error;
void set_last_error(const std::string &m) { g_last_error = m; }

int dtype_size(int dt) {
  switch (dt) {
    case VG_BOOL: case VG_U8: case VG_I8: return 1;
    case VG_U16: case VG_I16: return 2;
    case VG_U32: case VG_I32: case VG_F32: return 4;
    case VG_U64: case VG_I64: case VG_F64: return 8;
  }
  return 0;
}

void fail(int code, const std::string &msg) { throw Error{code, msg}; }

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess)
    fail(VG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

DevBuf &DevBuf::operator=(DevBuf &&o) noexcept {
  if (this != &o) {
    release();
    p = o.p;
    bytes = o.bytes;
    footprint = o.footprint;
    o.p = nullptr;
    o.bytes = 0;
  }
  return *this;
}

void DevBuf::alloc(size_t b, uint64_t *fp) {
  release();
  if (b == 0) b = 16;
  cudaError_t e = cudaMalloc(&p, b);
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    fail(VG_ERR_NOMEM, "cudaMalloc of " + std::to_string(b) + " bytes failed: " +
                           cudaGetErrorString(e));
  }
  bytes = b;
  footprint = fp;
  if (fp) *fp += b;
}

void DevBuf::release() {
  if (p) {
    cudaFree(p);
    if (footprint) *footprint -= bytes;
  }
  p = nullptr;
  bytes = 0;
}

int AgentTypeDesc::field_index(const std::string &n) const {
  for (size_t i = 0; i < fields.size(); i++)
    if (fields[i].name == n) return (int)i;
  return -1;
}
int EdgeTypeDesc::field_index(const std::string &n) const {
  for (size_t i = 0; i < fields.size(); i++)
    if (fields[i].name == n) return (int)i;
  return -1;
}
const AgentTypeDesc &Model::at(int nr) const {
  if (nr < 1 || nr > (int)atypes.size())
    fail(VG_ERR_ARG, "unknown agent type number " + std::to_string(nr));
  return atypes[nr - 1];
}
const EdgeTypeDesc &Model::et(int e) const {
  if (e < 0 || e >= (int)etypes.size())
    fail(VG_ERR_ARG, "unknown edge type index " + std::to_string(e));
  return etypes[e];
}

void *Sim::scratch(size_t bytes) {
  if (bytes > scratch_bytes) {
    d_scratch.alloc(bytes, &footprint);
    scratch_bytes = bytes;
  }
  return d_scratch.p;
}

const void *Sim::const_table(const std::string &key, const void *host, size_t bytes) {
  ConstTable &t = const_tables[key];
  const uint8_t *h = (const uint8_t *)host;
  if (t.dev.p && t.host.size() == bytes && std::equal(t.host.begin(), t.host.end(), h))
    return t.dev.p;
  if (!t.dev.p || t.dev.bytes < bytes) t.dev.alloc(std::max<size_t>(bytes, 16), &footprint);
  t.host.assign(h, h + bytes);
  // from the kept host copy, which outlives the asynchronous transfer
  VG_CUDA(cudaMemcpyAsync(t.dev.p, t.host.data(), bytes, cudaMemcpyHostToDevice, stream));
  return t.dev.p;
}

void Sim::ensure_device() {
  if (device_ready) return;
  if (!stream) {
    VG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    own_stream = true;
  }
  d_status.alloc(16, &footprint);
  VG_CUDA(cudaMemsetAsync(d_status.p, 0, 16, stream));
  device_ready = true;
}

int Sim::raster_index(const std::string &n) const {
  for (size_t i = 0; i < rasters.size(); i++)
    if (rasters[i].name == n) return (int)i;
  return -1;
}

void check_device_status(Sim &s, const char *what) {
  int h = 0;
  VG_CUDA(cudaMemcpyAsync(&h, s.d_status.p, 4, cudaMemcpyDeviceToHost, s.stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
  if (h) {
    VG_CUDA(cudaMemsetAsync(s.d_status.p, 0, 4, s.stream));
    fail(VG_ERR_DEVICE, std::string(what) + ": device status " + std::to_string(h));
  }
}

DevAgentView agent_view(Sim &s, int nr) {
  DevAgentView v{};
  AgentStore &a = s.agents[nr - 1];
  v.n = a.n;
  for (size_t f = 0; f < a.rd.size() && f < (size_t)MAX_FIELDS; f++) {
    v.rd[f] = a.rd[f].p;
    v.wr[f] = a.wr[f].p;
  }
  v.died_rd = a.died_rd.as<uint8_t>();
  v.died_wr = a.died_wr.as<uint8_t>();
  return v;
}

DevCSRView csr_view(Sim &s, int e, int T) {
  DevCSRView v{};
  EdgeStore &es = s.edges[e];
  if (T < (int)es.csr.size()) {
    CSR &c = es.csr[T];
    v.nrows = c.nrows;
    v.nedges = c.nedges;
    v.row_ptr = c.row_ptr.as<uint32_t>();
    v.src = c.src.as<uint32_t>();
    v.src_type = c.src_type.as<uint8_t>();
    v.src_type_const = c.src_type_const;
    for (size_t f = 0; f < c.payload.size() && f < (size_t)MAX_FIELDS; f++)
      v.payload[f] = c.payload[f].p;
  }
  return v;
}

// grow the slot capacity of an agent type, keeping contents
void agent_reserve(Sim &s, int nr, uint64_t slots) {
  AgentStore &a = s.agents[nr - 1];
  const AgentTypeDesc &ad = s.model->at(nr);
  if (slots <= a.cap && !a.rd.empty()) return;
  uint64_t nc = std::max<uint64_t>({slots, a.cap * 2, 1024});
  auto grow = [&](DevBuf &b, size_t esz) {
    DevBuf nb;
    nb.alloc(nc * esz, &s.footprint);
    VG_CUDA(cudaMemsetAsync(nb.p, 0, nc * esz, s.stream));
    if (b.p && a.n) VG_CUDA(cudaMemcpyAsync(nb.p, b.p, a.n * esz, cudaMemcpyDeviceToDevice, s.stream));
    b = std::move(nb);
  };
  a.rd.resize(ad.fields.size());
  a.wr.resize(ad.fields.size());
  for (size_t f = 0; f < ad.fields.size(); f++) {
    grow(a.rd[f], ad.fields[f].size);
    grow(a.wr[f], ad.fields[f].size);
  }
  if (!ad.immortal()) {
    grow(a.died_rd, 1);
    grow(a.died_wr, 1);
  }
  a.cap = nc;
  VG_CUDA(cudaStreamSynchronize(s.stream));
}

}  // namespace vg

using namespace vg;

#define API_BEGIN try {
#define API_END                           \
  return VG_OK;                           \
  }                                       \
  catch (const Error &e) {                \
    g_last_error = e.msg;                 \
    return e.code;                        \
  }                                       \
  catch (const std::exception &e) {       \
    g_last_error = e.what();              \
    return VG_ERR_ARG;                    \
  }

static Sim &S(vg_sim *s) {
  if (!s || !s->s) fail(VG_ERR_ARG, "null simulation handle");
  return *s->s;
}

static Model &MD(const vg_model *m) {
  if (!m || !m->m) fail(VG_ERR_ARG, "null model handle");
  return *m->m;
}

static const char *NM(const char *name) {
  if (!name) fail(VG_ERR_ARG, "null name");
  return name;
}

static void check_field_args(int nfields, const char *const *names, const int *dtypes) {
  if (nfields < 0) fail(VG_ERR_ARG, "negative field count");
  if (nfields > 0 && (!names || !dtypes)) fail(VG_ERR_ARG, "null field arrays");
  for (int i = 0; i < nfields; i++)
    if (!names[i]) fail(VG_ERR_ARG, "null field name");
}

static void check_fields(const std::vector<FieldDesc> &fs) {
  if (fs.size() > (size_t)MAX_FIELDS)
    fail(VG_ERR_ARG, "at most " + std::to_string(MAX_FIELDS) + " fields per type");
}

extern "C" {

const char *vg_last_error(void) { return g_last_error.c_str(); }
int vg_version(void) { return 10000; }

int vg_device_count(int *out) {
  API_BEGIN
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *out = n;
  API_END
}

// ------------------------------------------------------------------ model
int vg_model_create(vg_model **out) {
  API_BEGIN
  if (!out) fail(VG_ERR_ARG, "null output pointer");
  *out = new vg_model{std::make_shared<Model>()};
  API_END
}

void vg_model_destroy(vg_model *m) { delete m; }

int vg_model_register_agenttype(vg_model *m, const char *name, int nfields,
                                const char *const *names, const int *dtypes,
                                unsigned hints, int *type_nr_out) {
  API_BEGIN
  Model &M = MD(m);
  NM(name);
  check_field_args(nfields, names, dtypes);
  if (M.finalized) fail(VG_ERR_STATE, "model already created");
  for (auto &a : M.atypes)
    if (a.name == name) fail(VG_ERR_ASSERT, std::string("Type ") + name + " is already registered");
  if ((int)M.atypes.size() + 1 >= MAX_AGENT_TYPES)
    fail(VG_ERR_ASSERT, "Can not add new type, maximal number of types already registered");
  if (hints & ~(VG_HINT_IMMORTAL | VG_HINT_INDEPENDENT))
    fail(VG_ERR_ASSERT, std::string("The agent type hint is unknown for type ") + name);
  AgentTypeDesc a;
  a.name = name;
  a.hints = hints;
  for (int i = 0; i < nfields; i++) {
    int sz = dtype_size(dtypes[i]);
    if (!sz) fail(VG_ERR_ARG, "unknown field dtype");
    a.fields.push_back({names[i], dtypes[i], sz});
  }
  check_fields(a.fields);
  a.nr = (int)M.atypes.size() + 1;
  M.atypes.push_back(a);
  if (type_nr_out) *type_nr_out = a.nr;
  API_END
}

int vg_model_register_edgetype(vg_model *m, const char *name, int nfields,
                               const char *const *names, const int *dtypes,
                               unsigned hints, int target, int64_t size,
                               int *edge_type_out) {
  API_BEGIN
  Model &M = MD(m);
  NM(name);
  check_field_args(nfields, names, dtypes);
  if (M.finalized) fail(VG_ERR_STATE, "model already created");
  for (auto &e : M.etypes)
    if (e.name == name) fail(VG_ERR_ASSERT, std::string("Type ") + name + " is already registered");
  if ((int)M.etypes.size() >= MAX_EDGE_TYPES) fail(VG_ERR_ARG, "too many edge types");
  // src/ModelTypes.jl:181-226
  if (hints & VG_HINT_NUMEDGESONLY) hints |= VG_HINT_STATELESS | VG_HINT_IGNOREFROM;
  if (hints & VG_HINT_HASEDGEONLY)
    hints |= VG_HINT_STATELESS | VG_HINT_IGNOREFROM | VG_HINT_SINGLEEDGE;
  if ((hints & VG_HINT_SINGLETYPE) && target <= 0)
    fail(VG_ERR_ASSERT, std::string("For type ") + name +
                            " the :SingleType hint is set, but in this case the agent "
                            "type must also be specified via the target keyword.");
  if (target > 0) hints |= VG_HINT_SINGLETYPE;
  if (nfields == 0) hints |= VG_HINT_STATELESS;  // detect_stateless
  if ((hints & VG_HINT_SINGLETYPE) && (hints & VG_HINT_SINGLEEDGE) &&
      !((hints & VG_HINT_STATELESS) && (hints & VG_HINT_IGNOREFROM)))
    fail(VG_ERR_ASSERT, "The hints :SingleEdge and :SingleType can be only combined "
                        "when the type has also the hints :Stateless and :IgnoreFrom.");
  if (target > 0 && target > (int)M.atypes.size())
    fail(VG_ERR_ARG, "target agent type is not registered");
  EdgeTypeDesc e;
  e.name = name;
  e.hints = hints;
  e.target = target;
  e.size = size;
  for (int i = 0; i < nfields; i++) {
    int sz = dtype_size(dtypes[i]);
    if (!sz) fail(VG_ERR_ARG, "unknown field dtype");
    e.fields.push_back({names[i], dtypes[i], sz});
  }
  check_fields(e.fields);
  e.idx = (int)M.etypes.size();
  M.etypes.push_back(e);
  if (edge_type_out) *edge_type_out = e.idx;
  API_END
}

int vg_model_register_param(vg_model *m, const char *name, double d) {
  API_BEGIN
  MD(m).params.push_back({NM(name), d});
  API_END
}
int vg_model_register_global(vg_model *m, const char *name, double d) {
  API_BEGIN
  MD(m).globals.push_back({NM(name), d});
  API_END
}

int vg_model_finalize(vg_model *m, const char *name) {
  API_BEGIN
  Model &M = MD(m);
  M.name = name ? name : "";
  M.finalized = true;
  API_END
}

int vg_model_edge_hints(const vg_model *m, int e, unsigned *out) {
  API_BEGIN
  if (!out) fail(VG_ERR_ARG, "null output pointer");
  *out = MD(m).et(e).hints;
  API_END
}

int vg_model_type_by_name(const vg_model *m, const char *name, int *out) {
  API_BEGIN
  NM(name);
  if (!out) fail(VG_ERR_ARG, "null output pointer");
  for (auto &a : MD(m).atypes)
    if (a.name == name) { *out = a.nr; return VG_OK; }
  for (auto &e : MD(m).etypes)
    if (e.name == name) { *out = VG_EDGE(e.idx); return VG_OK; }
  fail(VG_ERR_ARG, std::string("unknown type ") + name);
  API_END
}

// ------------------------------------------------------------- lifecycle
int vg_sim_create(vg_model *m, const char *name, void *stream, vg_sim **out) {
  API_BEGIN
  if (!out) fail(VG_ERR_ARG, "null output pointer");
  if (!MD(m).finalized) fail(VG_ERR_STATE, "call create_model (vg_model_finalize) first");
  auto s = std::make_unique<Sim>();
  s->model = m->m;
  s->name = name ? name : m->m->name;
  s->stream = (cudaStream_t)stream;  // NULL: created on first device use
  s->agents.resize(m->m->atypes.size());
  s->edges.resize(m->m->etypes.size());
  for (auto &a : s->agents) (void)a;
  for (size_t i = 0; i < m->m->atypes.size(); i++)
    s->agents[i].h_fields.resize(m->m->atypes[i].fields.size());
  for (auto &p : m->m->params) s->params[p.first] = p.second;
  for (auto &g : m->m->globals) s->globals[g.first] = g.second;
  *out = new vg_sim{std::move(s)};
  API_END
}

Sim::~Sim() {
  if (copy_stream) cudaStreamDestroy(copy_stream);
  if (xchg_flags_host) cudaFreeHost(xchg_flags_host);
}

int vg_sim_destroy(vg_sim *s) {
  API_BEGIN
  if (!s) return VG_OK;
  if (s->s) {
    if (s->s->device_ready) cudaStreamSynchronize(s->s->stream);
    cudaStream_t st = s->s->stream;
    bool own = s->s->own_stream;
    s->s.reset();
    if (own) cudaStreamDestroy(st);
  }
  delete s;
  API_END
}

int vg_sim_set_stream(vg_sim *h, void *stream) {
  API_BEGIN
  Sim &s = S(h);
  if (s.device_ready) VG_CUDA(cudaStreamSynchronize(s.stream));
  if (s.own_stream) cudaStreamDestroy(s.stream);
  s.own_stream = false;
  s.stream = (cudaStream_t)stream;
  API_END
}

int vg_sim_synchronize(vg_sim *h) {
  API_BEGIN
  S(h).ensure_device();
  VG_CUDA(cudaStreamSynchronize(S(h).stream));
  check_device_status(S(h), "asynchronous transition");
  API_END
}

int vg_sim_set_async(vg_sim *h, int async) {
  API_BEGIN
  Sim &s = S(h);
  if (s.async && !async && s.device_ready) check_device_status(s, "asynchronous transition");
  s.async = async != 0;
  API_END
}

int vg_write_agents(vg_sim *h, int nr, const void *const *fields, uint64_t n) {
  API_BEGIN
  Sim &s = S(h);
  const AgentTypeDesc &ad = s.model->at(nr);
  if (!s.initialized) fail(VG_ERR_STATE, "vg_write_agents runs after finish_init!");
  if (s.intransition) fail(VG_ERR_ASSERT, "agent states cannot be set inside a transition");
  AgentStore &a = s.agents[nr - 1];
  if (n > a.n) fail(VG_ERR_ARG, "more values than agent slots");
  for (size_t f = 0; f < ad.fields.size(); f++) {
    if (!fields || !fields[f]) continue;
    VG_CUDA(cudaMemcpyAsync(a.rd[f].p, fields[f], n * ad.fields[f].size, cudaMemcpyHostToDevice,
                            s.stream));
  }
  if (!s.async) VG_CUDA(cudaStreamSynchronize(s.stream));
  API_END
}

int vg_sim_num_transitions(vg_sim *h, int64_t *out) {
  API_BEGIN
  *need(out, "output pointer") = S(h).num_transitions;
  API_END
}

int vg_sim_device_bytes(vg_sim *h, uint64_t *out) {
  API_BEGIN
  *need(out, "output pointer") = S(h).footprint;
  API_END
}

int vg_disable_transition_checks(vg_sim *h, int disable) {
  API_BEGIN
  Sim &s = S(h);
  s.check_readable = !disable;
  s.intransition = disable != 0;
  API_END
}

static void copy_buf(Sim &dst, DevBuf &to, const DevBuf &from, cudaStream_t st) {
  if (!from.p) return;
  to.alloc(from.bytes, &dst.footprint);
  VG_CUDA(cudaMemcpyAsync(to.p, from.p, from.bytes, cudaMemcpyDeviceToDevice, st));
}

int vg_sim_copy(vg_sim *h, vg_sim **out) {
  API_BEGIN
  Sim &s = S(h);
  s.ensure_device();
  auto c = std::make_unique<Sim>();
  c->model = s.model;
  c->name = s.name;
  c->ensure_device();
  VG_CUDA(cudaStreamSynchronize(s.stream));
  c->initialized = s.initialized;
  c->num_transitions = s.num_transitions;
  c->check_readable = s.check_readable;
  c->params = s.params;
  c->globals = s.globals;
  c->global_series = s.global_series;
  c->bindings = s.bindings;
  c->rasters = s.rasters;
  c->agents.resize(s.agents.size());
  for (size_t i = 0; i < s.agents.size(); i++) {
    AgentStore &a = s.agents[i], &b = c->agents[i];
    b.n = a.n; b.cap = a.cap; b.nreuse = a.nreuse; b.reuse_cap = a.reuse_cap;
    b.nliving = a.nliving; b.h_fields = a.h_fields; b.h_n = a.h_n;
    b.rd.resize(a.rd.size());
    b.wr.resize(a.wr.size());
    for (size_t f = 0; f < a.rd.size(); f++) {
      copy_buf(*c, b.rd[f], a.rd[f], c->stream);
      copy_buf(*c, b.wr[f], a.wr[f], c->stream);
    }
    copy_buf(*c, b.died_rd, a.died_rd, c->stream);
    copy_buf(*c, b.died_wr, a.died_wr, c->stream);
    copy_buf(*c, b.reuse, a.reuse, c->stream);
  }
  c->edges.resize(s.edges.size());
  for (size_t e = 0; e < s.edges.size(); e++) {
    EdgeStore &a = s.edges[e], &b = c->edges[e];
    b.implicit = a.implicit; b.st = a.st; b.nstaged = a.nstaged;
    b.single_seen = a.single_seen;
    for (auto &seg : a.staged) {
      EdgeSegment ns;
      ns.device = seg.device; ns.n = seg.n; ns.h_from = seg.h_from; ns.h_to = seg.h_to;
      ns.h_payload = seg.h_payload;
      copy_buf(*c, ns.d_from, seg.d_from, c->stream);
      copy_buf(*c, ns.d_to, seg.d_to, c->stream);
      ns.d_payload.resize(seg.d_payload.size());
      for (size_t f = 0; f < seg.d_payload.size(); f++)
        copy_buf(*c, ns.d_payload[f], seg.d_payload[f], c->stream);
      b.staged.push_back(std::move(ns));
    }
    b.csr.resize(a.csr.size());
    for (size_t T = 0; T < a.csr.size(); T++) {
      CSR &x = a.csr[T], &y = b.csr[T];
      y.nrows = x.nrows; y.nedges = x.nedges; y.src_type_const = x.src_type_const;
      y.max_degree = csr_max_degree(s, x);
      copy_buf(*c, y.row_ptr, x.row_ptr, c->stream);
      copy_buf(*c, y.src, x.src, c->stream);
      copy_buf(*c, y.src_type, x.src_type, c->stream);
      y.payload.resize(x.payload.size());
      for (size_t f = 0; f < x.payload.size(); f++)
        copy_buf(*c, y.payload[f], x.payload[f], c->stream);
    }
  }
  VG_CUDA(cudaStreamSynchronize(c->stream));
  *out = new vg_sim{std::move(c)};
  API_END
}

// -------------------------------------------------------- params/globals
int vg_set_param(vg_sim *h, const char *name, double v) {
  API_BEGIN
  Sim &s = S(h);
  if (s.initialized)
    fail(VG_ERR_ASSERT, "You can call `set_param!` only before `finish_init!`. For values "
                        "that change while the simulation is running, register them as "
                        "globals and use `set_global!` instead.");
  s.params[name] = v;
  API_END
}
int vg_param(vg_sim *h, const char *name, double *out) {
  API_BEGIN
  Sim &s = S(h);
  auto it = s.params.find(name);
  if (it == s.params.end()) fail(VG_ERR_ARG, std::string("unknown param ") + name);
  *out = it->second;
  API_END
}
int vg_set_global(vg_sim *h, const char *name, double v) {
  API_BEGIN
  S(h).globals[name] = v;
  API_END
}
int vg_get_global(vg_sim *h, const char *name, double *out) {
  API_BEGIN
  Sim &s = S(h);
  auto it = s.globals.find(name);
  if (it == s.globals.end()) fail(VG_ERR_ARG, std::string("unknown global ") + name);
  *out = it->second;
  API_END
}
int vg_bind_param(vg_sim *h, const char *transition, int slot, int kind, const char *name) {
  API_BEGIN
  Sim &s = S(h);
  need(transition, "transition name");
  need(name, "param or global name");
  bool known = false;
  for (auto &t : transitions()) known |= std::strcmp(t.name, transition) == 0;
  if (!known) fail(VG_ERR_ARG, std::string("unknown transition ") + transition);
  if (slot < 0 || slot >= 64) fail(VG_ERR_ARG, "parameter slot 0..63");
  if (kind == 0 && !s.params.count(name)) fail(VG_ERR_ARG, std::string("unknown param ") + name);
  if (kind == 1 && !s.globals.count(name)) fail(VG_ERR_ARG, std::string("unknown global ") + name);
  if (kind != 0 && kind != 1) fail(VG_ERR_ARG, "kind 0 (param) or 1 (global)");
  auto &v = s.bindings[transition];
  for (auto &b : v)
    if (b.slot == slot) {
      b.kind = kind;
      b.name = name;
      return VG_OK;
    }
  v.push_back({slot, kind, name});
  API_END
}

int vg_unbind_params(vg_sim *h, const char *transition) {
  API_BEGIN
  Sim &s = S(h);
  if (transition) s.bindings.erase(transition);
  else s.bindings.clear();
  API_END
}

int vg_push_global(vg_sim *h, const char *name, double v) {
  API_BEGIN
  S(h).global_series[name].push_back(v);
  API_END
}
int vg_global_series(vg_sim *h, const char *name, double *out, uint64_t cap,
                     uint64_t *n_out) {
  API_BEGIN
  need(n_out, "count pointer");
  auto &v = S(h).global_series[need(name, "name")];
  *n_out = v.size();
  if (out) std::memcpy(out, v.data(), std::min<uint64_t>(cap, v.size()) * 8);
  API_END
}

// ----------------------------------------------------------------- agents
int vg_add_agents(vg_sim *h, int nr, uint64_t n, const void *const *fields,
                  uint64_t *ids_out) {
  API_BEGIN
  Sim &s = S(h);
  const AgentTypeDesc &ad = s.model->at(nr);
  if (s.initialized)
    fail(VG_ERR_ASSERT, "You can call add_agent! only in the initialization phase (until "
                        "`finish_init!` is called) or within a transition function called "
                        "by `apply`.");
  AgentStore &a = s.agents[nr - 1];
  if (a.h_n + n > NR_MASK) fail(VG_ERR_ASSERT, "agent_nr is too big");
  for (size_t f = 0; f < ad.fields.size(); f++) {
    size_t sz = ad.fields[f].size;
    auto &col = a.h_fields[f];
    size_t old = col.size();
    col.resize(old + n * sz);
    if (fields && fields[f]) std::memcpy(col.data() + old, fields[f], n * sz);
    else std::memset(col.data() + old, 0, n * sz);
  }
  if (ids_out)
    for (uint64_t i = 0; i < n; i++) ids_out[i] = make_id(nr, a.h_n + 1 + i);
  a.h_n += n;
  API_END
}

int vg_add_agent_per_process(vg_sim *h, int nr, const void *const *fields,
                             uint64_t *id_out) {
  API_BEGIN
  Sim &s = S(h);
  const AgentTypeDesc &ad = s.model->at(nr);
  if (!s.initialized)
    fail(VG_ERR_ASSERT, "add_agent_per_process! can only be called after finish_init!");
  if (s.intransition)
    fail(VG_ERR_ASSERT, "add_agent_per_process! cannot be called within a transition function");
  AgentStore &a = s.agents[nr - 1];
  uint64_t slot;  // 1-based agent number; reuse a died slot first (LIFO)
  if (!ad.immortal() && a.nreuse > 0) {
    VG_CUDA(cudaMemcpyAsync(&slot, a.reuse.as<uint64_t>() + a.nreuse - 1, 8,
                            cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    a.nreuse--;
  } else {
    agent_reserve(s, nr, a.n + 1);
    slot = ++a.n;
  }
  for (size_t f = 0; f < ad.fields.size(); f++) {
    size_t sz = ad.fields[f].size;
    VG_CUDA(cudaMemcpyAsync(a.rd[f].as<uint8_t>() + (slot - 1) * sz, fields[f], sz,
                            cudaMemcpyHostToDevice, s.stream));
    VG_CUDA(cudaMemcpyAsync(a.wr[f].as<uint8_t>() + (slot - 1) * sz, fields[f], sz,
                            cudaMemcpyHostToDevice, s.stream));
  }
  if (!ad.immortal()) {
    VG_CUDA(cudaMemsetAsync(a.died_rd.as<uint8_t>() + slot - 1, 0, 1, s.stream));
    VG_CUDA(cudaMemsetAsync(a.died_wr.as<uint8_t>() + slot - 1, 0, 1, s.stream));
  }
  a.nliving++;
  VG_CUDA(cudaStreamSynchronize(s.stream));
  *id_out = make_id(nr, slot);
  API_END
}

static void require_readable_agent(Sim &s, int nr) {
  if (s.check_readable && !s.agents[nr - 1].readable)
    fail(VG_ERR_ASSERT, s.model->at(nr).name +
                            " must be in the `read` argument of the transition function.");
}

static bool slot_died(Sim &s, int nr, uint64_t slot) {
  const AgentTypeDesc &ad = s.model->at(nr);
  if (ad.immortal()) return false;
  AgentStore &a = s.agents[nr - 1];
  uint8_t d = 0;
  VG_CUDA(cudaMemcpyAsync(&d, a.died_rd.as<uint8_t>() + slot - 1, 1, cudaMemcpyDeviceToHost, s.stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
  return d != 0;
}

int vg_agentstate(vg_sim *h, uint64_t id, int nr, void *const *out) {
  API_BEGIN
  Sim &s = S(h);
  const AgentTypeDesc &ad = s.model->at(nr);
  if (id_type(id) != nr) fail(VG_ERR_ASSERT, "The id of the agent does not match the given type");
  uint64_t slot = id_nr(id);
  AgentStore &a = s.agents[nr - 1];
  if (!s.initialized) {
    if (slot == 0 || slot > a.h_n) fail(VG_ERR_ASSERT, "agent does not exist");
    for (size_t f = 0; f < ad.fields.size(); f++)
      std::memcpy(out[f], a.h_fields[f].data() + (slot - 1) * ad.fields[f].size, ad.fields[f].size);
    return VG_OK;
  }
  require_readable_agent(s, nr);
  if (slot == 0 || slot > a.n) fail(VG_ERR_ASSERT, "agent does not exist");
  if (slot_died(s, nr, slot))
    fail(VG_ERR_ASSERT, "agentstate was requested for agent " + std::to_string(id) +
                            " that has been removed");
  for (size_t f = 0; f < ad.fields.size(); f++) {
    size_t sz = ad.fields[f].size;
    VG_CUDA(cudaMemcpyAsync(out[f], a.rd[f].as<uint8_t>() + (slot - 1) * sz, sz,
                            cudaMemcpyDeviceToHost, s.stream));
  }
  VG_CUDA(cudaStreamSynchronize(s.stream));
  API_END
}

int vg_agent_slots(vg_sim *h, int nr, uint64_t *out) {
  API_BEGIN
  need(out, "output pointer");
  Sim &s = S(h);
  s.model->at(nr);
  AgentStore &a = s.agents[nr - 1];
  *out = s.initialized ? a.n : a.h_n;
  API_END
}

static std::vector<uint8_t> read_died(Sim &s, int nr) {
  AgentStore &a = s.agents[nr - 1];
  std::vector<uint8_t> d(a.n, 0);
  if (!s.model->at(nr).immortal() && a.n) {
    VG_CUDA(cudaMemcpyAsync(d.data(), a.died_rd.p, a.n, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
  }
  return d;
}

int vg_num_agents(vg_sim *h, int nr, uint64_t *out) {
  API_BEGIN
  need(out, "output pointer");
  Sim &s = S(h);
  s.model->at(nr);
  AgentStore &a = s.agents[nr - 1];
  if (!s.initialized) {
    *out = a.h_n;
    return VG_OK;
  }
  auto d = read_died(s, nr);
  uint64_t c = 0;
  for (auto x : d) c += (x == 0);
  *out = c;
  API_END
}

int vg_read_agents(vg_sim *h, int nr, void *const *fields_out, uint8_t *died_out,
                   uint64_t cap, uint64_t *n_out) {
  API_BEGIN
  need(n_out, "count pointer");
  Sim &s = S(h);
  const AgentTypeDesc &ad = s.model->at(nr);
  AgentStore &a = s.agents[nr - 1];
  uint64_t n = s.initialized ? a.n : a.h_n;
  *n_out = n;
  uint64_t m = std::min(n, cap);
  if (!m) return VG_OK;
  if (s.initialized && s.async) check_device_status(s, "asynchronous transition");
  for (size_t f = 0; f < ad.fields.size(); f++) {
    if (!fields_out || !fields_out[f]) continue;
    size_t sz = ad.fields[f].size;
    if (s.initialized)
      VG_CUDA(cudaMemcpyAsync(fields_out[f], a.rd[f].p, m * sz, cudaMemcpyDeviceToHost, s.stream));
    else
      std::memcpy(fields_out[f], a.h_fields[f].data(), m * sz);
  }
  if (died_out) {
    if (s.initialized && !ad.immortal())
      VG_CUDA(cudaMemcpyAsync(died_out, a.died_rd.p, m, cudaMemcpyDeviceToHost, s.stream));
    else
      std::memset(died_out, 0, m);
  }
  VG_CUDA(cudaStreamSynchronize(s.stream));
  API_END
}

int vg_all_agents(vg_sim *h, int nr, void *const *fields_out, uint64_t *ids_out,
                  uint64_t cap, uint64_t *n_out) {
  API_BEGIN
  Sim &s = S(h);
  const AgentTypeDesc &ad = s.model->at(nr);
  AgentStore &a = s.agents[nr - 1];
  uint64_t n = s.initialized ? a.n : a.h_n;
  std::vector<uint8_t> died = s.initialized ? read_died(s, nr) : std::vector<uint8_t>(n, 0);
  std::vector<std::vector<uint8_t>> cols(ad.fields.size());
  for (size_t f = 0; f < ad.fields.size(); f++) {
    cols[f].resize(n * ad.fields[f].size);
    if (!n) continue;
    if (s.initialized)
      VG_CUDA(cudaMemcpyAsync(cols[f].data(), a.rd[f].p, cols[f].size(), cudaMemcpyDeviceToHost, s.stream));
    else
      std::memcpy(cols[f].data(), a.h_fields[f].data(), cols[f].size());
  }
  VG_CUDA(cudaStreamSynchronize(s.stream));
  uint64_t k = 0;
  for (uint64_t i = 0; i < n; i++) {
    if (died[i]) continue;
    if (k < cap) {
      for (size_t f = 0; f < ad.fields.size(); f++)
        if (fields_out && fields_out[f])
          std::memcpy((uint8_t *)fields_out[f] + k * ad.fields[f].size,
                      cols[f].data() + i * ad.fields[f].size, ad.fields[f].size);
      if (ids_out) ids_out[k] = make_id(nr, i + 1);
    }
    k++;
  }
  *n_out = k;
  API_END
}

int vg_agent_field_device_ptr(vg_sim *h, int nr, int field, void **out) {
  API_BEGIN
  Sim &s = S(h);
  const AgentTypeDesc &ad = s.model->at(nr);
  if (field < 0 || field >= (int)ad.fields.size()) fail(VG_ERR_ARG, "bad field");
  if (!s.initialized) fail(VG_ERR_STATE, "device buffers exist after finish_init!");
  *out = s.agents[nr - 1].rd[field].p;
  API_END
}

}  // extern "C"

// ------------------------------------------------------------------ edges
static void stage_host_edges(Sim &s, int e, uint64_t n, const uint64_t *from,
                             const uint64_t *to, const void *const *payload) {
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  if (es.implicit) fail(VG_ERR_ARG, "edge type " + ed.name + " holds implicit raster edges");
  // :SingleEdge check of _can_add (src/EdgeMethods.jl:257-294)
  bool check_single = ed.singleedge() && !ed.singletype() && !(ed.ignorefrom() && ed.stateless());
  if (es.staged.empty() || es.staged.back().device) {
    EdgeSegment seg;
    seg.h_payload.resize(ed.stores_payload() ? ed.fields.size() : 0);
    es.staged.push_back(std::move(seg));
  }
  EdgeSegment &seg = es.staged.back();
  for (uint64_t i = 0; i < n; i++) {
    if (id_type(to[i]) < 1 || id_type(to[i]) > (int)s.model->atypes.size())
      fail(VG_ERR_ASSERT, "add_edge!: the target is not a valid agent id");
    if (ed.singletype() && id_type(to[i]) != ed.target)
      fail(VG_ERR_ASSERT, "The :SingleType hint is set for " + ed.name +
                              ", and the agent type is specified as " +
                              s.model->at(ed.target).name + ".");
    if (check_single) {
      auto it = es.single_seen.find(to[i]);
      if (it != es.single_seen.end()) {
        // allowed only when the stored value is identical
        uint64_t prev = it->second;  // global staged index
        bool same = true;
        // locate previous record (host segments only)
        uint64_t base = 0;
        for (auto &sg : es.staged) {
          if (prev < base + sg.n) {
            uint64_t j = prev - base;
            if (!sg.device) {
              if (ed.stores_src() && sg.h_from[j] != (from ? from[i] : 0)) same = false;
              for (size_t f = 0; f < sg.h_payload.size(); f++) {
                size_t sz = ed.fields[f].size;
                const uint8_t *old_v = sg.h_payload[f].data() + j * sz;
                if (payload && payload[f]) {
                  if (std::memcmp(old_v, (const uint8_t *)payload[f] + i * sz, sz)) same = false;
                } else {  // a missing payload is staged as zeros
                  for (size_t b = 0; b < sz; b++)
                    if (old_v[b]) same = false;
                }
              }
            }
            break;
          }
          base += sg.n;
        }
        if (!same)
          fail(VG_ERR_ASSERT, "An edge has already been added to the agent with the id " +
                                  std::to_string(to[i]) +
                                  " (and the edgetype hints containing the :SingleEdge hint).");
        continue;  // identical value: the container keeps one edge
      }
      es.single_seen[to[i]] = es.nstaged;
    }
    seg.h_from.push_back(from ? from[i] : 0);
    seg.h_to.push_back(to[i]);
    for (size_t f = 0; f < seg.h_payload.size(); f++) {
      size_t sz = ed.fields[f].size;
      auto &col = seg.h_payload[f];
      size_t old = col.size();
      col.resize(old + sz);
      if (payload && payload[f]) std::memcpy(col.data() + old, (const uint8_t *)payload[f] + i * sz, sz);
      else std::memset(col.data() + old, 0, sz);
    }
    seg.n++;
    es.nstaged++;
  }
}

namespace vg {
// Upload staged segments of edge type e into one device record batch, in
// call order.  Returns the record count.
uint64_t upload_staged(Sim &s, int e, DevBuf &from, DevBuf &to,
                       std::vector<DevBuf> &payload) {
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  uint64_t n = 0;
  for (auto &sg : es.staged) n += sg.n;
  int nf = ed.stores_payload() ? (int)ed.fields.size() : 0;
  from.alloc(std::max<uint64_t>(n, 1) * 8, &s.footprint);
  to.alloc(std::max<uint64_t>(n, 1) * 8, &s.footprint);
  payload.resize(nf);
  for (int f = 0; f < nf; f++) payload[f].alloc(std::max<uint64_t>(n, 1) * ed.fields[f].size, &s.footprint);
  uint64_t off = 0;
  for (auto &sg : es.staged) {
    if (!sg.n) continue;
    auto kind = sg.device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    VG_CUDA(cudaMemcpyAsync(from.as<uint64_t>() + off, sg.device ? sg.d_from.p : (void *)sg.h_from.data(), sg.n * 8, kind, s.stream));
    VG_CUDA(cudaMemcpyAsync(to.as<uint64_t>() + off, sg.device ? sg.d_to.p : (void *)sg.h_to.data(), sg.n * 8, kind, s.stream));
    for (int f = 0; f < nf; f++) {
      size_t sz = ed.fields[f].size;
      const void *srcp = sg.device ? sg.d_payload[f].p : (const void *)sg.h_payload[f].data();
      VG_CUDA(cudaMemcpyAsync(payload[f].as<uint8_t>() + off * sz, srcp, sg.n * sz, kind, s.stream));
    }
    off += sg.n;
  }
  VG_CUDA(cudaStreamSynchronize(s.stream));
  es.staged.clear();
  es.nstaged = 0;
  es.single_seen.clear();
  return n;
}

void flush_staged_edges(Sim &s, int e, bool merge) {
  DevBuf from, to;
  std::vector<DevBuf> pl;
  uint64_t n = upload_staged(s, e, from, to, pl);
  std::vector<const void *> pp;
  for (auto &b : pl) pp.push_back(b.p);
  build_csr_from_records(s, e, from.as<uint64_t>(), to.as<uint64_t>(), pp, n, true,
                         nullptr, merge);
}
}  // namespace vg

extern "C" {

int vg_add_edges(vg_sim *h, int e, uint64_t n, const uint64_t *from,
                 const uint64_t *to, const void *const *payload) {
  API_BEGIN
  if (n) need(to, "target ids");
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (s.initialized && !s.intransition)
    fail(VG_ERR_ASSERT, "You can call add_edge! only in the initialization phase (until "
                        "`finish_init!` is called) or within a transition function called "
                        "by `apply`.");
  if (s.initialized && s.check_readable && !s.edges[e].writeable)
    fail(VG_ERR_ASSERT, ed.name + " must be in the `write` argument of the transition function.");
  if (ed.stores_src() && !from) fail(VG_ERR_ARG, "from ids are required");
  stage_host_edges(s, e, n, from, to, payload);
  if (s.initialized) flush_staged_edges(s, e, true);  // visible immediately
  API_END
}

int vg_add_graph(vg_sim *h, int type_nr, uint64_t nv, const void *const *fields, int e,
                 uint64_t ne, const uint64_t *src, const uint64_t *dst, int directed,
                 const void *const *payload, uint64_t *ids_out) {
  API_BEGIN
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (s.initialized)
    fail(VG_ERR_ASSERT, "add_graph! adds agents: only in the initialization phase (until "
                        "`finish_init!` is called).");
  if (ne) {
    need(src, "source vertices");
    need(dst, "target vertices");
    if (ed.stores_payload())
      for (size_t f = 0; f < ed.fields.size(); f++)
        if (!payload || !payload[f]) fail(VG_ERR_ARG, "null edge field values");
  }
  for (uint64_t k = 0; k < ne; k++)
    if (src[k] < 1 || src[k] > nv || dst[k] < 1 || dst[k] > nv)
      fail(VG_ERR_ARG, "graph edge " + std::to_string(k + 1) + " names a vertex outside 1.." +
                           std::to_string(nv));
  std::vector<uint64_t> ids(nv);
  int rc = vg_add_agents(h, type_nr, nv, fields, ids.data());
  if (rc) fail(rc, vg_last_error());
  // for each graph edge in order: add_edge!(src, dst) and, undirected,
  // add_edge!(dst, src) with the same state
  const uint64_t m = directed ? ne : 2 * ne;
  std::vector<uint64_t> from(m), to(m);
  const int nf = ed.stores_payload() ? (int)ed.fields.size() : 0;
  std::vector<std::vector<uint8_t>> cols(nf);
  std::vector<const void *> pl(nf);
  for (int f = 0; f < nf; f++) {
    const size_t sz = ed.fields[f].size;
    cols[f].resize(m * sz);
    for (uint64_t k = 0; k < ne; k++) {
      const uint8_t *v = (const uint8_t *)payload[f] + k * sz;
      if (directed) {
        std::memcpy(cols[f].data() + k * sz, v, sz);
      } else {
        std::memcpy(cols[f].data() + 2 * k * sz, v, sz);
        std::memcpy(cols[f].data() + (2 * k + 1) * sz, v, sz);
      }
    }
    pl[f] = cols[f].data();
  }
  for (uint64_t k = 0; k < ne; k++) {
    const uint64_t a = ids[src[k] - 1], b = ids[dst[k] - 1];
    if (directed) {
      from[k] = a;
      to[k] = b;
    } else {
      from[2 * k] = a;
      to[2 * k] = b;
      from[2 * k + 1] = b;
      to[2 * k + 1] = a;
    }
  }
  if (m) {
    rc = vg_add_edges(h, e, m, from.data(), to.data(), nf ? pl.data() : nullptr);
    if (rc) fail(rc, vg_last_error());
  }
  if (ids_out) std::memcpy(ids_out, ids.data(), nv * 8);
  API_END
}

int vg_remove_edges(vg_sim *h, int e, uint64_t n, const uint64_t *from,
                    const uint64_t *to) {
  API_BEGIN
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (s.initialized && !s.intransition)
    fail(VG_ERR_ASSERT, "You can call remove_edges! only in the initialization phase (until "
                        "`finish_init!` is called) or within a transition function called "
                        "by `apply`.");
  if (n) need(to, "target ids");
  if (from && ed.ignorefrom())
    fail(VG_ERR_ASSERT, "remove_edges! with a source agent is not defined for edgetypes "
                        "with the :IgnoreFrom hint.");
  // Host path: materialise the current edges, filter, rebuild.
  if (!s.initialized) {
    EdgeStore &es = s.edges[e];
    for (auto &sg : es.staged)
      if (sg.device) fail(VG_ERR_STATE, "remove_edges! on device-staged edges before finish_init!");
    // One filtering pass for all n removals: dropping the edges that match
    // any of the keys equals dropping them key by key, and keeps the
    // insertion order of the rest.
    struct PairHash {
      size_t operator()(const std::pair<uint64_t, uint64_t> &p) const {
        return std::hash<uint64_t>()(p.first * 0x9e3779b97f4a7c15ull ^ p.second);
      }
    };
    std::unordered_set<uint64_t> drop_to;
    std::unordered_set<std::pair<uint64_t, uint64_t>, PairHash> drop_pair;
    for (uint64_t i = 0; i < n; i++) {
      if (from)
        drop_pair.insert({to[i], from[i]});
      else
        drop_to.insert(to[i]);
    }
    if (n) {
      for (auto &sg : es.staged) {
        EdgeSegment ns;
        ns.h_payload.resize(sg.h_payload.size());
        for (uint64_t j = 0; j < sg.n; j++) {
          bool drop = from ? drop_pair.count({sg.h_to[j], sg.h_from[j]}) != 0
                           : drop_to.count(sg.h_to[j]) != 0;
          if (drop) continue;
          ns.h_from.push_back(sg.h_from[j]);
          ns.h_to.push_back(sg.h_to[j]);
          for (size_t f = 0; f < sg.h_payload.size(); f++) {
            size_t sz = ed.fields[f].size;
            ns.h_payload[f].insert(ns.h_payload[f].end(), sg.h_payload[f].begin() + j * sz,
                                   sg.h_payload[f].begin() + (j + 1) * sz);
          }
          ns.n++;
        }
        sg = std::move(ns);
      }
    }
    es.nstaged = 0;
    es.single_seen.clear();
    uint64_t k = 0;
    for (auto &sg : es.staged) {
      for (uint64_t j = 0; j < sg.n; j++, k++)
        if (ed.singleedge()) es.single_seen[sg.h_to[j]] = k;
      es.nstaged += sg.n;
    }
    return VG_OK;
  }
  fail(VG_ERR_STATE, "remove_edges! after finish_init! runs inside transitions");
  API_END
}

// ---------------------------------------------------------- finish_init!
int vg_finish_init(vg_sim *h) {
  API_BEGIN
  Sim &s = S(h);
  if (s.initialized) fail(VG_ERR_ASSERT, "You can not call finish_init! twice for the same simulation");
  s.ensure_device();
  // agents: upload the staged SoA columns; read == write after finish_write!
  for (size_t i = 0; i < s.agents.size(); i++) {
    AgentStore &a = s.agents[i];
    const AgentTypeDesc &ad = s.model->atypes[i];
    int nr = (int)i + 1;
    agent_reserve(s, nr, std::max<uint64_t>(a.h_n, 1));
    a.n = a.h_n;
    for (size_t f = 0; f < ad.fields.size(); f++) {
      if (!a.n) continue;
      VG_CUDA(cudaMemcpyAsync(a.rd[f].p, a.h_fields[f].data(), a.n * ad.fields[f].size,
                              cudaMemcpyHostToDevice, s.stream));
      VG_CUDA(cudaMemcpyAsync(a.wr[f].p, a.h_fields[f].data(), a.n * ad.fields[f].size,
                              cudaMemcpyHostToDevice, s.stream));
    }
    a.nliving = a.n;
    VG_CUDA(cudaStreamSynchronize(s.stream));
    for (auto &c : a.h_fields) std::vector<uint8_t>().swap(c);
  }
  for (size_t e = 0; e < s.edges.size(); e++) {
    EdgeStore &es = s.edges[e];
    if (es.implicit) continue;
    flush_staged_edges(s, (int)e, false);
  }
  s.initialized = true;
  s.num_transitions = 1;  // src/Simulation.jl:473
  API_END
}

}  // extern "C"

// -------------------------------------------------------------- accessors
namespace vg {
// Host view of one target row of an edge type (implicit or CSR).
struct HostRow {
  bool present = false;     // a container exists for this agent
  std::vector<uint64_t> from;
  std::vector<std::vector<uint8_t>> payload;
  uint64_t count = 0;
};

void stencil_sources(const Sim &, const StencilDesc &st, uint64_t cell,
                     std::vector<uint64_t> &out_lin);

HostRow host_row(Sim &s, int e, uint64_t to, bool want_data) {
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  HostRow r;
  int T = id_type(to);
  uint64_t nr = id_nr(to);
  if (T < 1 || T > (int)s.model->atypes.size()) fail(VG_ERR_ASSERT, "invalid agent id");
  if (ed.singletype() && T != ed.target)
    fail(VG_ERR_ASSERT, "The :SingleType hint is set for " + ed.name +
                            ", and the agent type is specified as " +
                            s.model->at(ed.target).name + ". But the type for the given agent is " +
                            s.model->at(T).name + ".");
  if (es.implicit) {
    const StencilDesc &st = es.st;
    const Raster &R = s.rasters[st.raster];
    if (T != R.type_nr || nr < R.first_nr || nr >= R.first_nr + R.ncells) return r;
    std::vector<uint64_t> lin;
    stencil_sources(s, st, nr - R.first_nr, lin);
    r.count = lin.size();
    r.present = r.count > 0;
    if (want_data) {
      for (auto l : lin) r.from.push_back(make_id(R.type_nr, R.first_nr + l));
      r.payload.resize(ed.stores_payload() ? ed.fields.size() : 0);
      for (size_t f = 0; f < r.payload.size(); f++) {
        size_t sz = ed.fields[f].size, off = 0;
        for (size_t g = 0; g < f; g++) off += ed.fields[g].size;
        for (size_t k = 0; k < lin.size(); k++)
          r.payload[f].insert(r.payload[f].end(), st.payload.begin() + off, st.payload.begin() + off + sz);
      }
    }
    return r;
  }
  if (!s.initialized) {
    // staged edges (write container before finish_init!)
    for (auto &sg : es.staged) {
      if (sg.device) fail(VG_ERR_STATE, "edges staged on the device are read after finish_init!");
      for (uint64_t j = 0; j < sg.n; j++) {
        if (sg.h_to[j] != to) continue;
        r.count++;
        if (want_data) {
          r.from.push_back(sg.h_from[j]);
          r.payload.resize(sg.h_payload.size());
          for (size_t f = 0; f < sg.h_payload.size(); f++) {
            size_t sz = ed.fields[f].size;
            r.payload[f].insert(r.payload[f].end(), sg.h_payload[f].begin() + j * sz,
                                sg.h_payload[f].begin() + (j + 1) * sz);
          }
        }
      }
    }
    if (ed.bool_only() && r.count > 1) r.count = 1;
    r.present = r.count > 0;
    return r;
  }
  if (T >= (int)es.csr.size()) return r;
  CSR &c = es.csr[T];
  if (nr == 0 || nr > c.nrows) return r;
  uint32_t rp[2];
  VG_CUDA(cudaMemcpyAsync(rp, c.row_ptr.as<uint32_t>() + nr - 1, 8, cudaMemcpyDeviceToHost, s.stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
  r.count = rp[1] - rp[0];
  r.present = r.count > 0;
  if (want_data && r.count) {
    if (c.src.p) {
      std::vector<uint32_t> src(r.count);
      std::vector<uint8_t> st(r.count, (uint8_t)std::max(c.src_type_const, 0));
      VG_CUDA(cudaMemcpyAsync(src.data(), c.src.as<uint32_t>() + rp[0], r.count * 4, cudaMemcpyDeviceToHost, s.stream));
      if (c.src_type.p)
        VG_CUDA(cudaMemcpyAsync(st.data(), c.src_type.as<uint8_t>() + rp[0], r.count, cudaMemcpyDeviceToHost, s.stream));
      VG_CUDA(cudaStreamSynchronize(s.stream));
      for (uint64_t k = 0; k < r.count; k++) r.from.push_back(make_id(st[k], (uint64_t)src[k] + 1));
    }
    r.payload.resize(c.payload.size());
    for (size_t f = 0; f < c.payload.size(); f++) {
      size_t sz = ed.fields[f].size;
      r.payload[f].resize(r.count * sz);
      VG_CUDA(cudaMemcpyAsync(r.payload[f].data(), c.payload[f].as<uint8_t>() + (uint64_t)rp[0] * sz,
                              r.count * sz, cudaMemcpyDeviceToHost, s.stream));
    }
    VG_CUDA(cudaStreamSynchronize(s.stream));
  }
  return r;
}
}  // namespace vg

static void require_readable_edge(Sim &s, int e) {
  if (s.initialized && s.check_readable && !s.edges[e].readable)
    fail(VG_ERR_ASSERT, "You try to access an edge of type " + s.model->et(e).name +
                            " but the type is not in the `read` argument of the apply! function.");
}

static void write_row(const EdgeTypeDesc &ed, const HostRow &r, uint64_t *from_out,
                      void *const *payload_out, uint64_t cap) {
  uint64_t m = std::min<uint64_t>(cap, r.count);
  if (from_out)
    for (uint64_t k = 0; k < m && k < r.from.size(); k++) from_out[k] = r.from[k];
  if (payload_out)
    for (size_t f = 0; f < r.payload.size(); f++)
      if (payload_out[f]) std::memcpy(payload_out[f], r.payload[f].data(), m * ed.fields[f].size);
}

extern "C" {

int vg_edges(vg_sim *h, uint64_t to, int e, uint64_t *from_out,
             void *const *payload_out, uint64_t cap, int64_t *count_out) {
  API_BEGIN
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (ed.stateless() || ed.ignorefrom())
    fail(VG_ERR_ASSERT, "edges is not defined for the hint combination of " + ed.name);
  require_readable_edge(s, e);
  HostRow r = host_row(s, e, to, true);
  *count_out = r.present ? (int64_t)r.count : -1;
  write_row(ed, r, from_out, payload_out, cap);
  API_END
}

int vg_neighborids(vg_sim *h, uint64_t to, int e, uint64_t *from_out, uint64_t cap,
                   int64_t *count_out) {
  API_BEGIN
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (ed.ignorefrom())
    fail(VG_ERR_ASSERT, "neighborids is not defined for the hint combination of " + ed.name);
  require_readable_edge(s, e);
  HostRow r = host_row(s, e, to, true);
  *count_out = r.present ? (int64_t)r.count : -1;
  write_row(ed, r, from_out, nullptr, cap);
  API_END
}

int vg_edgestates(vg_sim *h, uint64_t to, int e, void *const *payload_out,
                  uint64_t cap, int64_t *count_out) {
  API_BEGIN
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (ed.stateless())
    fail(VG_ERR_ASSERT, "edgestates is not defined for the hint combination of " + ed.name);
  require_readable_edge(s, e);
  HostRow r = host_row(s, e, to, true);
  *count_out = r.present ? (int64_t)r.count : -1;
  write_row(ed, r, nullptr, payload_out, cap);
  API_END
}

int vg_num_edges(vg_sim *h, uint64_t to, int e, int64_t *out) {
  API_BEGIN
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (ed.singleedge())
    fail(VG_ERR_ASSERT, "num_edges is not defined for the hint combination of " + ed.name);
  require_readable_edge(s, e);
  HostRow r = host_row(s, e, to, false);
  *out = (int64_t)r.count;
  API_END
}

int vg_has_edge(vg_sim *h, uint64_t to, int e, int *out) {
  API_BEGIN
  Sim &s = S(h);
  require_readable_edge(s, e);
  HostRow r = host_row(s, e, to, false);
  *out = r.count > 0;
  API_END
}

int vg_num_edges_total(vg_sim *h, int e, int write, uint64_t *out) {
  API_BEGIN
  need(out, "output pointer");
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  if (es.implicit) {
    const Raster &R = s.rasters[es.st.raster];
    uint64_t t = 0;
    std::vector<uint64_t> lin;
    for (uint64_t c = 0; c < R.ncells; c++) {
      stencil_sources(s, es.st, c, lin);
      t += ed.bool_only() ? (lin.empty() ? 0 : 1) : lin.size();
    }
    *out = t;
    return VG_OK;
  }
  if (!s.initialized) {
    if (!write) { *out = 0; return VG_OK; }
    uint64_t t = 0;
    if (ed.bool_only()) {
      std::map<uint64_t, int> seen;
      for (auto &sg : es.staged) for (auto x : sg.h_to) seen[x] = 1;
      t = seen.size();
    } else {
      for (auto &sg : es.staged) t += sg.n;
    }
    *out = t;
    return VG_OK;
  }
  *out = csr_edges_total(es);
  API_END
}

int vg_read_edges(vg_sim *h, int e, int T, uint64_t *row_ptr_out, uint64_t *from_out,
                  void *const *payload_out, uint64_t *nrows_out, uint64_t *nedges_out) {
  API_BEGIN
  Sim &s = S(h);
  need(nrows_out, "row count pointer");
  need(nedges_out, "edge count pointer");
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  if (!s.initialized) fail(VG_ERR_STATE, "call finish_init! first");
  if (es.implicit) {
    const Raster &R = s.rasters[es.st.raster];
    std::vector<uint64_t> lin;
    uint64_t nrows = (T == R.type_nr) ? s.agents[T - 1].n : 0, ne = 0, k = 0;
    if (row_ptr_out) row_ptr_out[0] = 0;
    for (uint64_t r = 0; r < nrows; r++) {
      if (r + 1 >= R.first_nr && r + 1 < R.first_nr + R.ncells) {
        stencil_sources(s, es.st, r + 1 - R.first_nr, lin);
        for (auto l : lin) {
          if (from_out) from_out[k] = make_id(R.type_nr, R.first_nr + l);
          k++;
        }
        ne += lin.size();
      }
      if (row_ptr_out) row_ptr_out[r + 1] = ne;
    }
    *nrows_out = nrows;
    *nedges_out = ne;
    return VG_OK;
  }
  if (T < 1 || T >= (int)es.csr.size()) {
    *nrows_out = 0;
    *nedges_out = 0;
    if (row_ptr_out) row_ptr_out[0] = 0;
    return VG_OK;
  }
  CSR &c = es.csr[T];
  *nrows_out = c.nrows;
  *nedges_out = c.nedges;
  if (row_ptr_out) {
    std::vector<uint32_t> rp(c.nrows + 1, 0);
    if (c.row_ptr.p) VG_CUDA(cudaMemcpyAsync(rp.data(), c.row_ptr.p, rp.size() * 4, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    for (size_t i = 0; i < rp.size(); i++) row_ptr_out[i] = rp[i];
  }
  if (from_out && c.nedges) {
    std::vector<uint32_t> src(c.nedges, 0);
    std::vector<uint8_t> st(c.nedges, (uint8_t)std::max(c.src_type_const, 0));
    if (c.src.p) VG_CUDA(cudaMemcpyAsync(src.data(), c.src.p, c.nedges * 4, cudaMemcpyDeviceToHost, s.stream));
    if (c.src_type.p) VG_CUDA(cudaMemcpyAsync(st.data(), c.src_type.p, c.nedges, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    for (uint64_t k = 0; k < c.nedges; k++)
      from_out[k] = c.src.p ? make_id(st[k], (uint64_t)src[k] + 1) : 0;
  }
  if (payload_out && c.nedges)
    for (size_t f = 0; f < c.payload.size(); f++)
      if (payload_out[f])
        VG_CUDA(cudaMemcpyAsync(payload_out[f], c.payload[f].p, c.nedges * ed.fields[f].size,
                                cudaMemcpyDeviceToHost, s.stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
  API_END
}

}  // extern "C"

// ----------------------------------------------------------------- raster
namespace vg {

// stencil(metric, n, distance) -- src/Raster.jl:82-110: all offsets of
// Iterators.product((-d):d, ...) with the first dimension fastest, zero
// removed, filtered by the metric.
std::vector<int> make_stencil(int metric, int n, double distance) {
  int d = (int)std::floor(distance);
  std::vector<int> out;
  int side = 2 * d + 1;
  int64_t total = 1;
  for (int i = 0; i < n; i++) total *= side;
  for (int64_t lin = 0; lin < total; lin++) {
    int off[MAX_DIMS];
    int64_t t = lin;
    bool zero = true;
    double sq = 0;
    int l1 = 0;
    for (int i = 0; i < n; i++) {
      off[i] = (int)(t % side) - d;
      t /= side;
      if (off[i]) zero = false;
      sq += (double)off[i] * off[i];
      l1 += std::abs(off[i]);
    }
    if (zero) continue;
    if (metric == VG_METRIC_EUCLIDEAN && !(std::sqrt(sq) <= distance)) continue;
    if (metric == VG_METRIC_MANHATTEN && !(l1 <= distance)) continue;
    for (int i = 0; i < n; i++) out.push_back(off[i]);
  }
  return out;
}

// _checkpos -- src/Raster.jl:479-499 (1-based positions, mod1 wrap)
static bool checkpos(const int64_t *pos, const int64_t *dims, int n, int periodic,
                     int64_t *out) {
  bool oob = false;
  for (int i = 0; i < n; i++) {
    if (pos[i] < 1 || pos[i] > dims[i]) {
      oob = true;
      out[i] = ((pos[i] - 1) % dims[i] + dims[i]) % dims[i] + 1;
    } else {
      out[i] = pos[i];
    }
  }
  return !oob || periodic;
}

static uint64_t lin_of(const int64_t *pos, const int64_t *dims, int n) {
  uint64_t l = 0, m = 1;
  for (int i = 0; i < n; i++) {
    l += (uint64_t)(pos[i] - 1) * m;
    m *= dims[i];
  }
  return l;
}

// Sources of the implicit stencil edges into `cell` (0-based linear index),
// in insertion order: connect_raster_neighbors! iterates the source cells
// in column-major order and, for each, the stencil offsets in order.  The
// sources of one target are therefore ordered by (source index, offset).
void stencil_sources(const Sim &, const StencilDesc &st, uint64_t cell,
                     std::vector<uint64_t> &out) {
  out.clear();
  int n = st.ndims;
  int64_t tpos[MAX_DIMS];
  uint64_t t = cell;
  for (int i = 0; i < n; i++) {
    tpos[i] = (int64_t)(t % st.dims[i]) + 1;
    t /= st.dims[i];
  }
  std::vector<std::pair<uint64_t, int>> srcs;
  for (int k = 0; k < st.noff; k++) {
    // source org with checkpos(org + s) == target
    int64_t org[MAX_DIMS], chk[MAX_DIMS], sh[MAX_DIMS];
    bool ok = true;
    for (int i = 0; i < n; i++) {
      org[i] = tpos[i] - st.offsets[k * n + i];
      if (org[i] < 1 || org[i] > st.dims[i]) {
        if (!st.periodic) { ok = false; break; }
        org[i] = ((org[i] - 1) % st.dims[i] + st.dims[i]) % st.dims[i] + 1;
      }
    }
    if (!ok) continue;
    for (int i = 0; i < n; i++) sh[i] = org[i] + st.offsets[k * n + i];
    if (!checkpos(sh, st.dims, n, st.periodic, chk)) continue;
    bool same = true;
    for (int i = 0; i < n; i++) same &= chk[i] == tpos[i];
    if (!same) continue;
    srcs.push_back({lin_of(org, st.dims, n), k});
  }
  std::sort(srcs.begin(), srcs.end());
  for (auto &p : srcs) out.push_back(p.first);
}

}  // namespace vg

extern "C" {

int vg_add_raster(vg_sim *h, const char *name, int ndims, const int64_t *dims, int nr,
                  const void *const *fields, uint64_t *ids_out) {
  API_BEGIN
  Sim &s = S(h);
  if (s.initialized) fail(VG_ERR_ASSERT, "add_raster! can be only called before finish_init!");
  if (ndims < 1 || ndims > MAX_DIMS) fail(VG_ERR_ARG, "raster dimensions 1..4");
  if (s.raster_index(name) >= 0) fail(VG_ERR_ARG, std::string("raster exists: ") + name);
  Raster R;
  R.name = name;
  R.ndims = ndims;
  R.ncells = 1;
  for (int i = 0; i < ndims; i++) {
    R.dims[i] = dims[i];
    R.ncells *= (uint64_t)dims[i];
  }
  R.type_nr = nr;
  R.first_nr = s.agents[nr - 1].h_n + 1;
  std::vector<uint64_t> ids;
  if (ids_out == nullptr) ids.resize(R.ncells);
  int rc = vg_add_agents(h, nr, R.ncells, fields, ids_out ? ids_out : ids.data());
  if (rc) return rc;
  s.rasters.push_back(R);
  API_END
}

int vg_connect_raster_neighbors(vg_sim *h, const char *name, int e,
                                const void *const *payload, double distance, int metric,
                                int periodic, int implicit) {
  API_BEGIN
  Sim &s = S(h);
  int ri = s.raster_index(name);
  if (ri < 0) fail(VG_ERR_ARG, std::string("unknown raster ") + name);
  const Raster &R = s.rasters[ri];
  const EdgeTypeDesc &ed = s.model->et(e);
  StencilDesc st;
  st.raster = ri;
  st.ndims = R.ndims;
  for (int i = 0; i < R.ndims; i++) st.dims[i] = R.dims[i];
  st.offsets = make_stencil(metric, R.ndims, distance);
  st.noff = (int)(st.offsets.size() / R.ndims);
  st.periodic = periodic;
  st.target_type = R.type_nr;
  size_t psz = 0;
  for (auto &f : ed.fields) psz += f.size;
  st.payload.resize(psz);
  if (ed.stores_payload()) {
    size_t off = 0;
    for (size_t f = 0; f < ed.fields.size(); f++) {
      if (payload && payload[f]) std::memcpy(st.payload.data() + off, payload[f], ed.fields[f].size);
      off += ed.fields[f].size;
    }
  }
  EdgeStore &es = s.edges[e];
  if (implicit) {
    if (es.nstaged || csr_edges_total(es))
      fail(VG_ERR_ARG, "implicit raster edges need an edge type without other edges");
    es.implicit = true;
    es.st = st;
    return VG_OK;
  }
  // explicit: emit org -> shifted for org in column-major order, offsets in order
  std::vector<uint64_t> from, to;
  std::vector<std::vector<uint8_t>> pl(ed.stores_payload() ? ed.fields.size() : 0);
  int n = R.ndims;
  for (uint64_t c = 0; c < R.ncells; c++) {
    int64_t org[MAX_DIMS], p[MAX_DIMS], sh[MAX_DIMS];
    uint64_t t = c;
    for (int i = 0; i < n; i++) { org[i] = (int64_t)(t % R.dims[i]) + 1; t /= R.dims[i]; }
    for (int k = 0; k < st.noff; k++) {
      for (int i = 0; i < n; i++) p[i] = org[i] + st.offsets[k * n + i];
      if (!checkpos(p, R.dims, n, periodic, sh)) continue;
      from.push_back(make_id(R.type_nr, R.first_nr + c));
      to.push_back(make_id(R.type_nr, R.first_nr + lin_of(sh, R.dims, n)));
      size_t off = 0;
      for (size_t f = 0; f < pl.size(); f++) {
        pl[f].insert(pl[f].end(), st.payload.begin() + off, st.payload.begin() + off + ed.fields[f].size);
        off += ed.fields[f].size;
      }
    }
  }
  std::vector<const void *> pp;
  for (auto &v : pl) pp.push_back(v.data());
  bool was_in = s.intransition;
  if (s.initialized) s.intransition = true;
  bool chk = s.check_readable;
  s.check_readable = false;
  int rc = vg_add_edges(h, e, from.size(), from.data(), to.data(), pp.empty() ? nullptr : pp.data());
  s.intransition = was_in;
  s.check_readable = chk;
  if (rc) return rc;
  API_END
}

int vg_move_to(vg_sim *h, const char *name, uint64_t id, const int64_t *pos, int efrom,
               const void *const *pfrom, int eto, const void *const *pto, double distance,
               int metric, int periodic, int only_surrounding) {
  API_BEGIN
  Sim &s = S(h);
  int ri = s.raster_index(name);
  if (ri < 0) fail(VG_ERR_ARG, std::string("unknown raster ") + name);
  const Raster &R = s.rasters[ri];
  int n = R.ndims;
  need(pos, "position");
  auto cell = [&](const int64_t *p) { return make_id(R.type_nr, R.first_nr + lin_of(p, R.dims, n)); };
  auto add = [&](int e, uint64_t f, uint64_t t, const void *const *pl) {
    int rc = vg_add_edges(h, e, 1, &f, &t, pl);
    if (rc) fail(rc, vg_last_error());
  };
  if (!only_surrounding) {
    if (efrom >= 0) add(efrom, cell(pos), id, pfrom);
    if (eto >= 0) add(eto, id, cell(pos), pto);
  }
  if (distance >= 1) {
    auto off = make_stencil(metric, n, distance);
    int noff = (int)(off.size() / n);
    for (int k = 0; k < noff; k++) {
      int64_t p[MAX_DIMS], sh[MAX_DIMS];
      for (int i = 0; i < n; i++) p[i] = pos[i] + off[k * n + i];
      if (!checkpos(p, R.dims, n, periodic, sh)) continue;
      if (efrom >= 0) add(efrom, cell(sh), id, pfrom);
      if (eto >= 0) add(eto, id, cell(sh), pto);
    }
  }
  API_END
}

int vg_cellid(vg_sim *h, const char *name, const int64_t *pos, uint64_t *out) {
  API_BEGIN
  Sim &s = S(h);
  int ri = s.raster_index(name);
  if (ri < 0) fail(VG_ERR_ARG, std::string("unknown raster ") + name);
  const Raster &R = s.rasters[ri];
  need(pos, "position");
  for (int i = 0; i < R.ndims; i++)
    if (pos[i] < 1 || pos[i] > R.dims[i]) fail(VG_ERR_ARG, "position outside the raster");
  *need(out, "output pointer") = make_id(R.type_nr, R.first_nr + lin_of(pos, R.dims, R.ndims));
  API_END
}

int vg_raster_dims(vg_sim *h, const char *name, int64_t *dims_out, int *ndims_out) {
  API_BEGIN
  Sim &s = S(h);
  int ri = s.raster_index(name);
  if (ri < 0) fail(VG_ERR_ARG, std::string("unknown raster ") + name);
  const Raster &R = s.rasters[ri];
  *need(ndims_out, "dimension count pointer") = R.ndims;
  if (dims_out)
    for (int i = 0; i < R.ndims; i++) dims_out[i] = R.dims[i];
  API_END
}

int vg_rastervalues(vg_sim *h, const char *name, int field, void *out) {
  API_BEGIN
  Sim &s = S(h);
  int ri = s.raster_index(name);
  if (ri < 0) fail(VG_ERR_ARG, std::string("unknown raster ") + name);
  if (!s.initialized) fail(VG_ERR_ASSERT, "rastervalues can be only called after finish_init!");
  const Raster &R = s.rasters[ri];
  const AgentTypeDesc &ad = s.model->at(R.type_nr);
  if (field < 0 || field >= (int)ad.fields.size()) fail(VG_ERR_ARG, "bad field");
  size_t sz = ad.fields[field].size;
  AgentStore &a = s.agents[R.type_nr - 1];
  VG_CUDA(cudaMemcpyAsync(out, a.rd[field].as<uint8_t>() + (R.first_nr - 1) * sz, R.ncells * sz,
                          cudaMemcpyDeviceToHost, s.stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
  API_END
}

}  // extern "C"
