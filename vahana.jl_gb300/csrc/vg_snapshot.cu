// Checkpoint and restore of an initialized simulation: everything apply!
// and the accessors read -- per agent type the read state, died flags, the
// LIFO reuse stack and nextid; per edge type the CSR of every target type
// (or the implicit raster stencil); rasters, params, globals and
// num_transitions -- in one little-endian binary file with a fingerprint of
// the model, checked on load.  Write buffers are scratch between
// transitions and restored as copies of the read state; derived gather
// layouts are rebuilt on first use.
//
// The reference's write_snapshot / read_snapshot! (src/HDF5.jl:688-715,
// 1594-1660) store the same information in HDF5 files; this file format is
// the library's own.
#include <cstdio>
#include <cstring>
#include <memory>

#include "vg_internal.h"

namespace vg {
void set_last_error(const std::string &m);
}  // namespace vg

using namespace vg;

namespace {

constexpr char MAGIC[8] = {'V', 'G', 'S', 'N', 'A', 'P', '0', '1'};

Sim &S(vg_sim *h) {
  if (!h || !h->s) fail(VG_ERR_ARG, "null simulation");
  return *h->s;
}

struct File {
  FILE *f = nullptr;
  std::string path;
  File(const char *p, const char *mode) : path(p) {
    f = std::fopen(p, mode);
    if (!f) fail(VG_ERR_ARG, std::string("cannot open ") + p);
  }
  ~File() {
    if (f) std::fclose(f);
  }
  void put(const void *p, size_t n) {
    if (n && std::fwrite(p, 1, n, f) != n) fail(VG_ERR_ARG, "write failed: " + path);
  }
  void get(void *p, size_t n) {
    if (n && std::fread(p, 1, n, f) != n) fail(VG_ERR_ARG, "truncated snapshot: " + path);
  }
  template <class T> void put(const T &v) { put(&v, sizeof(T)); }
  template <class T> T get() {
    T v;
    get(&v, sizeof(T));
    return v;
  }
  void put_str(const std::string &s) {
    put<uint64_t>(s.size());
    put(s.data(), s.size());
  }
  std::string get_str() {
    uint64_t n = get<uint64_t>();
    if (n > (1u << 20)) fail(VG_ERR_ARG, "corrupt snapshot: " + path);
    std::string s(n, '\0');
    get(&s[0], n);
    return s;
  }
};

// the model as text: type names, fields, dtypes, hints, targets, in order
std::string fingerprint(const Model &m) {
  std::string r = m.name + "|";
  for (auto &a : m.atypes) {
    r += "A:" + a.name + ":" + std::to_string(a.hints);
    for (auto &f : a.fields) r += "," + f.name + "/" + std::to_string(f.dtype);
    r += ";";
  }
  for (auto &e : m.etypes) {
    r += "E:" + e.name + ":" + std::to_string(e.hints) + ":" + std::to_string(e.target);
    for (auto &f : e.fields) r += "," + f.name + "/" + std::to_string(f.dtype);
    r += ";";
  }
  return r;
}

void put_dev(File &F, const DevBuf &b, uint64_t bytes, cudaStream_t st) {
  F.put<uint64_t>(bytes);
  if (!bytes) return;
  std::vector<uint8_t> h(bytes);
  VG_CUDA(cudaMemcpyAsync(h.data(), b.p, bytes, cudaMemcpyDeviceToHost, st));
  VG_CUDA(cudaStreamSynchronize(st));
  F.put(h.data(), bytes);
}

// reads a device column written by put_dev into b (allocated with at least
// `cap` bytes)
void get_dev(File &F, DevBuf &b, uint64_t cap, Sim &s) {
  uint64_t bytes = F.get<uint64_t>();
  if (bytes > cap) fail(VG_ERR_ARG, "corrupt snapshot column");
  if (!b.p) b.alloc(std::max<uint64_t>(cap, 1), &s.footprint);
  if (!bytes) return;
  std::vector<uint8_t> h(bytes);
  F.get(h.data(), bytes);
  VG_CUDA(cudaMemcpyAsync(b.p, h.data(), bytes, cudaMemcpyHostToDevice, s.stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
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

int vg_sim_save(vg_sim *h, const char *path) {
  API_BEGIN
  Sim &s = S(h);
  if (!s.initialized) fail(VG_ERR_STATE, "save: call finish_init! first");
  if (s.intransition) fail(VG_ERR_STATE, "save: not inside a transition");
  for (auto &es : s.edges)
    if (es.nstaged) fail(VG_ERR_STATE, "save: edges staged but not yet built");
  s.ensure_device();
  VG_CUDA(cudaStreamSynchronize(s.stream));
  File F(path, "wb");
  F.put(MAGIC, 8);
  F.put_str(fingerprint(*s.model));
  F.put_str(s.name);
  F.put<int64_t>(s.num_transitions);
  F.put<uint8_t>(s.check_readable ? 1 : 0);
  F.put<uint64_t>(s.params.size());
  for (auto &kv : s.params) {
    F.put_str(kv.first);
    F.put<double>(kv.second);
  }
  F.put<uint64_t>(s.globals.size());
  for (auto &kv : s.globals) {
    F.put_str(kv.first);
    F.put<double>(kv.second);
  }
  F.put<uint64_t>(s.global_series.size());
  for (auto &kv : s.global_series) {
    F.put_str(kv.first);
    F.put<uint64_t>(kv.second.size());
    F.put(kv.second.data(), kv.second.size() * 8);
  }
  F.put<uint64_t>(s.rasters.size());
  for (auto &r : s.rasters) {
    F.put_str(r.name);
    F.put<int32_t>(r.ndims);
    F.put(r.dims, sizeof(r.dims));
    F.put<int32_t>(r.type_nr);
    F.put<uint64_t>(r.first_nr);
    F.put<uint64_t>(r.ncells);
  }
  for (size_t t = 0; t < s.agents.size(); t++) {
    AgentStore &a = s.agents[t];
    const AgentTypeDesc &ad = s.model->at((int)t + 1);
    F.put<uint64_t>(a.n);
    F.put<uint64_t>(a.nreuse);
    F.put<uint64_t>(a.nliving);
    if (a.n && a.rd.size() < ad.fields.size()) fail(VG_ERR_STATE, "save: agent columns missing");
    for (size_t f = 0; f < ad.fields.size(); f++) {
      if (a.n) put_dev(F, a.rd[f], a.n * ad.fields[f].size, s.stream);
      else F.put<uint64_t>(0);
    }
    if (!ad.immortal()) {
      put_dev(F, a.died_rd, a.n, s.stream);
      put_dev(F, a.reuse, a.nreuse * 8, s.stream);
    }
  }
  for (size_t e = 0; e < s.edges.size(); e++) {
    EdgeStore &es = s.edges[e];
    const EdgeTypeDesc &ed = s.model->et((int)e);
    F.put<uint8_t>(es.implicit ? 1 : 0);
    if (es.implicit) {
      const StencilDesc &sd = es.st;
      F.put<int32_t>(sd.raster);
      F.put<int32_t>(sd.ndims);
      F.put(sd.dims, sizeof(sd.dims));
      F.put<int32_t>(sd.noff);
      F.put<uint64_t>(sd.offsets.size());
      F.put(sd.offsets.data(), sd.offsets.size() * sizeof(int));
      F.put<int32_t>(sd.periodic);
      F.put<int32_t>(sd.target_type);
      F.put<uint64_t>(sd.payload.size());
      F.put(sd.payload.data(), sd.payload.size());
      continue;
    }
    F.put<uint64_t>(es.csr.size());
    for (size_t T = 0; T < es.csr.size(); T++) {
      CSR &c = es.csr[T];
      const bool present = c.row_ptr.p != nullptr;
      F.put<uint8_t>(present ? 1 : 0);
      if (!present) continue;
      F.put<uint64_t>(c.nrows);
      F.put<uint64_t>(c.nedges);
      F.put<int32_t>(c.src_type_const);
      F.put<uint32_t>(csr_max_degree(s, c));
      put_dev(F, c.row_ptr, (c.nrows + 1) * 4, s.stream);
      put_dev(F, c.src, c.src.p ? c.nedges * 4 : 0, s.stream);
      put_dev(F, c.src_type, c.src_type.p ? c.nedges : 0, s.stream);
      F.put<uint64_t>(c.payload.size());
      for (size_t f = 0; f < c.payload.size(); f++)
        put_dev(F, c.payload[f], c.nedges * ed.fields[f].size, s.stream);
    }
  }
  API_END
}

int vg_sim_load(vg_model *m, const char *path, void *stream, vg_sim **out) {
  API_BEGIN
  if (!m || !m->m || !m->m->finalized) fail(VG_ERR_ARG, "load: finalized model required");
  if (!path || !out) fail(VG_ERR_ARG, "load: null path or output pointer");
  File F(path, "rb");
  char magic[8];
  F.get(magic, 8);
  if (std::memcmp(magic, MAGIC, 8) != 0) fail(VG_ERR_ARG, "not a simulation snapshot");
  if (F.get_str() != fingerprint(*m->m))
    fail(VG_ERR_ASSERT, "the snapshot was written for a different model");
  vg_sim *h = nullptr;
  int rc = vg_sim_create(m, F.get_str().c_str(), stream, &h);
  if (rc) fail(rc, vg_last_error());
  std::unique_ptr<vg_sim, int (*)(vg_sim *)> guard(h, vg_sim_destroy);
  Sim &s = S(h);
  s.ensure_device();
  s.num_transitions = F.get<int64_t>();
  s.check_readable = F.get<uint8_t>() != 0;
  for (uint64_t k = F.get<uint64_t>(); k--;) {
    std::string n = F.get_str();
    s.params[n] = F.get<double>();
  }
  for (uint64_t k = F.get<uint64_t>(); k--;) {
    std::string n = F.get_str();
    s.globals[n] = F.get<double>();
  }
  for (uint64_t k = F.get<uint64_t>(); k--;) {
    std::string n = F.get_str();
    uint64_t len = F.get<uint64_t>();
    if (len > (1ull << 32)) fail(VG_ERR_ARG, "corrupt snapshot");
    std::vector<double> v(len);
    F.get(v.data(), len * 8);
    s.global_series[n] = std::move(v);
  }
  s.rasters.clear();
  for (uint64_t k = F.get<uint64_t>(); k--;) {
    Raster r;
    r.name = F.get_str();
    r.ndims = F.get<int32_t>();
    F.get(r.dims, sizeof(r.dims));
    r.type_nr = F.get<int32_t>();
    r.first_nr = F.get<uint64_t>();
    r.ncells = F.get<uint64_t>();
    s.rasters.push_back(r);
  }
  for (size_t t = 0; t < s.agents.size(); t++) {
    AgentStore &a = s.agents[t];
    const int nr = (int)t + 1;
    const AgentTypeDesc &ad = s.model->at(nr);
    const uint64_t n = F.get<uint64_t>();
    const uint64_t nreuse = F.get<uint64_t>();
    const uint64_t nliving = F.get<uint64_t>();
    if (n > (1ull << 36) || nreuse > n || nliving > n) fail(VG_ERR_ARG, "corrupt snapshot");
    agent_reserve(s, nr, std::max<uint64_t>(n, 1));
    for (size_t f = 0; f < ad.fields.size(); f++) {
      const uint64_t sz = ad.fields[f].size;
      get_dev(F, a.rd[f], a.cap * sz, s);
      if (n)
        VG_CUDA(cudaMemcpyAsync(a.wr[f].p, a.rd[f].p, n * sz, cudaMemcpyDeviceToDevice, s.stream));
    }
    if (!ad.immortal()) {
      get_dev(F, a.died_rd, a.cap, s);
      if (n)
        VG_CUDA(cudaMemcpyAsync(a.died_wr.p, a.died_rd.p, n, cudaMemcpyDeviceToDevice, s.stream));
      a.reuse_cap = std::max<uint64_t>(nreuse, 1);
      a.reuse.release();
      get_dev(F, a.reuse, a.reuse_cap * 8, s);
    }
    a.n = n;
    a.nreuse = nreuse;
    a.nliving = nliving;
  }
  for (size_t e = 0; e < s.edges.size(); e++) {
    EdgeStore &es = s.edges[e];
    const EdgeTypeDesc &ed = s.model->et((int)e);
    es.implicit = F.get<uint8_t>() != 0;
    es.staged.clear();
    es.nstaged = 0;
    if (es.implicit) {
      StencilDesc &sd = es.st;
      sd.raster = F.get<int32_t>();
      sd.ndims = F.get<int32_t>();
      F.get(sd.dims, sizeof(sd.dims));
      sd.noff = F.get<int32_t>();
      uint64_t no = F.get<uint64_t>();
      if (no > (1u << 20)) fail(VG_ERR_ARG, "corrupt snapshot");
      sd.offsets.resize(no);
      F.get(sd.offsets.data(), no * sizeof(int));
      sd.periodic = F.get<int32_t>();
      sd.target_type = F.get<int32_t>();
      uint64_t np = F.get<uint64_t>();
      if (np > 4096) fail(VG_ERR_ARG, "corrupt snapshot");
      sd.payload.resize(np);
      F.get(sd.payload.data(), np);
      continue;
    }
    const uint64_t ncsr = F.get<uint64_t>();
    if (ncsr > MAX_AGENT_TYPES) fail(VG_ERR_ARG, "corrupt snapshot");
    s.csr_epoch++;
    es.csr.clear();
    es.csr.resize(ncsr);
    for (uint64_t T = 0; T < ncsr; T++) {
      if (!F.get<uint8_t>()) continue;
      CSR &c = es.csr[T];
      c.nrows = F.get<uint64_t>();
      c.nedges = F.get<uint64_t>();
      c.src_type_const = F.get<int32_t>();
      c.max_degree = F.get<uint32_t>();
      if (c.nrows > (1ull << 36) || c.nedges >= (1ull << 32)) fail(VG_ERR_ARG, "corrupt snapshot");
      get_dev(F, c.row_ptr, (c.nrows + 1) * 4, s);
      // source columns exist only when they were written
      {
        uint64_t bytes = F.get<uint64_t>();
        if (bytes) {
          if (bytes != c.nedges * 4) fail(VG_ERR_ARG, "corrupt snapshot");
          c.src.alloc(std::max<uint64_t>(c.nedges, 1) * 4, &s.footprint);
          std::vector<uint8_t> hb(bytes);
          F.get(hb.data(), bytes);
          VG_CUDA(cudaMemcpy(c.src.p, hb.data(), bytes, cudaMemcpyHostToDevice));
        }
        bytes = F.get<uint64_t>();
        if (bytes) {
          if (bytes != c.nedges) fail(VG_ERR_ARG, "corrupt snapshot");
          c.src_type.alloc(std::max<uint64_t>(c.nedges, 1), &s.footprint);
          std::vector<uint8_t> hb(bytes);
          F.get(hb.data(), bytes);
          VG_CUDA(cudaMemcpy(c.src_type.p, hb.data(), bytes, cudaMemcpyHostToDevice));
        }
      }
      const uint64_t npl = F.get<uint64_t>();
      if (npl != (ed.stores_payload() ? ed.fields.size() : 0)) fail(VG_ERR_ARG, "corrupt snapshot");
      c.payload.resize(npl);
      for (uint64_t f = 0; f < npl; f++)
        get_dev(F, c.payload[f], std::max<uint64_t>(c.nedges, 1) * ed.fields[f].size, s);
    }
  }
  s.initialized = true;
  VG_CUDA(cudaStreamSynchronize(s.stream));
  *out = guard.release();
  API_END
}

}  // extern "C"
