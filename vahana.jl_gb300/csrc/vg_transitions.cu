// Transition kernels bound by name (the `f` of apply!, src/Simulation.jl:
// 720-821).  Every kernel sweeps the agents of the called type in index
// order semantics (transition_with_read!, src/AgentMethods.jl:193-207):
// died agents are skipped, a returned state is written to the write buffer
// (transition_with_write!, :159-181) and `nothing` marks the agent died.
//
// Floating-point arithmetic on the ordered paths uses explicitly rounded
// intrinsics (__dadd_rn, __dmul_rn, __ddiv_rn) in the reference's
// left-to-right order, so results are bit-identical to the sequential CPU
// fold (the library is also compiled with -fmad=false).
#include <algorithm>
#include <cstring>
#include <vector>

#include "vg_internal.h"
#include "vg_philox.cuh"

namespace vg {

namespace {

constexpr int TPB = 256;
inline unsigned nblk(uint64_t n, int tpb = TPB) {
  uint64_t b = (n + tpb - 1) / tpb;
  return (unsigned)std::max<uint64_t>(b, 1);
}

__device__ __forceinline__ void set_status(int *st, int code) {
  atomicCAS(st, 0, code);
}

// ----------------------------------------------------------- field access
__device__ __forceinline__ int64_t ld_i64(const void *p, int dt, uint64_t i) {
  switch (dt) {
    case VG_BOOL: case VG_U8: return ((const uint8_t *)p)[i];
    case VG_I8: return ((const int8_t *)p)[i];
    case VG_U16: return ((const uint16_t *)p)[i];
    case VG_I16: return ((const int16_t *)p)[i];
    case VG_U32: return ((const uint32_t *)p)[i];
    case VG_I32: return ((const int32_t *)p)[i];
    case VG_U64: case VG_I64: return ((const int64_t *)p)[i];
    case VG_F32: return (int64_t)((const float *)p)[i];
    case VG_F64: return (int64_t)((const double *)p)[i];
  }
  return 0;
}
__device__ __forceinline__ double ld_f64(const void *p, int dt, uint64_t i) {
  switch (dt) {
    case VG_F32: return (double)((const float *)p)[i];
    case VG_F64: return ((const double *)p)[i];
    case VG_U64: return (double)((const uint64_t *)p)[i];
  }
  return (double)ld_i64(p, dt, i);
}
__device__ __forceinline__ void st_i64(void *p, int dt, uint64_t i, int64_t v) {
  switch (dt) {
    case VG_BOOL: ((uint8_t *)p)[i] = v != 0; break;
    case VG_U8: case VG_I8: ((uint8_t *)p)[i] = (uint8_t)v; break;
    case VG_U16: case VG_I16: ((uint16_t *)p)[i] = (uint16_t)v; break;
    case VG_U32: case VG_I32: ((uint32_t *)p)[i] = (uint32_t)v; break;
    case VG_U64: case VG_I64: ((int64_t *)p)[i] = v; break;
    case VG_F32: ((float *)p)[i] = (float)v; break;
    case VG_F64: ((double *)p)[i] = (double)v; break;
  }
}
__device__ __forceinline__ void st_f64(void *p, int dt, uint64_t i, double v) {
  switch (dt) {
    case VG_F32: ((float *)p)[i] = (float)v; break;
    case VG_F64: ((double *)p)[i] = v; break;
    default: st_i64(p, dt, i, (int64_t)v);
  }
}
__device__ __forceinline__ bool is_float(int dt) { return dt == VG_F32 || dt == VG_F64; }

// ------------------------------------------------------------ sweep frame
struct Sweep {
  DevAgentView a;
  int nfields;
  int fsize[MAX_FIELDS];
  int fdt[MAX_FIELDS];
  int mortal;
  int writes;              // the called type is in `write`
  const uint32_t *with_rp; // with_edge: row_ptr of that edge type, or null
  uint64_t with_nrows;
  int type_nr;
  int *status;
};

__device__ void sw_copy(const Sweep &s, uint64_t i) {
  for (int f = 0; f < s.nfields; f++) {
    switch (s.fsize[f]) {
      case 1: ((uint8_t *)s.a.wr[f])[i] = ((const uint8_t *)s.a.rd[f])[i]; break;
      case 2: ((uint16_t *)s.a.wr[f])[i] = ((const uint16_t *)s.a.rd[f])[i]; break;
      case 4: ((uint32_t *)s.a.wr[f])[i] = ((const uint32_t *)s.a.rd[f])[i]; break;
      case 8: ((uint64_t *)s.a.wr[f])[i] = ((const uint64_t *)s.a.rd[f])[i]; break;
    }
  }
  if (s.mortal) s.a.died_wr[i] = 0;
}

// Returns true when agent i is swept.  Died agents stay died; with_edge
// restricts the sweep to targets of that edge type (src/AgentMethods.jl:
// 209-229), the others keep their state.
__device__ __forceinline__ bool sw_begin(const Sweep &s, uint64_t i) {
  if (s.mortal && s.a.died_rd[i]) {
    if (s.writes) s.a.died_wr[i] = 1;
    return false;
  }
  if (s.with_rp) {
    bool has = i < s.with_nrows && s.with_rp[i + 1] > s.with_rp[i];
    if (!has) {
      if (s.writes) sw_copy(s, i);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void sw_die(const Sweep &s, uint64_t i) {
  if (!s.mortal) {
    set_status(s.status, 201);  // `nothing` returned for an immortal agent
    sw_copy(s, i);
    return;
  }
  s.a.died_wr[i] = 1;
}

// source field of every agent type (flexible neighbour states)
struct SrcTable {
  const void *ptr[MAX_AGENT_TYPES];
  int dt[MAX_AGENT_TYPES];
  const uint8_t *died[MAX_AGENT_TYPES];
};

__device__ __forceinline__ int edge_src_type(const DevCSRView &c, uint64_t k) {
  return c.src_type ? (int)c.src_type[k] : c.src_type_const;
}

// --------------------------------------------------- generic neighbour ops
// mode 0: dst = sum of the neighbours' field (neighbor_sum)
// mode 1: dst = own dst || any neighbour field != 0 (neighbor_or)
// mode 2: dst = number of edges (count_edges)
__global__ void k_neighbor_op(Sweep s, DevCSRView c, SrcTable t, int dst,
                              int mode) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.a.n || !sw_begin(s, i)) return;
  int ddt = s.fdt[dst];
  int64_t si = 0;
  double sf = 0.0;
  bool anyv = false;
  uint32_t b = 0, e = 0;
  if (i < c.nrows) {
    b = c.row_ptr[i];
    e = c.row_ptr[i + 1];
  }
  for (uint32_t k = b; k < e && mode != 2; k++) {
    int ty = edge_src_type(c, k);
    uint32_t j = c.src[k];
    if (ty <= 0 || ty >= MAX_AGENT_TYPES || !t.ptr[ty]) {
      set_status(s.status, 202);  // source type not readable
      continue;
    }
    if (t.died[ty] && t.died[ty][j]) set_status(s.status, 203);
    if (mode == 0) {
      if (is_float(ddt)) sf = __dadd_rn(sf, ld_f64(t.ptr[ty], t.dt[ty], j));
      else si = (int64_t)((uint64_t)si + (uint64_t)ld_i64(t.ptr[ty], t.dt[ty], j));
    } else {
      anyv |= ld_i64(t.ptr[ty], t.dt[ty], j) != 0;
    }
  }
  if (!s.writes) return;
  sw_copy(s, i);
  if (mode == 0) {
    if (is_float(ddt)) st_f64(s.a.wr[dst], ddt, i, sf);
    else st_i64(s.a.wr[dst], ddt, i, si);
  } else if (mode == 1) {
    bool own = ld_i64(s.a.rd[dst], ddt, i) != 0;
    st_i64(s.a.wr[dst], ddt, i, (own || anyv) ? 1 : 0);
  } else {
    st_i64(s.a.wr[dst], ddt, i, (int64_t)(e - b));
  }
}

// die_if: kind 0 always; 1 field >= arg; 2 field % arg != 0; 3 the agent has
// no edge of the given edge type (num_edges == 0)
__global__ void k_die_if(Sweep s, int kind, int field, double arg,
                         const uint32_t *rp2, uint64_t nrows2) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.a.n || !sw_begin(s, i)) return;
  bool die = false;
  if (kind == 0) die = true;
  else if (kind == 1) die = ld_f64(s.a.rd[field], s.fdt[field], i) >= arg;
  else if (kind == 2) die = (ld_i64(s.a.rd[field], s.fdt[field], i) % (int64_t)arg) != 0;
  else if (kind == 3) die = !(rp2 && i < nrows2 && rp2[i + 1] > rp2[i]);
  if (!s.writes) return;
  if (die) sw_die(s, i);
  else sw_copy(s, i);
}

// set_field: kind 0 constant; 1 (agent id mod 2 == 1)
__global__ void k_set_field(Sweep s, int field, int kind, double value) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.a.n || !sw_begin(s, i)) return;
  if (!s.writes) return;
  sw_copy(s, i);
  int dt = s.fdt[field];
  if (kind == 0) {
    if (is_float(dt)) st_f64(s.a.wr[field], dt, i, value);
    else st_i64(s.a.wr[field], dt, i, (int64_t)value);
  } else {
    uint64_t id = ((uint64_t)s.type_nr << SHIFT_TYPE) | (i + 1);
    st_i64(s.a.wr[field], dt, i, (id % 2) == 1 ? 1 : 0);
  }
}

__global__ void k_keep(Sweep s) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.a.n || !sw_begin(s, i)) return;
  if (s.writes) sw_copy(s, i);
}

// edge appends with an order key (call position, caller index, sequence):
// the order in which the reference's sequential sweep calls add_edge!.
struct Append {
  uint64_t *to, *from, *key;
  void *payload[MAX_FIELDS];
  int psize[MAX_FIELDS];
  int npayload;
  unsigned long long *counter;
  uint64_t cap;
};

__device__ __forceinline__ uint64_t order_key(int call_pos, uint64_t i,
                                              uint32_t seq) {
  return ((uint64_t)call_pos << 60) | ((i & ((1ull << 40) - 1)) << 20) | seq;
}

// Slots of the append and removal buffers are reserved per warp: the lanes
// that add a record in this round vote, the lowest of them reserves all of
// the warp's slots with one atomicAdd on the buffer's counter, and each lane
// takes the next slot by its rank among the voters.  Every lane of the warp
// must call it (full mask; lanes with nothing to add pass want = false).
// The slot is only a place in the buffer: the record's order key decides its
// position in the rebuilt container.  -1: nothing wanted, or the buffer is
// full (err is recorded in the status word).
constexpr unsigned FULL_WARP = 0xffffffffu;

__device__ __forceinline__ int64_t warp_slot(unsigned long long *counter, uint64_t cap, bool want,
                                             int *status, int err) {
  const unsigned voters = __ballot_sync(FULL_WARP, want);
  if (!voters) return -1;
  const unsigned lane = threadIdx.x & 31;
  const int leader = __ffs(voters) - 1;
  unsigned long long base = 0;
  if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(voters));
  base = __shfl_sync(FULL_WARP, base, leader);
  if (!want) return -1;
  const unsigned long long k = base + __popc(voters & ((1u << lane) - 1u));
  if (k >= cap) {
    set_status(status, err);
    return -1;
  }
  return (int64_t)k;
}

// add_edge!(sim, id, id, state) for every swept agent
__global__ void k_self_edge(Sweep s, Append ap, int call_pos, const uint8_t *pl) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < s.a.n && sw_begin(s, i);
  if (live && s.writes) sw_copy(s, i);
  const int64_t k = warp_slot(ap.counter, ap.cap, live, s.status, 301);
  if (k < 0) return;
  uint64_t id = ((uint64_t)s.type_nr << SHIFT_TYPE) | (i + 1);
  ap.to[k] = id;
  ap.from[k] = id;
  ap.key[k] = order_key(call_pos, i, 0);
  int off = 0;
  for (int f = 0; f < ap.npayload; f++) {
    for (int b = 0; b < ap.psize[f]; b++)
      ((uint8_t *)ap.payload[f])[k * ap.psize[f] + b] = pl[off + b];
    off += ap.psize[f];
  }
}

// add_edges!(sim, id, edges(sim, id, ET)): re-add every in-edge of the agent
// (round q: the q-th in-edge of every lane that has one)
__global__ void k_readd_edges(Sweep s, DevCSRView c, Append ap, int call_pos) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < s.a.n && sw_begin(s, i);
  if (live && s.writes) sw_copy(s, i);
  const bool rows = live && i < c.nrows;
  const uint32_t b = rows ? c.row_ptr[i] : 0u;
  const uint32_t deg = rows ? c.row_ptr[i + 1] - b : 0u;
  const uint64_t id = ((uint64_t)s.type_nr << SHIFT_TYPE) | (i + 1);
  for (uint32_t q = 0; __any_sync(FULL_WARP, q < deg); q++) {
    const int64_t k = warp_slot(ap.counter, ap.cap, q < deg, s.status, 301);
    if (k < 0) continue;
    const uint32_t e = b + q;
    ap.to[k] = id;
    ap.from[k] = ((uint64_t)edge_src_type(c, e) << SHIFT_TYPE) | ((uint64_t)c.src[e] + 1);
    ap.key[k] = order_key(call_pos, i, q);
    for (int f = 0; f < ap.npayload; f++) {
      int sz = ap.psize[f];
      for (int bb = 0; bb < sz; bb++)
        ((uint8_t *)ap.payload[f])[k * sz + bb] = ((const uint8_t *)c.payload[f])[(uint64_t)e * sz + bb];
    }
  }
}

// remove_edges!: a swept agent keeps its state; mode 0: when its field 0
// passes the test (kind 0 always, 1 field >= arg, 2 field % arg != 0) it
// calls remove_edges!(sim, id, E); mode 1: for every source nid of its
// in-edges of E (read container, insertion order) whose field 0 passes the
// test it calls remove_edges!(sim, nid, id, E).
struct Removal {
  uint64_t *to, *from, *key;
  unsigned long long *counter;
  uint64_t cap;
};

__device__ __forceinline__ bool field_test(int kind, double arg, const void *p, int dt,
                                           uint64_t i) {
  if (kind == 0) return true;
  if (kind == 1) return ld_f64(p, dt, i) >= arg;
  return (ld_i64(p, dt, i) % (int64_t)arg) != 0;
}

// one removal record per lane with want (every lane of the warp calls it)
__device__ __forceinline__ void push_removal(const Removal &r, bool want, uint64_t to,
                                             uint64_t from, uint64_t key, int *status) {
  const int64_t k = warp_slot(r.counter, r.cap, want, status, 302);
  if (k < 0) return;
  r.to[k] = to;
  r.from[k] = from;
  r.key[k] = key;
}

__global__ void k_remove_edges(Sweep s, DevCSRView c, SrcTable t, int kind, double arg, int mode,
                               Removal rm, int call_pos) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < s.a.n && sw_begin(s, i);
  if (live && s.writes) sw_copy(s, i);
  const uint64_t id = ((uint64_t)s.type_nr << SHIFT_TYPE) | (i + 1);
  if (mode == 0) {
    const bool want = live && (s.nfields == 0 || field_test(kind, arg, s.a.rd[0], s.fdt[0], i));
    push_removal(rm, want, id, REMOVE_ALL, order_key(call_pos, i, 0) + 1, s.status);
    return;
  }
  // round j: the j-th in-edge of every lane that has one; a lane's records
  // are numbered q in insertion order of the edges that pass the test
  const bool rows = live && i < c.nrows;
  const uint32_t b = rows ? c.row_ptr[i] : 0u;
  const uint32_t deg = rows ? c.row_ptr[i + 1] - b : 0u;
  uint32_t q = 0;
  for (uint32_t j = 0; __any_sync(FULL_WARP, j < deg); j++) {
    bool want = false;
    uint64_t nid = 0;
    if (j < deg) {
      const uint32_t e = b + j;
      const int ty = edge_src_type(c, e);
      const uint32_t src = c.src[e];
      if (ty <= 0 || ty >= MAX_AGENT_TYPES || !t.ptr[ty]) {
        set_status(s.status, 202);  // source type not readable
      } else if (field_test(kind, arg, t.ptr[ty], t.dt[ty], src)) {
        want = true;
        nid = ((uint64_t)ty << SHIFT_TYPE) | ((uint64_t)src + 1);
      }
    }
    push_removal(rm, want, id, nid, order_key(call_pos, i, q) + 1, s.status);
    q += want;
  }
}

// ------------------------------------------- add_agent! within a transition
// spawn: every swept agent keeps its state and calls add_agent! k times
// (src/AgentMethods.jl:37-89) with a copy of its state whose field 0 is
// increased by offset j; with a link edge type, after each add_agent! it
// adds the edges new -> caller and caller -> new, payload field 0 = the new
// agent's id.  Pass 1 keeps the callers and flags them; the callers' rank
// (an exclusive scan in index order) numbers the new agents in the order of
// the sequential sweep: new agent s takes the s-th slot popped from the
// reuse stack (LIFO) and, when the stack is empty, the next fresh number.
constexpr int SPAWN_MAX = 8;
struct SpawnArgs {
  int k;
  double off[SPAWN_MAX];
  const uint64_t *reuse;  // 1-based agent numbers, top at nreuse - 1
  uint64_t nreuse, take;  // stack height, slots taken from it
  uint64_t n_old;         // nextid - 1 before the transition
};

__global__ void k_spawn_flags(Sweep s, uint32_t *flag) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.a.n) return;
  bool swept = sw_begin(s, i);
  flag[i] = swept ? 1u : 0u;
  if (swept && s.writes) sw_copy(s, i);
}

__global__ void k_spawn_new(Sweep s, uint64_t n_callers_scope, const uint32_t *flag,
                            const uint32_t *pos, SpawnArgs g, Append ap, int link_dt,
                            int call_pos) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool caller = i < n_callers_scope && flag[i];
  const uint64_t id = ((uint64_t)s.type_nr << SHIFT_TYPE) | (i + 1);
  for (int j = 0; j < g.k; j++) {
    const uint64_t q = caller ? (uint64_t)pos[i] * g.k + j : 0;
    const uint64_t nr = !caller ? 0
                        : q < g.take ? g.reuse[g.nreuse - 1 - q] : g.n_old + 1 + (q - g.take);
    const uint64_t t = nr - 1;
    if (caller) {
      for (int f = 0; f < s.nfields; f++) {
        switch (s.fsize[f]) {
          case 1: ((uint8_t *)s.a.wr[f])[t] = ((const uint8_t *)s.a.rd[f])[i]; break;
          case 2: ((uint16_t *)s.a.wr[f])[t] = ((const uint16_t *)s.a.rd[f])[i]; break;
          case 4: ((uint32_t *)s.a.wr[f])[t] = ((const uint32_t *)s.a.rd[f])[i]; break;
          case 8: ((uint64_t *)s.a.wr[f])[t] = ((const uint64_t *)s.a.rd[f])[i]; break;
        }
      }
      if (s.nfields > 0) {
        int dt = s.fdt[0];
        if (is_float(dt)) st_f64(s.a.wr[0], dt, t, ld_f64(s.a.rd[0], dt, i) + g.off[j]);
        else st_i64(s.a.wr[0], dt, t, ld_i64(s.a.rd[0], dt, i) + (int64_t)g.off[j]);
      }
      if (s.mortal) s.a.died_wr[t] = 0;
    }
    if (link_dt < 0) continue;
    const uint64_t nid = ((uint64_t)s.type_nr << SHIFT_TYPE) | nr;
    for (int d = 0; d < 2; d++) {
      const int64_t k = warp_slot(ap.counter, ap.cap, caller, s.status, 301);
      if (k < 0) continue;
      ap.from[k] = d == 0 ? nid : id;
      ap.to[k] = d == 0 ? id : nid;
      ap.key[k] = order_key(call_pos, i, 2 * j + d);
      if (ap.npayload > 0) st_i64(ap.payload[0], link_dt, k, (int64_t)nid);
    }
  }
}

// link_neighbors: an agent whose field 0 equals die_value returns nothing;
// every other agent keeps its state and, for each source nid of its
// in-edges of type E in insertion order, adds nid -> id and id -> nid of
// type F with payload field 0 = its own field 0.
__global__ void k_link_neighbors(Sweep s, DevCSRView c, Append ap, int pl_dt, int has_die,
                                 double die_value, int call_pos) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool live = i < s.a.n && sw_begin(s, i);
  const int dt0 = s.fdt[0];
  const double v = live && s.nfields > 0 ? ld_f64(s.a.rd[0], dt0, i) : 0.0;
  if (live && has_die && s.nfields > 0 && v == die_value) {
    if (s.writes) sw_die(s, i);
    live = false;
  } else if (live && s.writes) {
    sw_copy(s, i);
  }
  const bool rows = live && i < c.nrows;
  const uint32_t b = rows ? c.row_ptr[i] : 0u;
  const uint32_t deg = rows ? c.row_ptr[i + 1] - b : 0u;
  const uint64_t id = ((uint64_t)s.type_nr << SHIFT_TYPE) | (i + 1);
  const int64_t vi = live && s.nfields > 0 ? ld_i64(s.a.rd[0], dt0, i) : 0;
  for (uint32_t j = 0; __any_sync(FULL_WARP, j < deg); j++) {
    const bool has = j < deg;
    const uint32_t e = b + j;
    const uint64_t nid =
        has ? ((uint64_t)edge_src_type(c, e) << SHIFT_TYPE) | ((uint64_t)c.src[e] + 1) : 0;
    for (int d = 0; d < 2; d++) {
      const int64_t k = warp_slot(ap.counter, ap.cap, has, s.status, 301);
      if (k < 0) continue;
      ap.from[k] = d == 0 ? nid : id;
      ap.to[k] = d == 0 ? id : nid;
      ap.key[k] = order_key(call_pos, i, 2 * j + d);
      if (ap.npayload > 0) {
        if (is_float(pl_dt)) st_f64(ap.payload[0], pl_dt, k, v);
        else st_i64(ap.payload[0], pl_dt, k, vi);
      }
    }
  }
}

// ----------------------------------------------- move_to! in a transition
// move_to!(sim, raster, id, pos, edge_from_raster, edge_to_raster; distance,
// metric, periodic, only_surrounding) -- src/Raster.jl:437-477 -- called by
// every swept agent: the cell at pos (unless only_surrounding), then the
// cells at the stencil offsets in the reference's order, each wrapped
// (periodic) or dropped when outside the raster (_checkpos,
// src/Raster.jl:479-499); per cell first the cell -> agent edge
// (edge_from_raster), then the agent -> cell edge (edge_to_raster).  The
// order key numbers the calls, so the rebuilt containers hold them in the
// order of the sequential sweep.  The new position: mode 0 the agent's
// fields 0..ndims-1 (1-based; the state is kept); mode 1 the Int field
// `nbr_field` of the agent's first in-neighbour along edge type `nbr_edge`
// in every dimension, which also becomes the agent's field 0 (the rule of
// test/raster.jl:309-314).
struct MoveArgs {
  int ndims;
  int64_t dims[MAX_DIMS];
  int cell_type;
  uint64_t first_nr;
  const int32_t *off;  // noff offsets, ndims each
  int noff;
  int periodic, only_surrounding;
  int mode;
  DevCSRView nbr;       // mode 1: the agent's in-edges
  SrcTable nbr_val;     // mode 1: the neighbours' field, per source type
  int has_from, has_to, same;  // same: one edge type, one buffer for both
  Append from, to;
};

__device__ __forceinline__ void move_emit(const MoveArgs &m, bool want, const int64_t *p,
                                          uint64_t id, uint64_t key, int *status) {
  uint64_t lin = 0, mul = 1;
  for (int d = 0; d < m.ndims; d++) {
    lin += (uint64_t)(p[d] - 1) * mul;
    mul *= (uint64_t)m.dims[d];
  }
  const uint64_t cell = ((uint64_t)m.cell_type << SHIFT_TYPE) | (m.first_nr + lin);
  for (int dir = 0; dir < 2; dir++) {
    if (dir == 0 ? !m.has_from : !m.has_to) continue;  // uniform over the launch
    const Append &ap = (dir == 1 && !m.same) ? m.to : m.from;
    const int64_t k = warp_slot(ap.counter, ap.cap, want, status, 301);
    if (k < 0) continue;
    ap.to[k] = dir == 0 ? id : cell;
    ap.from[k] = dir == 0 ? cell : id;
    ap.key[k] = key + dir;
    for (int f = 0; f < ap.npayload; f++)  // payload fields zero
      for (int b = 0; b < ap.psize[f]; b++) ((uint8_t *)ap.payload[f])[k * ap.psize[f] + b] = 0;
  }
}

__global__ void k_move_to(Sweep s, MoveArgs m, int call_pos) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < s.a.n && sw_begin(s, i);
  int64_t pos[MAX_DIMS] = {1, 1, 1, 1};
  bool ok = live;
  if (live) {
    if (m.mode == 0) {
      for (int d = 0; d < m.ndims; d++) pos[d] = ld_i64(s.a.rd[d], s.fdt[d], i);
    } else {
      int64_t v = 0;
      const int ty = i < m.nbr.nrows && m.nbr.row_ptr[i + 1] > m.nbr.row_ptr[i]
                         ? edge_src_type(m.nbr, m.nbr.row_ptr[i]) : 0;
      if (ty > 0 && ty < MAX_AGENT_TYPES && m.nbr_val.ptr[ty]) {
        v = ld_i64(m.nbr_val.ptr[ty], m.nbr_val.dt[ty], m.nbr.src[m.nbr.row_ptr[i]]);
      } else if (ty != 0) {
        set_status(s.status, 202);  // source type not readable, or without the field
        ok = false;
      } else {
        set_status(s.status, 203);  // first() of no neighbour
        ok = false;
      }
      for (int d = 0; d < m.ndims; d++) pos[d] = v;
    }
    for (int d = 0; d < m.ndims; d++)
      if (pos[d] < 1 || pos[d] > m.dims[d]) ok = false;
    if (!ok && m.mode == 0) set_status(s.status, 204);  // position outside the raster
    if (s.writes) {
      sw_copy(s, i);
      if (m.mode == 1 && ok) st_i64(s.a.wr[0], s.fdt[0], i, pos[0]);
    }
  }
  const uint64_t id = ((uint64_t)s.type_nr << SHIFT_TYPE) | (i + 1);
  if (!m.only_surrounding) move_emit(m, ok, pos, id, order_key(call_pos, i, 0), s.status);
  for (int k = 0; k < m.noff; k++) {
    int64_t q[MAX_DIMS] = {1, 1, 1, 1};
    bool in = ok;
    for (int d = 0; d < m.ndims; d++) {
      int64_t v = pos[d] + m.off[k * m.ndims + d];
      if (v < 1 || v > m.dims[d]) {
        if (!m.periodic) in = false;
        v = ((v - 1) % m.dims[d] + m.dims[d]) % m.dims[d] + 1;
      }
      q[d] = v;
    }
    move_emit(m, in, q, id, order_key(call_pos, i, 2 * (uint32_t)(k + 1)), s.status);
  }
}

// ---------------------------------------------------------- SIR (cfg 0)
// Person{state::UInt8 (0 S, 1 I, 2 R), days::Int32}.  A susceptible agent
// with k infected in-neighbours is infected with p_k = 1 - (1 - beta)^k
// (p_k from the host table, built by the same repeated multiplication);
// an infected agent recovers when days reaches `recovery`.
constexpr int SIR_U = 16;

// One SIR step.  Launched with programmatic dependent launch when the
// contact rows cannot be written by the preceding kernel (Sim::csr_epoch):
// this grid lets the next step's grid be scheduled once all its blocks run,
// and each thread requests its row bounds and first SIR_U sources before
// griddepcontrol.wait; the states (written by the previous step) and every
// output are touched only after it.  Without the launch attribute the wait
// returns at once.  SIR_U sources are requested together, then their
// states: two memory round trips for a row of up to SIR_U in-edges.
__global__ void k_sir(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ src,
                      const uint8_t *st_rd, const int32_t *d_rd, uint8_t *st_wr, int32_t *d_wr,
                      uint64_t n, uint64_t nrows, const double *__restrict__ ptab,
                      uint32_t ptab_n, uint64_t seed, uint32_t step, int32_t recovery,
                      int *status) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool row = i < n && i < nrows;
  uint32_t q = row ? __ldg(rp + i) : 0u;
  const uint32_t e = row ? __ldg(rp + i + 1) : 0u;
  uint32_t sv[SIR_U];
#pragma unroll
  for (int u = 0; u < SIR_U; u++) sv[u] = q + u < e ? __ldg(src + q + u) : 0u;
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (i >= n) return;
  uint8_t s = st_rd[i];
  int32_t d = d_rd[i];
  if (s == 0) {
    uint32_t k = 0;
    while (q < e) {
#pragma unroll
      for (int u = 0; u < SIR_U; u++) k += (q + u < e ? st_rd[sv[u]] : 0) == 1;
      q += SIR_U;
#pragma unroll
      for (int u = 0; u < SIR_U; u++) sv[u] = q + u < e ? __ldg(src + q + u) : 0u;
    }
    if (k > 0) {
      if (k >= ptab_n) {
        set_status(status, 401);
      } else {
        if (unit_below(philox_u64(philox_draw(seed, i + 1, step, TAG_INFECT)), ptab[k])) {
          s = 1;
          d = 0;
        }
      }
    }
  } else if (s == 1) {
    d = d + 1;
    if (d >= recovery) s = 2;
  }
  st_wr[i] = s;
  d_wr[i] = d;
}

// ------------------------------------------------ Life B3/S23 (cfg 2)
// Cells of a 2-D raster, implicit Moore stencil (chebyshev, distance 1).
// The count of alive neighbours does not depend on edge order.
// Four cells per thread as the bytes of one 32-bit word (byte i = cell
// x + i): per row the sum of left, centre and right neighbours in every
// byte lane, three rows added and the centre subtracted; a lane never
// exceeds 8, so no byte lane carries into the next.
// Moore neighbourhood of 2-D Life with four cells per 32-bit word (one
// byte each, 0 or 1): the sums of three horizontally adjacent cells of a
// row for all four bytes at once (no byte exceeds 3, so no carries cross
// bytes).  A warp holds 32 consecutive words of a row; the neighbouring
// words come from the adjacent lanes, and only the warp's edge lanes load.
__device__ __forceinline__ uint32_t life_hsum(uint32_t c, uint32_t lw, uint32_t rw) {
  return ((c << 8) | (lw >> 24)) + c + ((c >> 8) | (rw << 24));
}

// blocks of 32 x 8 threads; each thread LIFE_ROWS consecutive rows of one
// word column.  All LIFE_ROWS + 2 rows it reads are requested before any
// is used (one memory latency per thread); rows outside a non-periodic
// raster read as 0, a periodic raster wraps (a compare, no modulo).
constexpr int LIFE_ROWS = 8;

__global__ void __launch_bounds__(256) k_life2d_x4(const uint32_t *__restrict__ a,
                                                   uint32_t *__restrict__ o, int64_t Wq,
                                                   int64_t H, int periodic) {
  const unsigned lane = threadIdx.x & 31;
  const int64_t qx = (int64_t)blockIdx.x * 32 + lane;
  const int64_t y0 = ((int64_t)blockIdx.y * blockDim.y + threadIdx.y) * LIFE_ROWS;
  if (y0 >= H) return;  // warp-uniform
  const int64_t y1 = y0 + LIFE_ROWS < H ? y0 + LIFE_ROWS : H;  // rows y0 .. y1-1 are written
  const bool valid = qx < Wq;
  const bool left_edge = valid && lane == 0;
  const bool right_edge = valid && (lane == 31 || qx + 1 >= Wq);
  uint32_t c[LIFE_ROWS + 2], lw[LIFE_ROWS + 2], rw[LIFE_ROWS + 2];
#pragma unroll
  for (int i = 0; i < LIFE_ROWS + 2; i++) {
    const int64_t y = y0 - 1 + i;  // rows y0-1 .. y1 are read
    int64_t yy = y < 0 ? H - 1 : (y >= H ? y - H : y);
    const bool use = y <= y1 && ((y >= 0 && y < H) || periodic);
    const uint32_t *row = a + yy * Wq;
    c[i] = use && valid ? row[qx] : 0u;
    lw[i] = use && left_edge ? (qx > 0 ? row[qx - 1] : (periodic ? row[Wq - 1] : 0u)) : 0u;
    rw[i] = use && right_edge ? (qx + 1 < Wq ? row[qx + 1] : (periodic ? row[0] : 0u)) : 0u;
  }
  uint32_t hs[LIFE_ROWS + 2];
#pragma unroll
  for (int i = 0; i < LIFE_ROWS + 2; i++) {
    const uint32_t l = __shfl_up_sync(0xffffffffu, c[i], 1);
    const uint32_t r = __shfl_down_sync(0xffffffffu, c[i], 1);
    hs[i] = life_hsum(c[i], left_edge ? lw[i] : l, right_edge ? rw[i] : r);
  }
#pragma unroll
  for (int j = 0; j < LIFE_ROWS; j++) {
    const int64_t y = y0 + j;
    const uint32_t self = c[j + 1];
    const uint32_t cnt = hs[j] + hs[j + 1] + hs[j + 2] - self;
    const uint32_t born = __vcmpeq4(cnt, 0x03030303u);
    const uint32_t stay = __vcmpeq4(cnt, 0x02020202u) & __vcmpne4(self, 0u);
    if (valid && y < y1) o[y * Wq + qx] = (born | stay) & 0x01010101u;
  }
}

__global__ void k_life2d(const uint8_t *__restrict__ a, uint8_t *__restrict__ o,
                         int64_t W, int64_t H, int periodic) {
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t y = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  int cnt = 0;
#pragma unroll
  for (int dy = -1; dy <= 1; dy++) {
    int64_t yy = y + dy;
    if (yy < 0 || yy >= H) {
      if (!periodic) continue;
      yy = (yy + H) % H;
    }
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
      if (!dx && !dy) continue;
      int64_t xx = x + dx;
      if (xx < 0 || xx >= W) {
        if (!periodic) continue;
        xx = (xx + W) % W;
      }
      cnt += __ldg(a + yy * W + xx);
    }
  }
  uint8_t alive = a[y * W + x];
  o[y * W + x] = (cnt == 3 || (alive && cnt == 2)) ? 1 : 0;
}

// general implicit stencil (any dims, offsets): count of alive sources
struct StencilArgs {
  int ndims;
  int64_t dims[MAX_DIMS];
  int noff;
  int8_t off[128 * MAX_DIMS];
  int periodic;
};

__global__ void k_life_stencil(const uint8_t *__restrict__ a, uint8_t *__restrict__ o,
                               uint64_t ncells, StencilArgs st, int birth_mask,
                               int survive_mask) {
  uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  int64_t pos[MAX_DIMS];
  uint64_t t = c;
  for (int i = 0; i < st.ndims; i++) {
    pos[i] = (int64_t)(t % st.dims[i]);
    t /= st.dims[i];
  }
  int cnt = 0;
  for (int k = 0; k < st.noff; k++) {
    uint64_t lin = 0, m = 1;
    bool ok = true;
    for (int i = 0; i < st.ndims; i++) {
      int64_t q = pos[i] - st.off[k * st.ndims + i];
      if (q < 0 || q >= st.dims[i]) {
        if (!st.periodic) { ok = false; break; }
        q = ((q % st.dims[i]) + st.dims[i]) % st.dims[i];
      }
      lin += (uint64_t)q * m;
      m *= st.dims[i];
    }
    if (ok) cnt += a[lin];
  }
  uint8_t alive = a[c];
  int bit = cnt < 31 ? (1 << cnt) : 0;
  o[c] = alive ? ((survive_mask & bit) ? 1 : 0) : ((birth_mask & bit) ? 1 : 0);
}

// ------------------------------------------------- random walk (cfg 2)
// Walker{x::Int32, y::Int32} (1-based cell position).  Each step a walker
// moves by one of the 8 Moore offsets, drawn by Philox, wraps (mod1) and
// calls move_to!(sim, raster, id, (x', y'), nothing, OnCell()): one edge
// walker -> cell.  Record i belongs to walker i, so records come out in the
// reference's sweep order without atomics.
__global__ void k_random_walk(const int32_t *__restrict__ x, const int32_t *__restrict__ y,
                              int32_t *__restrict__ xo, int32_t *__restrict__ yo, uint64_t n,
                              int64_t W, int64_t H, uint64_t seed, uint32_t step,
                              uint64_t *__restrict__ to, uint64_t *__restrict__ from,
                              int walker_type, int cell_type, uint64_t cell_first_nr) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Philox4 r = philox_draw(seed, i + 1, step, TAG_MOVE);
  uint32_t k = bounded32(r.v[0], 8);
  // Moore offsets in stencil order (first dimension fastest, centre removed)
  uint32_t m = k < 4 ? k : k + 1;
  int64_t nx = (int64_t)x[i] + (int)(m % 3) - 1;
  int64_t ny = (int64_t)y[i] + (int)(m / 3) - 1;
  nx = ((nx - 1) % W + W) % W + 1;
  ny = ((ny - 1) % H + H) % H + 1;
  xo[i] = (int32_t)nx;
  yo[i] = (int32_t)ny;
  from[i] = ((uint64_t)walker_type << SHIFT_TYPE) | (i + 1);
  to[i] = ((uint64_t)cell_type << SHIFT_TYPE) |
          (cell_first_nr + (uint64_t)(nx - 1) + (uint64_t)(ny - 1) * (uint64_t)W);
}

// ------------------------------------------------------------- launchers
Sweep make_sweep(ApplyCtx &c) {
  Sim &s = *c.sim;
  const AgentTypeDesc &ad = s.model->at(c.call_type);
  Sweep w{};
  w.a = agent_view(s, c.call_type);
  w.nfields = (int)ad.fields.size();
  for (int f = 0; f < w.nfields; f++) {
    w.fsize[f] = ad.fields[f].size;
    w.fdt[f] = ad.fields[f].dtype;
  }
  w.mortal = !ad.immortal();
  w.writes = c.writes_call() ? 1 : 0;
  w.type_nr = c.call_type;
  w.status = s.d_status.as<int>();
  if (c.with_edge >= 0) {
    EdgeStore &es = s.edges[c.with_edge];
    if (c.call_type < (int)es.csr.size() && es.csr[c.call_type].row_ptr.p) {
      w.with_rp = es.csr[c.call_type].row_ptr.as<uint32_t>();
      w.with_nrows = es.csr[c.call_type].nrows;
    } else {
      // no agent of this type is the target of such an edge: with_nrows = 0
      // makes every row empty (the pointer is never dereferenced)
      w.with_rp = (const uint32_t *)s.d_status.p;
      w.with_nrows = 0;
    }
  }
  return w;
}

int need_edge_param(ApplyCtx &c, int idx) {
  Sim &s = *c.sim;
  if (idx >= c.nparams) fail(VG_ERR_ARG, "transition parameter missing: edge type");
  int e = (int)c.params[idx];
  s.model->et(e);
  return e;
}

void require_read(ApplyCtx &c, int ref, const std::string &what) {
  if (!c.in_read(ref) && c.sim->check_readable) fail(VG_ERR_ASSERT, what);
}

void require_edge_read(ApplyCtx &c, int e) {
  require_read(c, VG_EDGE(e),
               "You try to access an edge of type " + c.sim->model->et(e).name +
                   " but the type is not in the `read` argument of the apply! function.");
}

void require_agent_read(ApplyCtx &c, int T) {
  require_read(c, T, c.sim->model->at(T).name +
                         " must be in the `read` argument of the transition function.");
}

// the source types present in a CSR must be readable
void require_sources_read(ApplyCtx &c, int e, int T) {
  Sim &s = *c.sim;
  EdgeStore &es = s.edges[e];
  if (T >= (int)es.csr.size()) return;
  CSR &cs = es.csr[T];
  if (cs.nedges == 0) return;
  std::vector<int> types;
  if (cs.src_type_const > 0) {
    types.push_back(cs.src_type_const);
  } else if (cs.src_type_const < 0) {
    std::vector<uint8_t> st(cs.nedges);
    VG_CUDA(cudaMemcpyAsync(st.data(), cs.src_type.p, cs.nedges, cudaMemcpyDeviceToHost, s.stream));
    VG_CUDA(cudaStreamSynchronize(s.stream));
    bool seen[256] = {false};
    for (auto t : st) seen[t] = true;
    for (int t = 1; t < 256; t++)
      if (seen[t]) types.push_back(t);
  }
  for (int t : types) require_agent_read(c, t);
}

SrcTable make_src_table(ApplyCtx &c, int field_index) {
  Sim &s = *c.sim;
  SrcTable t{};
  for (int T = 1; T <= (int)s.model->atypes.size() && T < MAX_AGENT_TYPES; T++) {
    const AgentTypeDesc &ad = s.model->at(T);
    if (field_index < (int)ad.fields.size() && !s.agents[T - 1].rd.empty()) {
      t.ptr[T] = s.agents[T - 1].rd[field_index].p;
      t.dt[T] = ad.fields[field_index].dtype;
    }
    t.died[T] = ad.immortal() ? nullptr : s.agents[T - 1].died_rd.as<uint8_t>();
  }
  return t;
}

void launch_neighbor_op(ApplyCtx &c, int mode) {
  Sim &s = *c.sim;
  int e = need_edge_param(c, 0);
  int sf = (int)c.param(1, 0), df = (int)c.param(2, 0);
  const AgentTypeDesc &ad = s.model->at(c.call_type);
  if (df < 0 || df >= (int)ad.fields.size()) fail(VG_ERR_ARG, "destination field out of range");
  require_edge_read(c, e);
  if (mode != 2) require_sources_read(c, e, c.call_type);
  Sweep w = make_sweep(c);
  DevCSRView v = csr_view(s, e, c.call_type);
  SrcTable t = make_src_table(c, sf);
  if (w.a.n == 0) return;
  k_neighbor_op<<<nblk(w.a.n), TPB, 0, s.stream>>>(w, v, t, df, mode);
  VG_CUDA(cudaGetLastError());
}

void tr_neighbor_sum(ApplyCtx &c) { launch_neighbor_op(c, 0); }
void tr_neighbor_or(ApplyCtx &c) { launch_neighbor_op(c, 1); }
void tr_count_edges(ApplyCtx &c) { launch_neighbor_op(c, 2); }

void tr_die_if(ApplyCtx &c) {
  Sim &s = *c.sim;
  int kind = (int)c.param(0, 0);
  int field = (int)c.param(1, 0);
  double arg = c.param(2, 0);
  const uint32_t *rp2 = nullptr;
  uint64_t n2 = 0;
  if (kind == 3) {
    int e = field;
    s.model->et(e);
    require_edge_read(c, e);
    DevCSRView v = csr_view(s, e, c.call_type);
    rp2 = v.row_ptr;
    n2 = v.nrows;
    field = 0;
  } else if (kind == 1 || kind == 2) {
    if (field < 0 || field >= (int)s.model->at(c.call_type).fields.size())
      fail(VG_ERR_ARG, "field out of range");
    require_agent_read(c, c.call_type);
  }
  Sweep w = make_sweep(c);
  if (w.a.n == 0) return;
  k_die_if<<<nblk(w.a.n), TPB, 0, s.stream>>>(w, kind, field, arg, rp2, n2);
  VG_CUDA(cudaGetLastError());
}

void tr_set_field(ApplyCtx &c) {
  Sim &s = *c.sim;
  int field = (int)c.param(0, 0);
  if (field < 0 || field >= (int)s.model->at(c.call_type).fields.size())
    fail(VG_ERR_ARG, "field out of range");
  Sweep w = make_sweep(c);
  if (w.a.n == 0) return;
  k_set_field<<<nblk(w.a.n), TPB, 0, s.stream>>>(w, field, (int)c.param(1, 0), c.param(2, 0));
  VG_CUDA(cudaGetLastError());
}

void tr_keep(ApplyCtx &c) {
  Sim &s = *c.sim;
  Sweep w = make_sweep(c);
  if (w.a.n == 0) return;
  k_keep<<<nblk(w.a.n), TPB, 0, s.stream>>>(w);
  VG_CUDA(cudaGetLastError());
}

Append make_append(ApplyCtx &c, int e, uint64_t cap) {
  Sim &s = *c.sim;
  const EdgeTypeDesc &ed = s.model->et(e);
  if (!c.in_write(VG_EDGE(e)) && s.check_readable)
    fail(VG_ERR_ASSERT, ed.name + " must be in the `write` argument of the transition function.");
  EdgeAppend *a = c.append_for(e, cap, false);
  Append ap{};
  ap.to = a->to.as<uint64_t>();
  ap.from = a->from.as<uint64_t>();
  ap.key = a->key.as<uint64_t>();
  ap.npayload = (int)a->payload.size();
  for (int f = 0; f < ap.npayload; f++) {
    ap.payload[f] = a->payload[f].p;
    ap.psize[f] = ed.fields[f].size;
  }
  ap.counter = a->counter.as<unsigned long long>();
  ap.cap = a->cap;
  return ap;
}

void tr_self_edge(ApplyCtx &c) {
  Sim &s = *c.sim;
  int e = need_edge_param(c, 0);
  const EdgeTypeDesc &ed = s.model->et(e);
  Sweep w = make_sweep(c);
  if (w.a.n == 0) return;
  Append ap = make_append(c, e, w.a.n);
  // constant payload from params[1..]: one value per field
  std::vector<uint8_t> pl;
  if (ed.stores_payload())
    for (size_t f = 0; f < ed.fields.size(); f++) {
      double v = c.param(1 + (int)f, 0);
      uint8_t buf[8] = {0};
      int dt = ed.fields[f].dtype;
      if (dt == VG_F64) std::memcpy(buf, &v, 8);
      else if (dt == VG_F32) { float x = (float)v; std::memcpy(buf, &x, 4); }
      else { int64_t x = (int64_t)v; std::memcpy(buf, &x, 8); }
      pl.insert(pl.end(), buf, buf + ed.fields[f].size);
    }
  uint8_t *d_pl = (uint8_t *)s.scratch(std::max<size_t>(pl.size(), 8));
  if (!pl.empty())
    VG_CUDA(cudaMemcpyAsync(d_pl, pl.data(), pl.size(), cudaMemcpyHostToDevice, s.stream));
  k_self_edge<<<nblk(w.a.n), TPB, 0, s.stream>>>(w, ap, c.call_pos, d_pl);
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaStreamSynchronize(s.stream));
}

void tr_readd_edges(ApplyCtx &c) {
  Sim &s = *c.sim;
  int e = need_edge_param(c, 0);
  const EdgeTypeDesc &ed = s.model->et(e);
  if (ed.stateless() || ed.ignorefrom())
    fail(VG_ERR_ASSERT, "edges is not defined for the hint combination of " + ed.name);
  require_edge_read(c, e);
  Sweep w = make_sweep(c);
  DevCSRView v = csr_view(s, e, c.call_type);
  if (w.a.n == 0) return;
  Append ap = make_append(c, e, std::max<uint64_t>(v.nedges, 1));
  k_readd_edges<<<nblk(w.a.n), TPB, 0, s.stream>>>(w, v, ap, c.call_pos);
  VG_CUDA(cudaGetLastError());
}

void tr_remove_edges(ApplyCtx &c) {
  Sim &s = *c.sim;
  const int E = need_edge_param(c, 0);
  const EdgeTypeDesc &ed = s.model->et(E);
  const int kind = (int)c.param(1, 0);
  const double arg = c.param(2, 0);
  const int mode = (int)c.param(3, 0);
  if (kind < 0 || kind > 2 || mode < 0 || mode > 1) fail(VG_ERR_ARG, "remove_edges: kind 0..2, mode 0..1");
  if (kind == 2 && arg == 0) fail(VG_ERR_ARG, "remove_edges: modulus 0");
  if (!c.in_write(VG_EDGE(E)) && s.check_readable)
    fail(VG_ERR_ASSERT, ed.name + " must be in the `write` argument of the transition function.");
  Sweep w = make_sweep(c);
  DevCSRView v = csr_view(s, E, c.call_type);
  SrcTable t{};
  uint64_t cap = w.a.n;
  if (mode == 1) {
    if (ed.ignorefrom())
      fail(VG_ERR_ASSERT, "remove_edges! with a source agent is not defined for edgetypes "
                          "with the :IgnoreFrom hint.");
    require_edge_read(c, E);
    require_sources_read(c, E, c.call_type);
    t = make_src_table(c, 0);
    cap = v.nedges;
  } else if (kind != 0) {
    require_agent_read(c, c.call_type);
  }
  if (w.a.n == 0) return;
  EdgeRemoval *r = c.removal_for(E, std::max<uint64_t>(cap, 1));
  Removal rm{r->to.as<uint64_t>(), r->from.as<uint64_t>(), r->key.as<uint64_t>(),
             r->counter.as<unsigned long long>(), r->cap};
  k_remove_edges<<<nblk(w.a.n), TPB, 0, s.stream>>>(w, v, t, kind, arg, mode, rm, c.call_pos);
  VG_CUDA(cudaGetLastError());
}

void tr_spawn(ApplyCtx &c) {
  Sim &s = *c.sim;
  const int T = c.call_type;
  const AgentTypeDesc &ad = s.model->at(T);
  const int k = (int)c.param(0, 1);
  if (k < 0 || k > SPAWN_MAX) fail(VG_ERR_ARG, "spawn: 0..8 new agents per caller");
  if (!c.writes_call())
    fail(VG_ERR_ASSERT, ad.name + " must be in the `write` argument of the transition function.");
  if (!ad.fields.empty()) require_agent_read(c, T);
  SpawnArgs g{};
  g.k = k;
  for (int j = 0; j < k; j++) g.off[j] = c.param(1 + j, 0);
  const int link = c.nparams > 1 + k ? (int)c.params[1 + k] : -1;
  int link_dt = -1;
  if (link >= 0) {
    const EdgeTypeDesc &ed = s.model->et(link);
    link_dt = ed.stores_payload() ? ed.fields[0].dtype : VG_I64;
    if (ed.stores_payload() && (link_dt == VG_F32 || link_dt == VG_F64))
      fail(VG_ERR_ARG, "spawn: the link edge's field 0 holds an agent id (an integer)");
  }
  Sweep w = make_sweep(c);
  const uint64_t n = w.a.n;
  if (n == 0) return;
  uint32_t *flag = nullptr, *pos = nullptr;
  VG_CUDA(cudaMallocAsync((void **)&flag, (n + 1) * 4, s.stream));
  VG_CUDA(cudaMallocAsync((void **)&pos, (n + 1) * 4, s.stream));
  k_spawn_flags<<<nblk(n), TPB, 0, s.stream>>>(w, flag);
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaMemsetAsync(flag + n, 0, 4, s.stream));
  exclusive_scan_u32(flag, pos, n + 1, s.stream, s);
  uint32_t m = 0;
  VG_CUDA(cudaMemcpyAsync(&m, pos + n, 4, cudaMemcpyDeviceToHost, s.stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
  AgentStore &a = s.agents[T - 1];
  const uint64_t total = (uint64_t)m * k;
  g.nreuse = ad.immortal() ? 0 : a.nreuse;
  g.take = std::min<uint64_t>(total, g.nreuse);
  g.reuse = a.reuse.as<uint64_t>();
  g.n_old = a.n;
  const uint64_t n_new = a.n + (total - g.take);
  agent_reserve(s, T, n_new);  // may move the columns: take the views after it
  Sweep w2 = make_sweep(c);
  Append ap{};
  if (link >= 0 && total > 0) ap = make_append(c, link, 2 * total);
  if (total > 0)
    k_spawn_new<<<nblk(n), TPB, 0, s.stream>>>(w2, n, flag, pos, g, ap, link >= 0 ? link_dt : -1,
                                               c.call_pos);
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaFreeAsync(flag, s.stream));
  VG_CUDA(cudaFreeAsync(pos, s.stream));
  a.nreuse = g.nreuse - g.take;
  a.n = n_new;
  a.nliving += total;
}

void tr_link_neighbors(ApplyCtx &c) {
  Sim &s = *c.sim;
  const int E = (int)c.param(0, -1), F = (int)c.param(1, -1);
  s.model->et(E);
  const EdgeTypeDesc &fd = s.model->et(F);
  require_edge_read(c, E);
  Sweep w = make_sweep(c);
  if (w.nfields > 0) require_agent_read(c, c.call_type);
  const int has_die = c.nparams > 2;
  const double die_value = c.param(2, 0);
  DevCSRView v = csr_view(s, E, c.call_type);
  if (w.a.n == 0) return;
  Append ap = make_append(c, F, std::max<uint64_t>(2 * v.nedges, 1));
  const int pl_dt = fd.stores_payload() ? fd.fields[0].dtype : -1;
  k_link_neighbors<<<nblk(w.a.n), TPB, 0, s.stream>>>(w, v, ap, pl_dt, has_die, die_value,
                                                      c.call_pos);
  VG_CUDA(cudaGetLastError());
}

void tr_sir(ApplyCtx &c) {
  Sim &s = *c.sim;
  const AgentTypeDesc &ad = s.model->at(c.call_type);
  if (ad.fields.size() < 2 || ad.fields[0].dtype != VG_U8 || ad.fields[1].dtype != VG_I32)
    fail(VG_ERR_ARG, "sir: agent type needs fields (state::UInt8, days::Int32)");
  if (!ad.immortal()) fail(VG_ERR_ARG, "sir: Person is :Immortal");
  int e = need_edge_param(c, 0);
  double beta = c.param(1, 0.05);
  int32_t rec = (int32_t)c.param(2, 7);
  uint64_t seed = (uint64_t)c.param(3, 0);
  require_edge_read(c, e);
  require_agent_read(c, c.call_type);
  if (!c.writes_call()) fail(VG_ERR_ARG, "sir: the called type must be in `write`");
  EdgeStore &es = s.edges[e];
  DevCSRView v = csr_view(s, e, c.call_type);
  if (v.nedges && v.src_type_const != c.call_type)
    fail(VG_ERR_ARG, "sir: contact sources must be of the called type");
  uint32_t maxdeg = c.call_type < (int)es.csr.size() ? csr_max_degree(s, es.csr[c.call_type]) : 0;
  // p_k = 1 - q^k by repeated multiplication, k = 0..maxdeg
  std::vector<double> ptab(maxdeg + 1);
  double q = 1.0, om = 1.0 - beta;
  ptab[0] = 0.0;
  for (uint32_t k = 1; k <= maxdeg; k++) {
    q = q * om;
    ptab[k] = 1.0 - q;
  }
  const double *d_ptab = (const double *)s.const_table("sir.p_infect", ptab.data(), ptab.size() * 8);
  DevAgentView a = agent_view(s, c.call_type);
  if (a.n == 0) return;
  // programmatic dependent launch only while no edge container was written
  // since the previous SIR step (the kernel reads its rows before waiting)
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(nblk(a.n));
  cfg.blockDim = dim3(TPB);
  cfg.stream = s.stream;
  cfg.attrs = attr;
  cfg.numAttrs = s.sir_epoch == s.csr_epoch ? 1 : 0;
  VG_CUDA(cudaLaunchKernelEx(&cfg, k_sir, v.row_ptr, v.src, (const uint8_t *)a.rd[0],
                             (const int32_t *)a.rd[1], (uint8_t *)a.wr[0], (int32_t *)a.wr[1],
                             a.n, v.nrows, d_ptab, (uint32_t)ptab.size(), seed,
                             (uint32_t)c.step, rec, s.d_status.as<int>()));
  s.sir_epoch = s.csr_epoch;
}

void tr_life(ApplyCtx &c) {
  Sim &s = *c.sim;
  const AgentTypeDesc &ad = s.model->at(c.call_type);
  if (ad.fields.empty() || (ad.fields[0].dtype != VG_BOOL && ad.fields[0].dtype != VG_U8))
    fail(VG_ERR_ARG, "life: cell field 0 must be Bool");
  int e = need_edge_param(c, 0);
  EdgeStore &es = s.edges[e];
  if (!es.implicit) fail(VG_ERR_ARG, "life: the neighbour edges must be implicit raster edges");
  require_edge_read(c, e);
  require_agent_read(c, c.call_type);
  if (!c.writes_call()) fail(VG_ERR_ARG, "life: the called type must be in `write`");
  const StencilDesc &st = es.st;
  const Raster &R = s.rasters[st.raster];
  if (R.type_nr != c.call_type) fail(VG_ERR_ARG, "life: raster cells must be the called type");
  AgentStore &A = s.agents[c.call_type - 1];
  if (R.first_nr != 1 || R.ncells != A.n)
    fail(VG_ERR_ARG, "life: the raster must hold all agents of its type");
  const uint8_t *in = A.rd[0].as<uint8_t>();
  uint8_t *out = A.wr[0].as<uint8_t>();
  int birth = (int)c.param(1, 8), survive = (int)c.param(2, 12);  // B3 = 1<<3, S23 = 1<<2|1<<3
  bool moore2d = st.ndims == 2 && st.noff == 8 && birth == 8 && survive == 12;
  if (moore2d) {
    for (int k = 0; k < 8; k++) {
      int ox = st.offsets[2 * k], oy = st.offsets[2 * k + 1];
      if (std::abs(ox) > 1 || std::abs(oy) > 1) moore2d = false;
    }
  }
  if (moore2d && st.dims[0] % 4 == 0 && ((uintptr_t)in % 4) == 0 && ((uintptr_t)out % 4) == 0) {
    const int64_t Wq = st.dims[0] / 4;
    dim3 blk(32, 8);
    dim3 grd((unsigned)((Wq + 31) / 32),
             (unsigned)((st.dims[1] + 8 * LIFE_ROWS - 1) / (8 * LIFE_ROWS)));
    k_life2d_x4<<<grd, blk, 0, s.stream>>>((const uint32_t *)in, (uint32_t *)out, Wq, st.dims[1],
                                          st.periodic);
  } else if (moore2d) {
    dim3 blk(32, 8);
    dim3 grd((unsigned)((st.dims[0] + 31) / 32), (unsigned)((st.dims[1] + 7) / 8));
    k_life2d<<<grd, blk, 0, s.stream>>>(in, out, st.dims[0], st.dims[1], st.periodic);
  } else {
    if (st.noff > 128) fail(VG_ERR_ARG, "life: at most 128 stencil offsets");
    StencilArgs sa{};
    sa.ndims = st.ndims;
    for (int i = 0; i < st.ndims; i++) sa.dims[i] = st.dims[i];
    sa.noff = st.noff;
    for (int k = 0; k < st.noff * st.ndims; k++) sa.off[k] = (int8_t)st.offsets[k];
    sa.periodic = st.periodic;
    k_life_stencil<<<nblk(R.ncells), TPB, 0, s.stream>>>(in, out, R.ncells, sa, birth, survive);
  }
  VG_CUDA(cudaGetLastError());
}

void tr_random_walk(ApplyCtx &c) {
  Sim &s = *c.sim;
  const AgentTypeDesc &ad = s.model->at(c.call_type);
  if (ad.fields.size() < 2 || ad.fields[0].dtype != VG_I32 || ad.fields[1].dtype != VG_I32)
    fail(VG_ERR_ARG, "random_walk: walker fields (x::Int32, y::Int32)");
  if (!ad.immortal()) fail(VG_ERR_ARG, "random_walk: walkers are :Immortal");
  int e = need_edge_param(c, 0);
  int ri = (int)c.param(1, 0);
  uint64_t seed = (uint64_t)c.param(2, 0);
  if (ri < 0 || ri >= (int)s.rasters.size()) fail(VG_ERR_ARG, "random_walk: raster index");
  const Raster &R = s.rasters[ri];
  if (R.ndims != 2) fail(VG_ERR_ARG, "random_walk: 2-D raster");
  const EdgeTypeDesc &ed = s.model->et(e);
  if (ed.stores_payload()) fail(VG_ERR_ARG, "random_walk: OnCell edges are stateless");
  if (!c.writes_call()) fail(VG_ERR_ARG, "random_walk: the called type must be in `write`");
  if (!c.in_write(VG_EDGE(e)))
    fail(VG_ERR_ASSERT, ed.name + " must be in the `write` argument of the transition function.");
  require_agent_read(c, c.call_type);
  DevAgentView a = agent_view(s, c.call_type);
  if (a.n == 0) return;
  EdgeAppend *ap = c.append_for(e, a.n, true);
  ap->fixed_count = a.n;
  ap->target_type = R.type_nr;  // walker -> cell records, typed by construction
  ap->src_type = c.call_type;
  k_random_walk<<<nblk(a.n), TPB, 0, s.stream>>>(
      (const int32_t *)a.rd[0], (const int32_t *)a.rd[1], (int32_t *)a.wr[0],
      (int32_t *)a.wr[1], a.n, R.dims[0], R.dims[1], seed, (uint32_t)c.step,
      ap->to.as<uint64_t>(), ap->from.as<uint64_t>(), c.call_type, R.type_nr, R.first_nr);
  VG_CUDA(cudaGetLastError());
}

// apply!(sim, move_to, [T], read, write; params = [raster, edge_from
// (-1: nothing), edge_to (-1: nothing), distance, metric (0 chebyshev, 1
// euclidean, 2 manhatten), periodic, only_surrounding, mode, nbr_edge,
// nbr_field]); mode and the last two as in k_move_to.
void tr_move_to(ApplyCtx &c) {
  Sim &s = *c.sim;
  const AgentTypeDesc &ad = s.model->at(c.call_type);
  const int ri = (int)c.param(0, -1);
  if (ri < 0 || ri >= (int)s.rasters.size()) fail(VG_ERR_ARG, "move_to: raster index");
  const Raster &R = s.rasters[ri];
  const int ef = (int)c.param(1, -1), et = (int)c.param(2, -1);
  const double distance = c.param(3, 0);
  const int metric = (int)c.param(4, VG_METRIC_CHEBYSHEV);
  const int mode = (int)c.param(7, 0);
  if (metric < 0 || metric > 2) fail(VG_ERR_ARG, "move_to: metric 0..2");
  if (mode < 0 || mode > 1) fail(VG_ERR_ARG, "move_to: mode 0 (own fields) or 1 (neighbour)");
  MoveArgs m{};
  m.ndims = R.ndims;
  for (int d = 0; d < R.ndims; d++) m.dims[d] = R.dims[d];
  m.cell_type = R.type_nr;
  m.first_nr = R.first_nr;
  m.periodic = c.param(5, 1) != 0;
  m.only_surrounding = c.param(6, 0) != 0;
  m.mode = mode;
  if (mode == 0) {
    if ((int)ad.fields.size() < R.ndims) fail(VG_ERR_ARG, "move_to: one Int field per dimension");
    for (int d = 0; d < R.ndims; d++)
      if (ad.fields[d].dtype == VG_F32 || ad.fields[d].dtype == VG_F64)
        fail(VG_ERR_ARG, "move_to: the position fields are integers");
    require_agent_read(c, c.call_type);
  } else {
    const int ne = need_edge_param(c, 8);
    require_edge_read(c, ne);
    require_sources_read(c, ne, c.call_type);
    m.nbr = csr_view(s, ne, c.call_type);
    if (ad.fields.empty() || ad.fields[0].dtype == VG_F32 || ad.fields[0].dtype == VG_F64)
      fail(VG_ERR_ARG, "move_to: mode 1 writes the position to an Int field 0");
    const int nf = (int)c.param(9, 0);
    if (nf < 0) fail(VG_ERR_ARG, "move_to: neighbour field");
    m.nbr_val = make_src_table(c, nf);
  }
  Sweep w = make_sweep(c);
  if (w.a.n == 0) return;
  std::vector<int> off = distance >= 1 ? make_stencil(metric, R.ndims, distance) : std::vector<int>();
  m.noff = (int)(off.size() / std::max(1, R.ndims));
  if (m.noff > (1 << 18)) fail(VG_ERR_ARG, "move_to: stencil too large");
  std::vector<int32_t> off32(off.begin(), off.end());
  const std::string key = "move_to:" + std::to_string(metric) + ":" + std::to_string(R.ndims) +
                          ":" + std::to_string(distance);
  m.off = off32.empty() ? nullptr
                        : (const int32_t *)s.const_table(key, off32.data(), off32.size() * 4);
  const uint64_t per = (uint64_t)(m.only_surrounding ? 0 : 1) + (uint64_t)m.noff;
  m.has_from = ef >= 0;
  m.has_to = et >= 0;
  m.same = m.has_from && m.has_to && ef == et;
  if (m.has_from) m.from = make_append(c, ef, std::max<uint64_t>(1, w.a.n * per * (m.same ? 2 : 1)));
  if (m.has_to && !m.same) m.to = make_append(c, et, std::max<uint64_t>(1, w.a.n * per));
  k_move_to<<<nblk(w.a.n), TPB, 0, s.stream>>>(w, m, c.call_pos);
  VG_CUDA(cudaGetLastError());
}

}  // namespace

const std::vector<TransitionDef> &transitions() {
  static const std::vector<TransitionDef> defs = {
      {"bounded_confidence", tr_bounded_confidence},
      {"sir", tr_sir},
      {"life", tr_life},
      {"random_walk", tr_random_walk},
      {"move_to", tr_move_to},
      {"neighbor_sum", tr_neighbor_sum},
      {"neighbor_or", tr_neighbor_or},
      {"count_edges", tr_count_edges},
      {"die_if", tr_die_if},
      {"set_field", tr_set_field},
      {"keep", tr_keep},
      {"self_edge", tr_self_edge},
      {"readd_edges", tr_readd_edges},
      {"spawn", tr_spawn},
      {"link_neighbors", tr_link_neighbors},
      {"remove_edges", tr_remove_edges},
  };
  return defs;
}

}  // namespace vg
