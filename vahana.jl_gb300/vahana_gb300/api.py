"""Python mirror of Vahana.jl's public API over the C ABI.

Names follow the reference (src/*.jl) with the trailing `!` dropped; the
mutating `apply!` is `apply_` and the copying `apply` is `apply`.  Agent and
edge types are declared with their fields (name, dtype), as the Julia
structs would be; transition functions are the kernels registered in the
library, named by string (`transition_names()` lists them).

Errors: where the reference raises AssertionError, so does this module.
"""
import ctypes as C
import os

import numpy as np

from ._lib import (DTYPES, HINTS, MAPS, METRICS, NP_DTYPES, OPS, VG_EDGE, check, lib)

# AgentID layout, src/Agent.jl:30-115 (process bits are always 0 here)
BITS_TYPE, BITS_PROCESS, BITS_AGENTNR = 8, 20, 36
SHIFT_TYPE = BITS_PROCESS + BITS_AGENTNR
SHIFT_RANK = BITS_AGENTNR


def agent_id(type_nr, nr, rank=0):
    return np.uint64((int(type_nr) << SHIFT_TYPE) | (int(rank) << SHIFT_RANK) | int(nr))


def type_nr(id):
    return int(id) >> SHIFT_TYPE


def process_nr(id):
    return (int(id) >> SHIFT_RANK) & ((1 << BITS_PROCESS) - 1)


def agent_nr(id):
    return int(id) & ((1 << BITS_AGENTNR) - 1)


def _cstrs(names):
    arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
    return arr


def _hints(hints):
    h = 0
    for x in hints:
        x = x if x.startswith(":") else ":" + x
        if x not in HINTS:
            raise AssertionError("The hint %s is unknown" % x)
        h |= HINTS[x]
    return h


class TypeInfo:
    def __init__(self, name, fields, kind, index):
        self.name = name
        self.fields = list(fields)
        self.kind = kind  # "agent" or "edge"
        self.index = index  # agent type number or edge type index

    @property
    def ref(self):
        return self.index if self.kind == "agent" else VG_EDGE(self.index)

    def field_index(self, name):
        for i, (n, _) in enumerate(self.fields):
            if n == name:
                return i
        raise KeyError("type %s has no field %s" % (self.name, name))

    def dtype(self, f):
        return NP_DTYPES[self.fields[f][1]]

    def __repr__(self):
        return "%s(%s)" % (self.name, ", ".join("%s::%s" % f for f in self.fields))


class ModelTypes:
    """ModelTypes() -- src/ModelTypes.jl:32-41, with the pipeable register_* calls."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().vg_model_create(C.byref(h)))
        self._h = h
        self.types = {}
        self.agent_types = []
        self.edge_types = []
        self.params = {}
        self.globals = {}

    def register_agenttype(self, name, fields=(), *hints):
        """register_agenttype!(types, T, hints...) -- src/ModelTypes.jl:81-106"""
        fields = list(fields)
        nr = C.c_int()
        names = _cstrs([f[0] for f in fields])
        dts = (C.c_int * max(len(fields), 1))(*[DTYPES[f[1]] for f in fields])
        check(lib().vg_model_register_agenttype(self._h, name.encode(), len(fields), names, dts,
                                                _hints(hints), C.byref(nr)))
        t = TypeInfo(name, fields, "agent", nr.value)
        self.types[name] = t
        self.agent_types.append(t)
        return self

    def register_edgetype(self, name, fields=(), *hints, target=None, size=None):
        """register_edgetype!(types, T, hints...; target, size) -- src/ModelTypes.jl:158-230"""
        fields = list(fields)
        e = C.c_int()
        names = _cstrs([f[0] for f in fields])
        dts = (C.c_int * max(len(fields), 1))(*[DTYPES[f[1]] for f in fields])
        tnr = self.types[target].index if target is not None else 0
        check(lib().vg_model_register_edgetype(self._h, name.encode(), len(fields), names, dts,
                                               _hints(hints), tnr, int(size or 0), C.byref(e)))
        t = TypeInfo(name, fields, "edge", e.value)
        hv = C.c_uint()
        check(lib().vg_model_edge_hints(self._h, e.value, C.byref(hv)))
        t.hints = hv.value
        self.types[name] = t
        self.edge_types.append(t)
        return self

    def register_param(self, name, default=0.0):
        check(lib().vg_model_register_param(self._h, name.encode(), float(default)))
        self.params[name] = default
        return self

    def register_global(self, name, default=0.0):
        check(lib().vg_model_register_global(self._h, name.encode(), float(default)))
        self.globals[name] = default
        return self

    def create_model(self, name):
        """create_model(types, name) -- src/Simulation.jl:115-207"""
        check(lib().vg_model_finalize(self._h, name.encode()))
        return Model(self, name)


class Model:
    def __init__(self, types, name):
        self.types = types
        self.name = name

    def __getitem__(self, n):
        return self.types.types[n]

    def has_hint(self, T, hint):
        t = self.types.types[T]
        return bool(t.hints & HINTS[hint if hint.startswith(":") else ":" + hint])


def create_model(types, name):
    return types.create_model(name)


class Simulation:
    def __init__(self, model, name=None, stream=None, _handle=None):
        self.model = model
        self.name = name or model.name
        if _handle is not None:
            self._h = _handle
        else:
            h = C.c_void_p()
            check(lib().vg_sim_create(model.types._h, self.name.encode(),
                                      C.c_void_p(stream) if stream else None, C.byref(h)))
            self._h = h
        self.rasters = {}

    def T(self, name):
        if isinstance(name, TypeInfo):
            return name
        return self.model.types.types[name]

    def close(self):
        if self._h:
            check(lib().vg_sim_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_simulation(model, params=None, globals=None, name=None, stream=None):
    """create_simulation(model, params, globals; name) -- src/Simulation.jl:261-339"""
    sim = Simulation(model, name=name, stream=stream)
    for k, v in (params or {}).items():
        set_param(sim, k, v)
    for k, v in (globals or {}).items():
        set_global(sim, k, v)
    return sim


def finish_simulation(sim):
    sim.close()


def copy_simulation(sim):
    h = C.c_void_p()
    check(lib().vg_sim_copy(sim._h, C.byref(h)))
    c = Simulation(sim.model, name=sim.name, _handle=h)
    c.rasters = dict(sim.rasters)
    return c


def save_simulation(sim, path):
    """Checkpoint of an initialized simulation (the role of write_snapshot,
    src/HDF5.jl:688-715; the library's own file format)."""
    check(lib().vg_sim_save(sim._h, os.fsencode(path)))


def load_simulation(model, path, stream=None):
    """Restore a checkpoint written by save_simulation for the same model
    (the role of read_snapshot!, src/HDF5.jl:1594-1660)."""
    h = C.c_void_p()
    check(lib().vg_sim_load(model.types._h, os.fsencode(path),
                            C.c_void_p(stream) if stream else None, C.byref(h)))
    return Simulation(model, _handle=h)


def finish_init(sim):
    check(lib().vg_finish_init(sim._h))


def num_transitions(sim):
    v = C.c_int64()
    check(lib().vg_sim_num_transitions(sim._h, C.byref(v)))
    return v.value


def disable_transition_checks(sim, disable):
    check(lib().vg_disable_transition_checks(sim._h, int(bool(disable))))


def synchronize(sim):
    check(lib().vg_sim_synchronize(sim._h))


def device_bytes(sim):
    v = C.c_uint64()
    check(lib().vg_sim_device_bytes(sim._h, C.byref(v)))
    return v.value


def set_async(sim, flag):
    check(lib().vg_sim_set_async(sim._h, int(bool(flag))))


def write_agents(sim, T, **fields):
    """Overwrite the first n agents' fields (between transitions) from host arrays."""
    t = sim.T(T)
    n = max([np.size(v) for v in fields.values()] or [0])
    cols = []
    ptrs = (C.c_void_p * max(len(t.fields), 1))()
    for i, (fname, dt) in enumerate(t.fields):
        if fname in fields:
            a = np.ascontiguousarray(np.asarray(fields[fname], dtype=NP_DTYPES[dt]))
            cols.append(a)
            ptrs[i] = a.ctypes.data
    check(lib().vg_write_agents(sim._h, t.index, ptrs, n))


def set_stream(sim, stream):
    check(lib().vg_sim_set_stream(sim._h, C.c_void_p(stream)))


# ------------------------------------------------------------ params/globals
def set_param(sim, name, v):
    check(lib().vg_set_param(sim._h, name.encode(), float(v)))


def param(sim, name):
    v = C.c_double()
    check(lib().vg_param(sim._h, name.encode(), C.byref(v)))
    return v.value


def set_global(sim, name, v):
    check(lib().vg_set_global(sim._h, name.encode(), float(v)))


def get_global(sim, name):
    v = C.c_double()
    check(lib().vg_get_global(sim._h, name.encode(), C.byref(v)))
    return v.value


def bind_param(sim, transition, slot, name, kind="global"):
    """Parameter slot `slot` of every later apply! of `transition` takes the
    current value of this simulation's global (or param) `name` -- the
    transition reads get_global(sim, name) / param(sim, name)."""
    check(lib().vg_bind_param(sim._h, transition.encode(), int(slot),
                              {"param": 0, "global": 1}[kind], name.encode()))


def unbind_params(sim, transition=None):
    check(lib().vg_unbind_params(sim._h, transition.encode() if transition else None))


def push_global(sim, name, v):
    check(lib().vg_push_global(sim._h, name.encode(), float(v)))


def global_series(sim, name):
    n = C.c_uint64()
    check(lib().vg_global_series(sim._h, name.encode(), None, 0, C.byref(n)))
    out = np.zeros(n.value, dtype=np.float64)
    check(lib().vg_global_series(sim._h, name.encode(),
                                 out.ctypes.data_as(C.POINTER(C.c_double)), n.value, C.byref(n)))
    return out


# ------------------------------------------------------------------- agents
def _columns(t, n, values):
    """SoA columns for n values of type t from keyword arrays/scalars."""
    cols = []
    for i, (fname, dt) in enumerate(t.fields):
        v = values.get(fname, 0)
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=NP_DTYPES[dt]), (n,)))
        cols.append(a)
    ptrs = (C.c_void_p * max(len(cols), 1))(*[c.ctypes.data for c in cols])
    return cols, ptrs


def add_agents(sim, T, n=None, **fields):
    """add_agents!(sim, agents) -- src/Agent.jl:174-180 (SoA columns)."""
    t = sim.T(T)
    if n is None:
        n = max([np.size(v) for v in fields.values()] or [1])
    cols, ptrs = _columns(t, n, fields)
    ids = np.zeros(n, dtype=np.uint64)
    check(lib().vg_add_agents(sim._h, t.index, n, ptrs,
                              ids.ctypes.data_as(C.POINTER(C.c_uint64))))
    return ids


def add_agent(sim, T, **fields):
    """add_agent!(sim, agent) -- src/AgentMethods.jl:65-89"""
    return add_agents(sim, T, 1, **fields)[0]


def add_agent_per_process(sim, T, **fields):
    t = sim.T(T)
    cols, ptrs = _columns(t, 1, fields)
    out = C.c_uint64()
    check(lib().vg_add_agent_per_process(sim._h, t.index, ptrs, C.byref(out)))
    return np.uint64(out.value)


def _empty_cols(t, n):
    cols = [np.zeros(n, dtype=NP_DTYPES[dt]) for _, dt in t.fields]
    ptrs = (C.c_void_p * max(len(cols), 1))(*[c.ctypes.data for c in cols])
    return cols, ptrs


def _as_dict(t, cols, i=None):
    if i is None:
        return {f[0]: c for f, c in zip(t.fields, cols)}
    return {f[0]: c[i].item() for f, c in zip(t.fields, cols)}


def agentstate(sim, id, T):
    """agentstate(sim, id, T) -- src/AgentMethods.jl:91-154"""
    t = sim.T(T)
    cols, ptrs = _empty_cols(t, 1)
    check(lib().vg_agentstate(sim._h, int(id), t.index, ptrs))
    return _as_dict(t, cols, 0)


def agentstate_flexible(sim, id):
    """agentstate_flexible(sim, id) -- src/Agent.jl:210-211"""
    t = [x for x in sim.model.types.agent_types if x.index == type_nr(id)][0]
    return agentstate(sim, id, t)


def num_agents(sim, T):
    v = C.c_uint64()
    check(lib().vg_num_agents(sim._h, sim.T(T).index, C.byref(v)))
    return v.value


def agent_slots(sim, T):
    v = C.c_uint64()
    check(lib().vg_agent_slots(sim._h, sim.T(T).index, C.byref(v)))
    return v.value


def read_agents(sim, T):
    """All slots (living and died) of the read state: (dict of columns, died)."""
    t = sim.T(T)
    n = agent_slots(sim, T)
    cols, ptrs = _empty_cols(t, n)
    died = np.zeros(n, dtype=np.uint8)
    out = C.c_uint64()
    check(lib().vg_read_agents(sim._h, t.index, ptrs,
                               died.ctypes.data_as(C.POINTER(C.c_uint8)), n, C.byref(out)))
    return _as_dict(t, cols), died.astype(bool)


def all_agents(sim, T):
    """all_agents(sim, T) -- src/Agent.jl:234-260 (list of dicts)."""
    t = sim.T(T)
    if not t.fields:
        raise AssertionError("all_agents can be only called for agent types that have fields.")
    cols, ids = _all(sim, t)
    return [_as_dict(t, cols, i) for i in range(len(ids))]


def _all(sim, t):
    n = C.c_uint64()
    check(lib().vg_all_agents(sim._h, t.index, None, None, 0, C.byref(n)))
    cols, ptrs = _empty_cols(t, n.value)
    ids = np.zeros(n.value, dtype=np.uint64)
    check(lib().vg_all_agents(sim._h, t.index, ptrs, ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                              n.value, C.byref(n)))
    return cols, ids


def all_agentids(sim, T):
    """all_agentids(sim, T) -- src/Agent.jl:287-313"""
    return _all(sim, sim.T(T))[1]


# -------------------------------------------------------------------- edges
def add_edges(sim, T, frm, to, **payload):
    """add_edge!/add_edges! in bulk -- src/EdgeMethods.jl:388-523."""
    t = sim.T(T)
    to = np.ascontiguousarray(np.atleast_1d(np.asarray(to, dtype=np.uint64)))
    n = to.size
    frm = np.ascontiguousarray(np.broadcast_to(np.asarray(frm, dtype=np.uint64), (n,)))
    cols, ptrs = _columns(t, n, payload)
    check(lib().vg_add_edges(sim._h, t.index, n, frm.ctypes.data_as(C.POINTER(C.c_uint64)),
                             to.ctypes.data_as(C.POINTER(C.c_uint64)),
                             ptrs if t.fields else None))


def add_edge(sim, frm, to, T, **payload):
    """add_edge!(sim, from, to, state); add_edge(sim, to, Edge(from, state), T)
    is the form add_edge!(sim, to, edge) (src/EdgeMethods.jl:388-523)."""
    if isinstance(to, Edge):
        frm, to, payload = to.frm, frm, dict(to.state or {}, **payload)
    add_edges(sim, T, [frm], [to], **payload)


def add_graph(sim, T, E, nv, src, dst, directed=True, agent_fields=None, edge_fields=None):
    """add_graph!(sim, graph, agent_constructor, edge_constructor) --
    src/GraphsSupport.jl:34-57.  nv vertices become agents of type T
    (agent_fields: name -> nv values, or a constant); the edges src[k] ->
    dst[k] (1-based vertex numbers, in the graph's edge order) become edges
    of type E with edge_fields (name -> one value per graph edge, or a
    constant); an undirected graph adds both directions, src -> dst first.
    Returns the new agents' ids."""
    t, e = sim.T(T), sim.T(E)
    src = np.ascontiguousarray(np.asarray(src, dtype=np.uint64).ravel())
    dst = np.ascontiguousarray(np.asarray(dst, dtype=np.uint64).ravel())
    if src.size != dst.size:
        raise ValueError("src and dst differ in length")
    acols, aptrs = _columns(t, nv, agent_fields or {})
    ecols, eptrs = _columns(e, src.size, edge_fields or {})
    ids = np.zeros(nv, dtype=np.uint64)
    check(lib().vg_add_graph(sim._h, t.index, nv, aptrs, e.index, src.size,
                             src.ctypes.data_as(C.POINTER(C.c_uint64)),
                             dst.ctypes.data_as(C.POINTER(C.c_uint64)), 1 if directed else 0,
                             eptrs if e.fields else None,
                             ids.ctypes.data_as(C.POINTER(C.c_uint64))))
    return ids


def remove_edges(sim, to, T, frm=None):
    """remove_edges!(sim, to, T) / remove_edges!(sim, from, to, T) -- src/EdgeMethods.jl:527-599"""
    t = sim.T(T)
    to = np.ascontiguousarray(np.atleast_1d(np.asarray(to, dtype=np.uint64)))
    fp = None
    if frm is not None:
        frm = np.ascontiguousarray(np.broadcast_to(np.asarray(frm, dtype=np.uint64), to.shape))
        fp = frm.ctypes.data_as(C.POINTER(C.c_uint64))
    check(lib().vg_remove_edges(sim._h, t.index, to.size, fp,
                                to.ctypes.data_as(C.POINTER(C.c_uint64))))


class Edge:
    """Edge{T}(from, state) -- src/Edge.jl:31-34"""

    def __init__(self, frm, state):
        self.frm = np.uint64(frm)
        self.state = state

    @property
    def from_(self):
        return self.frm

    def __eq__(self, o):
        return isinstance(o, Edge) and self.frm == o.frm and self.state == o.state

    def __repr__(self):
        return "Edge(%d, %r)" % (int(self.frm), self.state)


def _row(sim, fn, id, t, want_from, want_payload):
    cnt = C.c_int64()
    if fn == "edges":
        check(lib().vg_edges(sim._h, int(id), t.index, None, None, 0, C.byref(cnt)))
    elif fn == "neighborids":
        check(lib().vg_neighborids(sim._h, int(id), t.index, None, 0, C.byref(cnt)))
    else:
        check(lib().vg_edgestates(sim._h, int(id), t.index, None, 0, C.byref(cnt)))
    if cnt.value < 0:
        return None, None, -1
    n = cnt.value
    frm = np.zeros(max(n, 1), dtype=np.uint64)
    cols, ptrs = _empty_cols(t, max(n, 1))
    if fn == "edges":
        check(lib().vg_edges(sim._h, int(id), t.index, frm.ctypes.data_as(C.POINTER(C.c_uint64)),
                             ptrs, n, C.byref(cnt)))
    elif fn == "neighborids":
        check(lib().vg_neighborids(sim._h, int(id), t.index,
                                   frm.ctypes.data_as(C.POINTER(C.c_uint64)), n, C.byref(cnt)))
    else:
        check(lib().vg_edgestates(sim._h, int(id), t.index, ptrs, n, C.byref(cnt)))
    return frm[:n], [c[:n] for c in cols], n


def _state(t, cols, k):
    return {f[0]: c[k].item() for f, c in zip(t.fields, cols)}


def edges(sim, id, T):
    """edges(sim, id, T) -- src/EdgeMethods.jl:705-715"""
    t = sim.T(T)
    frm, cols, n = _row(sim, "edges", id, t, True, True)
    if n < 0:
        return None
    es = [Edge(frm[k], _state(t, cols, k)) for k in range(n)]
    return es[0] if sim.model.has_hint(t.name, ":SingleEdge") else es


def neighborids(sim, id, T):
    """neighborids(sim, id, T) -- src/EdgeMethods.jl:718-742"""
    t = sim.T(T)
    frm, cols, n = _row(sim, "neighborids", id, t, True, False)
    if n < 0:
        return None
    return frm[0] if sim.model.has_hint(t.name, ":SingleEdge") else list(frm)


def neighborids_iter(sim, id, T):
    t = sim.T(T)
    if sim.model.has_hint(t.name, ":SingleEdge") or sim.model.has_hint(t.name, ":IgnoreFrom"):
        raise AssertionError("neighborids_iter is not defined for edgetypes with the "
                             ":SingleEdge or :IgnoreFrom hint")
    r = neighborids(sim, id, T)
    return None if r is None else iter(r)


def edgestates(sim, id, T):
    """edgestates(sim, id, T) -- src/EdgeMethods.jl:805-829"""
    t = sim.T(T)
    frm, cols, n = _row(sim, "edgestates", id, t, False, True)
    if n < 0:
        return None
    es = [_state(t, cols, k) for k in range(n)]
    return es[0] if sim.model.has_hint(t.name, ":SingleEdge") else es


def edgestates_iter(sim, id, T):
    t = sim.T(T)
    if sim.model.has_hint(t.name, ":SingleEdge") or sim.model.has_hint(t.name, ":Stateless"):
        raise AssertionError("edgestates_iter is not defined for edgetypes with the "
                             ":SingleEdge or :Stateless hint")
    r = edgestates(sim, id, T)
    return None if r is None else iter(r)


def neighborstates(sim, id, T, AT):
    """neighborstates(sim, id, T, AT) -- src/EdgeMethods.jl:765-781"""
    ids = neighborids(sim, id, T)
    if ids is None:
        return None
    if sim.model.has_hint(sim.T(T).name, ":SingleEdge"):
        return agentstate(sim, ids, AT)
    return [agentstate(sim, i, AT) for i in ids]


def neighborstates_flexible(sim, id, T):
    """neighborstates_flexible -- src/Edge.jl:303-335"""
    ids = neighborids(sim, id, T)
    if ids is None:
        return None
    if sim.model.has_hint(sim.T(T).name, ":SingleEdge"):
        return agentstate_flexible(sim, ids)
    return [agentstate_flexible(sim, i) for i in ids]


def neighborstates_iter(sim, id, T, AT):
    """neighborstates_iter(sim, id, T, AT) -- src/EdgeMethods.jl:783-803"""
    t = sim.T(T)
    if sim.model.has_hint(t.name, ":SingleEdge") or sim.model.has_hint(t.name, ":IgnoreFrom"):
        raise AssertionError("neighborstates_iter is not defined for edgetypes with the "
                             ":SingleEdge or :IgnoreFrom hint")
    ids = neighborids(sim, id, T)
    return None if ids is None else (agentstate(sim, i, AT) for i in ids)


def neighborstates_flexible_iter(sim, id, T):
    """neighborstates_flexible_iter -- src/Edge.jl:328-335: no check of its
    own; :IgnoreFrom fails in neighborids, and the single id of a
    :SingleEdge row is iterated as one element, as a Julia number is."""
    ids = neighborids(sim, id, T)
    if ids is None:
        return None
    if sim.model.has_hint(sim.T(T).name, ":SingleEdge"):
        ids = [ids]
    return (agentstate_flexible(sim, i) for i in ids)


def num_edges(sim, id_or_T, T=None, write=None):
    """num_edges(sim, id, T) -- src/EdgeMethods.jl:851-869 and
    num_edges(sim, T; write) -- src/Edge.jl:373-389"""
    if T is None:
        t = sim.T(id_or_T)
        v = C.c_uint64()
        w = 0 if write is False else 1 if write else -1
        if w < 0:
            w = 1  # before finish_init! the write container, after it both agree
            initialized = num_transitions(sim) > 0
            w = 0 if initialized else 1
        check(lib().vg_num_edges_total(sim._h, t.index, w, C.byref(v)))
        return v.value
    t = sim.T(T)
    v = C.c_int64()
    check(lib().vg_num_edges(sim._h, int(id_or_T), t.index, C.byref(v)))
    return v.value


def has_edge(sim, id, T):
    """has_edge(sim, id, T) -- src/EdgeMethods.jl:873-892"""
    v = C.c_int()
    check(lib().vg_has_edge(sim._h, int(id), sim.T(T).index, C.byref(v)))
    return bool(v.value)


def read_edges(sim, E, T):
    """Bulk read of edge type E's CSR over target type T: (row_ptr, from, payload)."""
    e, t = sim.T(E), sim.T(T)
    nr, ne = C.c_uint64(), C.c_uint64()
    check(lib().vg_read_edges(sim._h, e.index, t.index, None, None, None, C.byref(nr),
                              C.byref(ne)))
    rp = np.zeros(nr.value + 1, dtype=np.uint64)
    frm = np.zeros(max(ne.value, 1), dtype=np.uint64)
    cols, ptrs = _empty_cols(e, max(ne.value, 1))
    check(lib().vg_read_edges(sim._h, e.index, t.index, rp.ctypes.data_as(C.POINTER(C.c_uint64)),
                              frm.ctypes.data_as(C.POINTER(C.c_uint64)),
                              ptrs if e.fields else None, C.byref(nr), C.byref(ne)))
    return rp, frm[:ne.value], {f[0]: c[:ne.value] for f, c in zip(e.fields, cols)}


# -------------------------------------------------------------- transitions
def transition_names():
    return lib().vg_transition_names().decode().split(",")


def _refs(sim, xs):
    if xs is None:
        return []
    if isinstance(xs, (str, TypeInfo)):
        xs = [xs]
    return [sim.T(x).ref for x in xs]


def _apply_args(sim, transition, call, read, write, add_existing, with_edge, params):
    c, r, w, a = (_refs(sim, call), _refs(sim, read), _refs(sim, write),
                  _refs(sim, add_existing))
    arr = lambda v: (C.c_int * max(len(v), 1))(*v)
    p = (C.c_double * max(len(params), 1))(*[float(x) for x in params])
    we = sim.T(with_edge).index if with_edge is not None else -1
    return (transition.encode(), arr(c), len(c), arr(r), len(r), arr(w), len(w), arr(a),
            len(a), we, p, len(params))


def _key(x):
    # lists become tuples; names, numbers and TypeInfo objects (hashed by
    # identity, and unique per model) are their own keys
    return tuple(x) if type(x) is list else x


def apply_(sim, transition, call, read, write, add_existing=(), with_edge=None, params=()):
    """apply!(sim, f, call, read, write; add_existing, with_edge) -- src/Simulation.jl:720-821

    The marshalled C arguments of a call are kept per simulation, keyed by
    the arguments, so that a step loop repeating the same apply! pays the
    conversion once."""
    cache = sim.__dict__.setdefault("_apply_cache", {})
    try:
        key = (transition, _key(call), _key(read), _key(write), _key(add_existing),
               _key(with_edge), _key(params))
        args = cache.get(key)
    except TypeError:  # an unhashable argument: marshal every time
        key, args = None, None
    if args is None:
        args = _apply_args(sim, transition, call, read, write, add_existing, with_edge, params)
        if key is not None:
            if len(cache) >= 64:
                cache.clear()
            cache[key] = args
    check(lib().vg_apply(sim._h, *args))
    return sim


class PreparedApply:
    """apply!(sim, transition, call, read, write, ...) prepared once in the
    library (vg_apply_prepare) and run by a call with one argument
    (vg_apply_call_run): the same vg_apply call each time (params or
    globals bound to parameter slots still take their values at each run)."""

    def __init__(self, sim, transition, call, read, write, add_existing=(), with_edge=None,
                 params=()):
        self._sim = sim
        self._h = None
        args = _apply_args(sim, transition, call, read, write, add_existing, with_edge, params)
        h = C.c_void_p()
        check(lib().vg_apply_prepare(sim._h, *args, C.byref(h)))
        self._h = h.value
        self._run = lib().vg_apply_call_run

    def __call__(self):
        if self._sim._h is None:
            raise RuntimeError("the simulation of this prepared apply! is closed")
        rc = self._run(self._h)
        if rc:
            check(rc)
        return self._sim

    def close(self):
        if self._h:
            lib().vg_apply_call_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prepare_apply(sim, transition, call, read, write, add_existing=(), with_edge=None,
                  params=()):
    """A callable that runs apply_(sim, transition, call, read, write, ...)
    with these arguments, prepared in the library once: the cheapest form of
    a step loop that repeats one apply! (params or globals bound to
    parameter slots still take their values at each call)."""
    return PreparedApply(sim, transition, call, read, write, add_existing, with_edge, params)


def apply_host(sim, transition, call, read, write, T, state, out=None, add_existing=(),
               with_edge=None, params=()):
    """apply! with type T's state kept in host memory (vg_apply_host): the
    columns in `state` (field name -> array of n values) are uploaded, the
    transition runs, and the new state of those n agents is written into
    `out` (field name -> preallocated array; allocated when None) and
    returned.  Pinned arrays (e.g. torch pin_memory tensors' numpy views) let
    the download overlap the transition's kernels."""
    t = sim.T(T)
    n = max([np.size(v) for v in state.values()] or [0])
    keep, ptr_in = [], (C.c_void_p * max(len(t.fields), 1))()
    for i, (fname, dt) in enumerate(t.fields):
        if fname in state:
            a = np.ascontiguousarray(np.asarray(state[fname], dtype=NP_DTYPES[dt]))
            keep.append(a)
            ptr_in[i] = a.ctypes.data
    if out is None:
        out = {f: np.empty(n, dtype=NP_DTYPES[dt]) for f, dt in t.fields}
    ptr_out = (C.c_void_p * max(len(t.fields), 1))()
    for i, (fname, dt) in enumerate(t.fields):
        if fname in out:
            a = out[fname]
            if a.dtype != np.dtype(NP_DTYPES[dt]) or not a.flags.c_contiguous or a.size < n:
                raise ValueError("out[%r]: %d contiguous values of %s" % (fname, n, dt))
            ptr_out[i] = a.ctypes.data
    args = _apply_args(sim, transition, call, read, write, add_existing, with_edge, params)
    check(lib().vg_apply_host(sim._h, *args, t.index, ptr_in, ptr_out, n))
    return out


def apply(sim, transition, call, read, write, **kw):
    """apply(sim, f, call, read, write) -- src/Simulation.jl:847-856 (on a copy)"""
    c = copy_simulation(sim)
    apply_(c, transition, call, read, write, **kw)
    return c


def mapreduce(sim, f, op, T, init=None, datatype=None, ordered=None):
    """mapreduce(sim, f, op, T; init, datatype) -- src/AgentMethods.jl:533-565,
    src/EdgeMethods.jl:972-1001.  `f` is a field name or (cmp, field, value)
    with cmp in ==, !=, <, >.

    ordered=None (default): Float + and * fold sequentially in the
    reference's order (bit-identical), every order-independent reduction
    takes a parallel tree.  ordered=True forces the sequential fold,
    ordered=False the tree (Float + and *: within 2 (n - 1) 2^-53 sum|f(x)|
    of the sequential result)."""
    t = sim.T(T)
    if isinstance(f, str):
        kind, field, arg = MAPS["field"], t.field_index(f), 0.0
        dt = t.fields[field][1]
    else:
        kind, field, arg = MAPS[f[0]], t.field_index(f[1]), float(f[2])
        dt = "bool"
    if datatype is None:
        datatype = "bool" if op in ("&", "|") else "i64"
    if dt in ("f32", "f64") and kind == MAPS["field"]:
        out_dt, out = 11, C.c_double()
    elif dt == "bool" and datatype == "bool" and op in ("&", "|", "max", "min"):
        out_dt, out = 1, C.c_uint8()
    else:
        out_dt, out = 9, C.c_int64()
    if datatype == "bool" and op in ("&", "|") and dt not in ("bool",) and kind == 0:
        out_dt, out = 9, C.c_int64()
    opc = OPS[op] | {None: 0, True: 0x100, False: 0x200}[ordered]
    fn = lib().vg_mapreduce_agents if t.kind == "agent" else lib().vg_mapreduce_edges
    check(fn(sim._h, t.index, field, kind, arg, opc, out_dt, int(init is not None),
             float(init or 0), C.byref(out)))
    v = out.value
    return bool(v) if out_dt == 1 else v


# ------------------------------------------------------------------ rasters
def add_raster(sim, name, dims, T, **fields):
    """add_raster!(sim, name, dims, constructor) -- src/Raster.jl:32-54.
    Field values are given column-major (first index fastest), or as arrays
    of shape `dims` (converted with order='F')."""
    t = sim.T(T)
    dims = tuple(int(d) for d in dims)
    n = int(np.prod(dims))
    flat = {}
    for k, v in fields.items():
        a = np.asarray(v)
        flat[k] = a.reshape(-1, order="F") if a.shape == dims else a
    cols, ptrs = _columns(t, n, flat)
    d = (C.c_int64 * len(dims))(*dims)
    ids = np.zeros(n, dtype=np.uint64)
    check(lib().vg_add_raster(sim._h, name.encode(), len(dims), d, t.index, ptrs,
                              ids.ctypes.data_as(C.POINTER(C.c_uint64))))
    sim.rasters[name] = dims
    return ids.reshape(dims, order="F")


def _payload_ptrs(t, payload):
    if not t.fields:
        return None, None
    cols, ptrs = _columns(t, 1, payload)
    return cols, ptrs


def connect_raster_neighbors(sim, name, E, distance=1, metric="chebyshev", periodic=True,
                             implicit=False, **payload):
    """connect_raster_neighbors!(sim, name, ctor; distance, metric, periodic) --
    src/Raster.jl:139-167 (constant edge state)."""
    t = sim.T(E)
    cols, ptrs = _payload_ptrs(t, payload)
    check(lib().vg_connect_raster_neighbors(sim._h, name.encode(), t.index, ptrs,
                                            float(distance), METRICS[metric], int(periodic),
                                            int(implicit)))


def move_to(sim, name, id, pos, edge_from_raster, edge_to_raster, distance=0,
            metric="chebyshev", periodic=True, only_surrounding=False, payload_from=None,
            payload_to=None):
    """move_to!(sim, name, id, pos, edge_from_raster, edge_to_raster; ...) -- src/Raster.jl:437-477"""
    ef = sim.T(edge_from_raster).index if edge_from_raster is not None else -1
    et = sim.T(edge_to_raster).index if edge_to_raster is not None else -1
    pf = _payload_ptrs(sim.T(edge_from_raster), payload_from or {})[1] if ef >= 0 else None
    pt = _payload_ptrs(sim.T(edge_to_raster), payload_to or {})[1] if et >= 0 else None
    p = (C.c_int64 * len(pos))(*[int(x) for x in pos])
    check(lib().vg_move_to(sim._h, name.encode(), int(id), p, ef, pf, et, pt, float(distance),
                           METRICS[metric], int(periodic), int(only_surrounding)))


def cellid(sim, name, pos):
    p = (C.c_int64 * len(pos))(*[int(x) for x in pos])
    out = C.c_uint64()
    check(lib().vg_cellid(sim._h, name.encode(), p, C.byref(out)))
    return np.uint64(out.value)


def _raster_dims(sim, name):
    if name not in sim.rasters:  # e.g. a simulation restored from a checkpoint
        dims = (C.c_int64 * 4)()
        nd = C.c_int()
        check(lib().vg_raster_dims(sim._h, name.encode(), dims, C.byref(nd)))
        sim.rasters[name] = tuple(dims[k] for k in range(nd.value))
    return sim.rasters[name]


def rastervalues(sim, name, field):
    """rastervalues(sim, name, field) -- src/Raster.jl:353-387 (array of shape dims)"""
    dims = _raster_dims(sim, name)
    ids = cellid(sim, name, [1] * len(dims))
    t = [x for x in sim.model.types.agent_types if x.index == type_nr(ids)][0]
    f = t.field_index(field)
    out = np.zeros(int(np.prod(dims)), dtype=t.dtype(f))
    check(lib().vg_rastervalues(sim._h, name.encode(), f, out.ctypes.data_as(C.c_void_p)))
    return out.reshape(dims, order="F")


def calc_rasterstate(sim, name, field, f_returns=None, T=None):
    """calc_rasterstate(sim, name, c -> c.field) -- src/Raster.jl:282-327"""
    return rastervalues(sim, name, field)
