"""ORACLE -- test infrastructure only.

A pure-Python restatement of Vahana.jl v1.4.7's state machine for the
transition step, with the reference's own container types and checks, used
to pin expected results (against the reference's known-answer tests, which
are ported in tests/test_oracle_kat.py) and as the checker of the GPU
library's generic engine on small cases.  Never imported by the product.

Restated from (paths in the reference source tree):
  containers per hint      src/EdgeMethods.jl:9-91   (construct_types)
  add_edge! / _can_add     src/EdgeMethods.jl:257-294, 375-523
  remove_edges!            src/EdgeMethods.jl:527-631, 897-920
  accessors                src/EdgeMethods.jl:705-892, src/Edge.jl:303-335
  agent ids                src/Agent.jl:30-115
  _get_next_id / add_agent! src/AgentMethods.jl:37-89
  agentstate               src/AgentMethods.jl:91-154
  sweep / write            src/AgentMethods.jl:159-268
  prepare/finish_write!    src/AgentMethods.jl:271-439, src/EdgeMethods.jl:639-684
  apply!                   src/Simulation.jl:720-821
  finish_init!             src/Simulation.jl:403-476 (one process)
  mapreduce / val4empty    src/AgentMethods.jl:533-565, src/EdgeMethods.jl:972-1001,
                           src/Helpers.jl:44-81
  raster                   src/Raster.jl:32-54, 82-167, 403-499
"""
import copy
import itertools
import math

SHIFT_TYPE, SHIFT_RANK = 56, 36
NR_MASK = (1 << 36) - 1
INT64_MAX = (1 << 63) - 1


def agent_id(type_nr, nr):
    return (type_nr << SHIFT_TYPE) | nr


def type_nr(id):
    return id >> SHIFT_TYPE


def agent_nr(id):
    return id & NR_MASK


class Edge:
    __slots__ = ("frm", "state")

    def __init__(self, frm, state):
        self.frm = frm
        self.state = state

    def __eq__(self, o):
        return isinstance(o, Edge) and self.frm == o.frm and self.state == o.state

    def __repr__(self):
        return "Edge(%d, %r)" % (self.frm, self.state)


class ModelTypes:
    def __init__(self):
        self.atypes = []  # (name, fields, hints)
        self.etypes = {}  # name -> dict
        self.anr = {}

    def register_agenttype(self, name, fields=(), *hints):
        hints = set(h if h.startswith(":") else ":" + h for h in hints)
        for h in hints:
            assert h in (":Immortal", ":Independent"), "The agent type hint %s is unknown" % h
        assert name not in self.anr, "Type %s is already registered" % name
        self.atypes.append({"name": name, "fields": [f[0] for f in fields], "hints": hints})
        self.anr[name] = len(self.atypes)
        return self

    def register_edgetype(self, name, fields=(), *hints, target=None, size=None):
        hints = set(h if h.startswith(":") else ":" + h for h in hints)
        if ":NumEdgesOnly" in hints:
            hints |= {":Stateless", ":IgnoreFrom"}
        if ":HasEdgeOnly" in hints:
            hints |= {":Stateless", ":IgnoreFrom", ":SingleEdge"}
        if ":SingleType" in hints:
            assert target is not None, "the :SingleType hint needs the target keyword"
        if target is not None:
            hints.add(":SingleType")
        if not fields:
            hints.add(":Stateless")  # detect_stateless
        assert not (":SingleType" in hints and ":SingleEdge" in hints and
                    not (":Stateless" in hints and ":IgnoreFrom" in hints)), \
            "The hints :SingleEdge and :SingleType can be only combined when the type has " \
            "also the hints :Stateless and :IgnoreFrom."
        self.etypes[name] = {"name": name, "fields": [f[0] for f in fields], "hints": hints,
                             "target": target, "size": size or 0}
        return self

    def create_model(self, name):
        return self


class _RW:
    def __init__(self):
        self.state = []
        self.reuse = []
        self.died = []


class Sim:
    """create_simulation -- src/Simulation.jl:261-339"""

    def __init__(self, model):
        self.m = model
        self.initialized = False
        self.intransition = False
        self.check_readable = True
        self.num_transitions = 0
        self.rasters = {}
        self.A = {}
        for a in model.atypes:
            self.A[a["name"]] = {"read": _RW(), "write": _RW(), "nextid": 1, "prepared": False,
                                 "writeable": False, "info": a}
        self.E = {}
        for n, e in model.etypes.items():
            self.E[n] = {"read": self._new_container(e), "write": self._new_container(e),
                         "readable": False, "writeable": False, "add_existing": False,
                         "aot": {}, "info": e}

    # ------------------------------------------------------------ helpers
    def hints(self, E):
        return self.m.etypes[E]["hints"]

    def _new_container(self, e):
        if ":SingleType" in e["hints"]:
            c = [None] * e["size"]
            if self._bits_ct(e):
                c = [self._zero_ct(e)] * e["size"]
            return c
        return {}

    def _bits_ct(self, e):
        h = e["hints"]
        return (":Stateless" in h and ":IgnoreFrom" in h) or (":SingleEdge" in h)

    def _zero_ct(self, e):
        h = e["hints"]
        if ":Stateless" in h and ":IgnoreFrom" in h and ":SingleEdge" in h:
            return False
        if ":Stateless" in h and ":IgnoreFrom" in h:
            return 0
        if ":SingleEdge" in h:
            return None  # isbitstype element: reads back as zero / unassigned
        return []

    def tnr(self, T):
        return self.m.anr[T]

    def tname(self, nr):
        return self.m.atypes[nr - 1]["name"]

    def immortal(self, T):
        return ":Immortal" in self.m.atypes[self.tnr(T) - 1]["hints"]

    def _value(self, E, frm, state):
        h = self.hints(E)
        if ":Stateless" in h and ":IgnoreFrom" in h and ":SingleEdge" in h:
            return True
        if ":IgnoreFrom" in h:
            return state
        if ":Stateless" in h:
            return frm
        return Edge(frm, state)

    def _key(self, E, to):
        return agent_nr(to) - 1 if ":SingleType" in self.hints(E) else to

    def _get(self, E, field, to):
        """_get_agent_container (src/EdgeMethods.jl:303-371): None if absent"""
        e = self.m.etypes[E]
        if ":SingleType" in e["hints"]:
            assert self.tname(type_nr(to)) == e["target"], \
                "The :SingleType hint is set for %s" % E
            nr = agent_nr(to)
            if nr > len(field):
                if self._bits_ct(e) and self._zero_ct(e) is not None:
                    return self._zero_ct(e)
                return None
            return field[nr - 1]
        return field.get(to)

    def _get_or_make(self, E, field, to):
        e = self.m.etypes[E]
        if ":SingleType" in e["hints"]:
            nr = agent_nr(to)
            while len(field) < nr:
                field.append(self._zero_ct(e) if self._bits_ct(e) else None)
            if field[nr - 1] is None and not self._bits_ct(e):
                field[nr - 1] = []
            return field[nr - 1]
        if to not in field:
            z = self._zero_ct(e)
            field[to] = [] if z == [] else z
        return field[to]

    def _set(self, E, field, to, v):
        e = self.m.etypes[E]
        if ":SingleType" in e["hints"]:
            nr = agent_nr(to)
            while len(field) < nr:
                field.append(self._zero_ct(e) if self._bits_ct(e) else None)
            field[nr - 1] = v
        else:
            field[to] = v


def create_simulation(model):
    return Sim(model)


def disable_transition_checks(sim, disable):
    sim.check_readable = not disable
    sim.intransition = disable


# ------------------------------------------------------------------ agents
def _next_id(sim, T):
    A = sim.A[T]
    mortal = not sim.immortal(T)
    if mortal and A["read"].reuse:
        nr = A["read"].reuse.pop()
        A["write"].died[nr - 1] = False
        return nr
    nr = A["nextid"]
    A["nextid"] = nr + 1
    w = A["write"]
    while len(w.state) < nr:
        w.state.append(None)
        if mortal:
            w.died.append(False)
    if mortal:
        w.died[nr - 1] = False
    return nr


def add_agent(sim, T, state):
    assert (not sim.initialized) or sim.intransition, \
        "You can call add_agent! only in the initialization phase"
    assert (not sim.initialized) or sim.A[T]["writeable"], \
        "%s must be in the `write` argument of the transition function." % T
    nr = _next_id(sim, T)
    sim.A[T]["write"].state[nr - 1] = dict(state)
    return agent_id(sim.tnr(T), nr)


def add_agents(sim, T, states):
    return [add_agent(sim, T, s) for s in states]


def agentstate(sim, id, T):
    assert type_nr(id) == sim.tnr(T), "The id of the agent does not match the given type"
    A = sim.A[T]
    assert A["prepared"] or not sim.check_readable, \
        "%s must be in the `read` argument of the transition function." % T
    nr = agent_nr(id)
    if not sim.immortal(T):
        assert not A["read"].died[nr - 1], \
            "agentstate was requested for agent %d that has been removed" % id
    return A["read"].state[nr - 1]


def agentstate_flexible(sim, id):
    return agentstate(sim, id, sim.tname(type_nr(id)))


def num_agents(sim, T):
    A = sim.A[T]
    if sim.immortal(T):
        return A["nextid"] - 1
    d = A["read"].died if sim.initialized else A["write"].died
    return sum(1 for x in d if not x)


def all_agents(sim, T):
    A = sim.A[T]
    rw = A["read"] if sim.initialized else A["write"]
    if sim.immortal(T):
        return list(rw.state)
    return [s for s, d in zip(rw.state, rw.died) if not d]


def all_agentids(sim, T):
    A = sim.A[T]
    rw = A["read"] if sim.initialized else A["write"]
    nr = sim.tnr(T)
    if sim.immortal(T):
        return [agent_id(nr, i + 1) for i in range(len(rw.state))]
    return [agent_id(nr, i + 1) for i, d in enumerate(rw.died) if not d]


# ------------------------------------------------------------------- edges
def add_edge(sim, frm, to, E, state=None):
    """add_edge!(sim, from, to, state) -- src/EdgeMethods.jl:388-523"""
    e = sim.m.etypes[E]
    h = e["hints"]
    Es = sim.E[E]
    assert (not sim.check_readable) or (not sim.initialized) or Es["writeable"], \
        "%s must be in the `write` argument of the transition function." % E
    assert (not sim.initialized) or sim.intransition, \
        "You can call add_edge! only in the initialization phase"
    field = Es["write"]
    if ":SingleType" not in h:
        assert 1 <= type_nr(to) <= len(sim.m.atypes), "invalid agent id"
    value = sim._value(E, frm, state)
    stateless, ignore, single = ":Stateless" in h, ":IgnoreFrom" in h, ":SingleEdge" in h
    if single and ":SingleType" not in h and not (ignore and stateless):
        key = sim._key(E, to)
        if key in field:
            assert field[key] == value, \
                "An edge has already been added to the agent with the id %d" % to
    # _push_agentsontarget
    if not ignore and not all(":Immortal" in a["hints"] for a in sim.m.atypes):
        if not sim.immortal(sim.tname(type_nr(frm))):
            Es["aot"].setdefault(frm, []).append(to)
    if stateless and ignore and not single:
        sim._set(E, field, to, sim._get_or_make(E, field, to) + 1)
    elif single:
        if ":SingleType" in h:
            sim._get_or_make(E, field, to)
        sim._set(E, field, to, value)
    else:
        sim._get_or_make(E, field, to).append(value)


def add_edges(sim, to, edges, E):
    for ed in edges:
        add_edge(sim, ed.frm, to, E, ed.state)


def remove_edges(sim, to, E, frm=None):
    """remove_edges! -- src/EdgeMethods.jl:527-599"""
    e = sim.m.etypes[E]
    h = e["hints"]
    field = sim.E[E]["write"]
    if frm is None:
        if ":SingleType" in h:
            sim._set(E, field, to, sim._zero_ct(e) if sim._bits_ct(e) else [])
        else:
            field.pop(to, None)
        return
    assert ":IgnoreFrom" not in h, \
        "remove_edges! with a source agent is not defined for edgetypes with the :IgnoreFrom hint."
    cur = sim._get(E, field, to) if (":SingleType" not in h or agent_nr(to) <= len(field)) else None
    if ":SingleEdge" in h:
        if cur is not None:
            f = cur if ":Stateless" in h else cur.frm
            if f == frm:
                remove_edges(sim, to, E)
    else:
        if cur is not None and len(cur) > 0:
            if ":Stateless" in h:
                new = [x for x in cur if x != frm]
            else:
                new = [x for x in cur if x.frm != frm]
            sim._set(E, field, to, new)


def _readable(sim, E):
    assert sim.E[E]["readable"] or not sim.check_readable, \
        "You try to access an edge of type %s but the type is not in the `read` argument " \
        "of the apply! function." % E


def _container(sim, id, E):
    _readable(sim, E)
    return sim._get(E, sim.E[E]["read"], id)


def edges(sim, id, E):
    h = sim.hints(E)
    assert ":Stateless" not in h and ":IgnoreFrom" not in h, \
        "edges is not defined for the hint combination of %s" % E
    c = _container(sim, id, E)
    return c


def neighborids(sim, id, E):
    h = sim.hints(E)
    assert ":IgnoreFrom" not in h, "neighborids is not defined for the hint combination of %s" % E
    c = _container(sim, id, E)
    if c is None:
        return None
    if ":Stateless" in h:
        return c
    if ":SingleEdge" in h:
        return c.frm
    return [x.frm for x in c]


def neighborstates(sim, id, E, T):
    ids = neighborids(sim, id, E)
    if ids is None:
        return None
    if ":SingleEdge" in sim.hints(E):
        return agentstate(sim, ids, T)
    return [agentstate(sim, i, T) for i in ids]


def neighborstates_flexible(sim, id, E):
    ids = neighborids(sim, id, E)
    if ids is None:
        return None
    if ":SingleEdge" in sim.hints(E):
        return agentstate_flexible(sim, ids)
    return [agentstate_flexible(sim, i) for i in ids]


def edgestates(sim, id, E):
    h = sim.hints(E)
    assert ":Stateless" not in h, "edgestates is not defined for the hint combination of %s" % E
    c = _container(sim, id, E)
    if c is None:
        return None
    if ":IgnoreFrom" in h:
        return c
    if ":SingleEdge" in h:
        return c.state
    return [x.state for x in c]


def num_edges(sim, id, E):
    h = sim.hints(E)
    assert ":SingleEdge" not in h, "num_edges is not defined for the hint combination of %s" % E
    c = _container(sim, id, E)
    if ":IgnoreFrom" in h and ":Stateless" in h:
        return 0 if c is None else c
    return 0 if c is None else len(c)


def has_edge(sim, id, E):
    h = sim.hints(E)
    if ":IgnoreFrom" in h and ":Stateless" in h:
        c = _container(sim, id, E)
        return not (c is None or c == 0 or c is False)
    if ":SingleEdge" not in h:
        return num_edges(sim, id, E) >= 1
    assert ":SingleType" not in h, "has_edge is not defined for the hint combination of %s" % E
    _readable(sim, E)
    return id in sim.E[E]["read"]


def _elements(sim, E, field):
    e = sim.m.etypes[E]
    h = e["hints"]
    items = field if isinstance(field, list) else list(field.values())
    out = []
    for c in items:
        if c is None:
            continue
        if ":SingleEdge" in h or (":Stateless" in h and ":IgnoreFrom" in h):
            out.append(c)
        else:
            out.extend(c)
    return out


def num_edges_total(sim, E, write=None):
    """num_edges(sim, T; write) -- src/Edge.jl:373-389, _num_edges :931-969"""
    if write is None:
        write = not sim.initialized
    field = sim.E[E]["write"] if write else sim.E[E]["read"]
    h = sim.hints(E)
    items = field if isinstance(field, list) else list(field.values())
    if ":IgnoreFrom" in h and ":Stateless" in h:
        return sum(int(c) for c in items if c)
    if ":SingleEdge" in h:
        return sum(1 for c in items if c is not None and c is not False)
    return sum(len(c) for c in items if c is not None)


# ------------------------------------------------------------------ reduce
def val4empty(op, init=None, datatype=None):
    """src/Helpers.jl:44-81"""
    if init is not None:
        return init
    mt = datatype or ("bool" if op in ("&", "|") else "int")
    tmax = True if mt == "bool" else INT64_MAX
    return {"+": 0, "*": 1, "max": -tmax, "min": tmax, "&": tmax,
            "|": (False if mt == "bool" else 0)}[op]


def _op(op):
    return {"+": lambda a, b: a + b, "*": lambda a, b: a * b, "max": max, "min": min,
            "&": lambda a, b: a & b, "|": lambda a, b: a | b}[op]


def _wrap64(v):
    if isinstance(v, bool) or not isinstance(v, int):
        return v
    v &= (1 << 64) - 1
    return v - (1 << 64) if v >> 63 else v


def mapreduce(sim, f, op, T, init=None, datatype=None):
    """agents: src/AgentMethods.jl:533-565; edges: src/EdgeMethods.jl:972-1001"""
    assert not sim.intransition or not sim.check_readable, \
        "You can not call mapreduce inside of a transition function."
    red = val4empty(op, init, datatype)
    fn = _op(op)
    if T in sim.A:
        A = sim.A[T]
        for i in range(A["nextid"] - 1):
            if not sim.immortal(T) and A["read"].died[i]:
                continue
            red = _wrap64(fn(f(A["read"].state[i]), red))
        return red
    h = sim.hints(T)
    assert ":Stateless" not in h, "mapreduce is not defined for the hint combination of %s" % T
    for x in _elements(sim, T, sim.E[T]["read"]):
        v = x if ":IgnoreFrom" in h else x.state
        red = _wrap64(fn(f(v), red))
    return red


# ----------------------------------------------------------- finish_write
def _finish_write_agent(sim, T):
    A = sim.A[T]
    w = A["write"]
    if not sim.immortal(T):
        tnr = sim.tnr(T)
        aids = [agent_id(tnr, nr) for nr in w.reuse]
        for id in aids:
            for E in sim.E:
                _remove_edges_agent_target(sim, id, E)
        if aids:
            for E in sim.E:
                _remove_edges_agent_source(sim, aids, E)
    A["read"].state = list(w.state)
    if not sim.immortal(T):
        A["read"].died = list(w.died)
    A["read"].reuse = A["read"].reuse + w.reuse
    w.reuse = []
    A["writeable"] = False


def _remove_edges_agent_target(sim, to, E):
    e = sim.m.etypes[E]
    field = sim.E[E]["write"]
    if ":SingleType" in e["hints"]:
        if sim.tname(type_nr(to)) == e["target"] and len(field) >= agent_nr(to):
            field[agent_nr(to) - 1] = sim._zero_ct(e) if sim._bits_ct(e) else []
    else:
        field.pop(to, None)


def _remove_edges_agent_source(sim, frm_list, E):
    if ":IgnoreFrom" in sim.hints(E):
        return
    aot = sim.E[E]["aot"]
    keep = sim.check_readable
    sim.check_readable = False
    for f in frm_list:
        if f in aot:
            for t in aot[f]:
                remove_edges(sim, t, E, frm=f)
            del aot[f]
    sim.check_readable = keep


def _finish_write_edge(sim, E):
    Es = sim.E[E]
    Es["read"] = Es["write"]
    Es["writeable"] = False


def finish_init(sim):
    """finish_init! (one process) -- src/Simulation.jl:403-476"""
    assert not sim.initialized, "You can not call finish_init! twice for the same simulation"
    for a in sim.m.atypes:
        _finish_write_agent(sim, a["name"])
    for E in sim.E:
        _finish_write_edge(sim, E)
    sim.initialized = True
    sim.num_transitions = 1


# ------------------------------------------------------------------ apply!
def apply_(sim, f, call, read, write, add_existing=(), with_edge=None):
    """apply! -- src/Simulation.jl:720-821"""
    assert sim.initialized, "You must call finish_init! before apply!"
    if with_edge is not None:
        assert ":SingleType" not in sim.hints(with_edge), \
            "The `with_edge` keyword can only be used for edgetypes without the :SingleType hint."
    sim.intransition = True
    call, read, write, add_existing = (list(x if isinstance(x, (list, tuple)) else [x])
                                       for x in (call, read, write, add_existing))
    for c in call:
        assert c not in add_existing, "%s can not be element of `add_existing`" % c
    for ae in add_existing:
        assert ae in write, "%s is in `add_existing` but not in `write`" % ae
    for T in read:
        if T in sim.E:
            sim.E[T]["readable"] = True
        else:
            sim.A[T]["prepared"] = True
    for T in write:
        if T in sim.E and T not in add_existing:
            sim.E[T]["aot"] = {}
    aex_all = call + add_existing
    for T in write:
        if T in sim.A:
            ae = T in aex_all
            if sim.immortal(T) and sim.initialized:
                assert ae, ("You can add %s to the `write` argument only when %s is also "
                            "included in the `add_existing` argument, as %s has the hint "
                            ":Immortal." % (T, T, T))
            A = sim.A[T]
            if not ae:
                A["read"], A["write"] = _RW(), _RW()
                A["nextid"] = 1
            A["writeable"] = True
        else:
            Es = sim.E[T]
            if T in add_existing:
                Es["write"] = copy.deepcopy(Es["read"]) if T in read else Es["read"]
            else:
                Es["write"] = sim._new_container(sim.m.etypes[T])
            Es["writeable"] = True
            Es["add_existing"] = T in add_existing
    for C in call:
        A = sim.A[C]
        tnr = sim.tnr(C)
        mortal = not sim.immortal(C)
        if with_edge is None:
            idxs = range(len(A["read"].state))
        else:
            idxs = [agent_nr(id) - 1 for id in list(sim.E[with_edge]["read"].keys())
                    if type_nr(id) == tnr]
        for i in idxs:
            if with_edge is None and mortal and A["read"].died[i]:
                continue
            id = agent_id(tnr, i + 1)
            arg = A["read"].state[i] if C in read else ("Val", C)
            new = f(arg, id, sim)
            if C in write:
                if not mortal:
                    assert new is not None, "You can not return `nothing` for immortal agents"
                    A["write"].state[i] = new
                elif new is None:
                    A["write"].reuse.append(i + 1)
                    A["write"].died[i] = True
                else:
                    A["write"].state[i] = new
    for T in read:
        if T in sim.E:
            sim.E[T]["readable"] = False
        else:
            sim.A[T]["prepared"] = False
    for T in write:
        if T in sim.A:
            _finish_write_agent(sim, T)
    for T in write:
        if T in sim.E:
            _finish_write_edge(sim, T)
    sim.intransition = False
    sim.num_transitions += 1
    return sim


# ------------------------------------------------------------------ raster
def _stencil(metric, n, distance):
    """stencil -- src/Raster.jl:82-110 (first dimension fastest, zero removed)"""
    d = int(math.floor(distance))
    out = []
    for t in itertools.product(*[range(-d, d + 1)] * n):
        s = tuple(reversed(t))  # Iterators.product: first index fastest
        if all(x == 0 for x in s):
            continue
        if metric == "euclidean" and not math.sqrt(sum(x * x for x in s)) <= distance:
            continue
        if metric == "manhatten" and not sum(abs(x) for x in s) <= distance:
            continue
        out.append(s)
    return out


def _checkpos(pos, dims, periodic):
    oob = any(p < 1 or p > d for p, d in zip(pos, dims))
    if not oob:
        return tuple(pos)
    if not periodic:
        return None
    return tuple(((p - 1) % d) + 1 for p, d in zip(pos, dims))


def _cartesian(dims):
    """CartesianIndices(dims) in column-major order"""
    for t in itertools.product(*[range(1, d + 1) for d in reversed(dims)]):
        yield tuple(reversed(t))


def add_raster(sim, name, dims, T, ctor):
    assert not sim.initialized, "add_raster! can be only called before finish_init!"
    grid = {}
    for pos in _cartesian(dims):
        grid[pos] = add_agent(sim, T, ctor(pos))
    sim.rasters[name] = (tuple(dims), grid)
    return grid


def connect_raster_neighbors(sim, name, E, ctor, distance=1, metric="chebyshev", periodic=True):
    dims, grid = sim.rasters[name]
    for org in _cartesian(dims):
        for s in _stencil(metric, len(dims), distance):
            sh = _checkpos([o + x for o, x in zip(org, s)], dims, periodic)
            if sh is not None:
                add_edge(sim, grid[org], grid[sh], E, ctor(org, sh))


def move_to(sim, name, id, pos, edge_from, edge_to, distance=0, metric="chebyshev",
            periodic=True, only_surrounding=False):
    """edge_from / edge_to: (edge type, state) or None"""
    dims, grid = sim.rasters[name]
    pos = tuple(pos)
    if not only_surrounding:
        if edge_from is not None:
            add_edge(sim, grid[pos], id, edge_from[0], edge_from[1])
        if edge_to is not None:
            add_edge(sim, id, grid[pos], edge_to[0], edge_to[1])
    if distance >= 1:
        for s in _stencil(metric, len(dims), distance):
            sh = _checkpos([p + x for p, x in zip(pos, s)], dims, periodic)
            if sh is not None:
                if edge_from is not None:
                    add_edge(sim, grid[sh], id, edge_from[0], edge_from[1])
                if edge_to is not None:
                    add_edge(sim, id, grid[sh], edge_to[0], edge_to[1])


def cellid(sim, name, pos):
    return sim.rasters[name][1][tuple(pos)]


def calc_rasterstate(sim, name, f, T):
    dims, grid = sim.rasters[name]
    keep = sim.check_readable, sim.intransition
    disable_transition_checks(sim, True)
    out = {pos: f(agentstate(sim, grid[pos], T)) for pos in _cartesian(dims)}
    sim.check_readable, sim.intransition = keep
    return out


# ---------------------------------------------- test-model transitions
# The named transitions of the GPU library, restated as Python transition
# functions with the reference's accessor calls (shape of test/core.jl:71-83,
# test/raster.jl:36-39, docs/examples/hegselmann.jl:134-144).
def tr_neighbor_sum(E, src_field, dst_field):
    def f(state, id, sim):
        ns = neighborstates_flexible(sim, id, E)
        s = 0
        if ns is not None:
            for n in ns:
                s = s + n[src_field]
        new = dict(state)
        new[dst_field] = s
        return new
    return f


def tr_neighbor_or(E, field):
    def f(state, id, sim):
        ns = neighborstates_flexible(sim, id, E)
        any_ = False
        if ns is not None:
            for n in ns:
                any_ = any_ or bool(n[field])
        new = dict(state)
        new[field] = bool(state[field]) or any_
        return new
    return f


def tr_count_edges(E, dst_field):
    def f(state, id, sim):
        new = dict(state)
        new[dst_field] = num_edges(sim, id, E)
        return new
    return f


def tr_die_if(kind, field=None, arg=None):
    def f(state, id, sim):
        if kind == "always":
            return None
        if kind == "ge":
            return None if state[field] >= arg else state
        if kind == "mod":
            return None if state[field] % arg != 0 else state
        if kind == "no_edges":
            return None if num_edges(sim, id, field) == 0 else state
        raise ValueError(kind)
    return f


def tr_set_field(field, kind, value=None):
    def f(state, id, sim):
        new = dict(state)
        new[field] = value if kind == "const" else (id % 2 == 1)
        return new
    return f


def tr_keep(state, id, sim):
    return state if not (isinstance(state, tuple) and state[0] == "Val") else None


def tr_self_edge(E, edge_state=None):
    def f(state, id, sim):
        add_edge(sim, id, id, E, edge_state)
        return state
    return f


def tr_readd_edges(E):
    def f(state, id, sim):
        es = edges(sim, id, E)
        if es is not None:
            add_edges(sim, id, list(es), E)
        return state
    return f


def tr_spawn(offsets, E=None):
    """add_agent! inside a transition (src/AgentMethods.jl:37-89): the agent
    keeps its state and adds one agent per offset, a copy of its state with
    field 0 increased by the offset; with E, after each add_agent! the edges
    new -> caller and caller -> new whose field 0 is the new agent's id
    (test/independent.jl:167-180)."""
    def f(state, id, sim):
        T = sim.tname(type_nr(id))
        fields = sim.m.atypes[sim.tnr(T) - 1]["fields"]
        for off in offsets:
            new = dict(state)
            if fields:
                new[fields[0]] = new[fields[0]] + off
            nid = add_agent(sim, T, new)
            if E is not None:
                ef = sim.m.etypes[E]["fields"]
                st = {ef[0]: nid} if ef else None
                add_edge(sim, nid, id, E, st)
                add_edge(sim, id, nid, E, dict(st) if st else None)
        return state
    return f


def tr_link_neighbors(E, F, die_value=None):
    """test/independent.jl:66-78: field 0 == die_value returns nothing;
    otherwise for every source of the in-edges of E, in insertion order,
    add_edge!(nid, id, F(foo)) and add_edge!(id, nid, F(foo))."""
    def f(state, id, sim):
        T = sim.tname(type_nr(id))
        fields = sim.m.atypes[sim.tnr(T) - 1]["fields"]
        v = state[fields[0]] if fields else 0
        if die_value is not None and fields and v == die_value:
            return None
        ef = sim.m.etypes[F]["fields"]
        for nid in neighborids(sim, id, E) or []:
            add_edge(sim, nid, id, F, {ef[0]: v} if ef else None)
            add_edge(sim, id, nid, F, {ef[0]: v} if ef else None)
        return state
    return f



def _field_test(kind, arg, v):
    if kind == 0:
        return True
    if kind == 1:
        return v >= arg
    return v % int(arg) != 0


def tr_remove_edges(E, kind, arg, mode):
    """remove_edges! inside a transition (src/EdgeMethods.jl:527-599): the
    agent keeps its state; mode 0: if its field 0 passes the test it calls
    remove_edges!(sim, id, E); mode 1: for every source nid of its in-edges
    of E (read container, insertion order) whose field 0 passes the test it
    calls remove_edges!(sim, nid, id, E)."""
    def f(state, id, sim):
        T = sim.tname(type_nr(id))
        fields = sim.m.atypes[sim.tnr(T) - 1]["fields"]
        if mode == 0:
            if not fields or _field_test(kind, arg, state[fields[0]]):
                remove_edges(sim, id, E)
            return state
        for nid in neighborids(sim, id, E) or []:
            src = agentstate_flexible(sim, nid)
            sf = sim.m.atypes[type_nr(nid) - 1]["fields"]
            if _field_test(kind, arg, src[sf[0]]):
                remove_edges(sim, id, E, frm=nid)
        return state
    return f
