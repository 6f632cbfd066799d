"""CPU tests of the C ABI: the library loads, exports every function
include/*.h declares, and its host-side logic (model registry, hint
normalisation, init-phase staging, raster stencils, accessor rules before
finish_init!) behaves as the reference's, without a GPU."""
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(vg_\w+)\s*\(", src))
    return sorted(names)


def test_every_declared_symbol_is_exported(vh):
    lib = vh.lib()
    names = declared()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []


def test_no_gpu_is_reported_not_faked(vh):
    import ctypes as C
    n = C.c_int(-1)
    vh.lib().vg_device_count(C.byref(n))
    assert n.value >= 0


def test_registry_rules(vh):
    """src/ModelTypes.jl:81-230"""
    m = vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
    with pytest.raises(AssertionError):
        m.register_agenttype("A", [("foo", "i64")])  # already registered
    with pytest.raises(AssertionError):
        m.register_agenttype("B", [], ":Bogus")
    with pytest.raises(AssertionError):  # SingleType+SingleEdge needs Stateless+IgnoreFrom
        m.register_edgetype("E1", [("w", "f64")], ":SingleType", ":SingleEdge", target="A")
    m.register_edgetype("E2", [], ":HasEdgeOnly")
    m.register_edgetype("E3", [], ":NumEdgesOnly")
    m.register_edgetype("E4", [("w", "f64")], target="A")  # target implies :SingleType
    m.register_edgetype("E5", [])                          # no field implies :Stateless
    model = m.create_model("rules")
    assert model.has_hint("E2", ":Stateless") and model.has_hint("E2", ":IgnoreFrom") \
        and model.has_hint("E2", ":SingleEdge")
    assert model.has_hint("E3", ":Stateless") and model.has_hint("E3", ":IgnoreFrom")
    assert model.has_hint("E4", ":SingleType")
    assert model.has_hint("E5", ":Stateless")


def test_prepared_apply_host_rules(vh):
    """A prepared apply! (vg_apply_prepare / vg_apply_call_run), without a
    GPU: an unknown transition is refused when the call is prepared; a run
    before finish_init! is refused with the reference's message (the same
    vg_apply call); after the simulation is closed the Python handle
    refuses to run instead of passing a stale simulation."""
    m = (vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
         .register_edgetype("E", [("w", "f64")]).create_model("prepared"))
    sim = vh.create_simulation(m)
    vh.add_agents(sim, "A", 3, foo=[1, 2, 3])
    with pytest.raises(Exception, match="unknown transition"):
        vh.prepare_apply(sim, "no_such_transition", ["A"], ["A"], ["A"])
    step = vh.prepare_apply(sim, "keep", ["A"], ["A"], ["A"])
    with pytest.raises(AssertionError, match="finish_init"):
        step()
    sim.close()
    with pytest.raises(RuntimeError, match="closed"):
        step()
    step.close()


def test_init_phase_staging_and_accessors(vh):
    """Before finish_init!: add_agent!/add_edge! staging, the :SingleEdge
    check of _can_add, num_edges(write=true), accessor hint rules."""
    m = (vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
         .register_edgetype("D", [("foo", "i64")])
         .register_edgetype("SE", [("foo", "i64")], ":SingleEdge")
         .register_edgetype("S", [], ":Stateless")
         .create_model("stage"))
    sim = vh.create_simulation(m)
    a1, a2, a3 = vh.add_agents(sim, "A", 3, foo=[1, 2, 3])
    assert vh.agent_nr(a3) == 3 and vh.type_nr(a3) == m["A"].index
    vh.add_edge(sim, a2, a3, "D", foo=1)
    vh.add_edge(sim, a1, a3, "D", foo=2)
    vh.add_edge(sim, a2, a3, "SE", foo=1)
    vh.add_edge(sim, a2, a3, "SE", foo=1)  # identical value: allowed
    with pytest.raises(AssertionError):
        vh.add_edge(sim, a1, a3, "SE", foo=2)
    vh.add_edge(sim, a1, a3, "S")
    vh.add_edge(sim, a2, vh.Edge(a3, {"foo": 7}), "D")  # add_edge!(sim, to, Edge(from, state))
    assert vh.edges(sim, a2, "D") == [vh.Edge(a3, {"foo": 7})]
    assert vh.num_edges(sim, "D", write=True) == 3
    vh.remove_edges(sim, a2, "D")
    assert vh.num_edges(sim, "D", write=True) == 2
    assert vh.num_edges(sim, "D", write=False) == 0
    assert vh.num_edges(sim, "SE", write=True) == 1
    assert vh.edges(sim, a3, "D") == [vh.Edge(a2, {"foo": 1}), vh.Edge(a1, {"foo": 2})]
    assert vh.neighborids(sim, a3, "S") == [a1]
    with pytest.raises(AssertionError):
        vh.edges(sim, a3, "S")  # stateless: edges is not defined
    with pytest.raises(AssertionError):
        vh.num_edges(sim, a3, "SE")  # single edge: num_edges is not defined
    assert vh.num_agents(sim, "A") == 3
    assert vh.mapreduce(sim, "foo", "+", "A") == 6
    assert vh.mapreduce(sim, "foo", "max", "A") == 3
    with pytest.raises(AssertionError):
        vh.apply_(sim, "keep", "A", [], [])  # apply! before finish_init!
    sim.close()


def test_raster_staging_counts(vh):
    """move_to! and connect_raster_neighbors! edge counts (test/raster.jl:374-436)
    on the staged edges, before any device work."""
    m = (vh.ModelTypes().register_agenttype("Position", [("v", "i64")])
         .register_agenttype("Mover", [("v", "i64")])
         .register_edgetype("On", [])
         .register_edgetype("G", [])
         .create_model("raster"))
    sim = vh.create_simulation(m)
    vh.add_raster(sim, "r", (10, 10), "Position", v=0)
    p = vh.add_agents(sim, "Mover", 3, v=1)
    vh.move_to(sim, "r", p[0], (4, 4), "On", None, distance=2)
    vh.move_to(sim, "r", p[1], (4, 4), "On", None, distance=2, metric="manhatten")
    vh.move_to(sim, "r", p[2], (4, 4), "On", None, distance=2.5, metric="euclidean")
    assert [vh.num_edges(sim, x, "On") for x in p] == [25, 13, 21]
    vh.connect_raster_neighbors(sim, "r", "G")
    assert vh.num_edges(sim, "G", write=True) == 800
    c = vh.cellid(sim, "r", (1, 1))
    ids = vh.neighborids(sim, c, "G")  # insertion order: source column-major
    assert [vh.agent_nr(i) for i in ids] == [2, 10, 11, 12, 20, 91, 92, 100]
    sim.close()


def test_params_and_globals(vh):
    """test/globals.jl:1-17 (set_global! of a scalar, push_global! twice onto
    a series) and register_param!/param/set_param! (src/Simulation.jl:587-630)"""
    m = (vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
         .register_param("beta", 0.1).register_global("count", 0.0).create_model("pg"))
    sim = vh.create_simulation(m)
    assert vh.param(sim, "beta") == 0.1
    vh.set_param(sim, "beta", 0.2)
    assert vh.param(sim, "beta") == 0.2
    vh.set_global(sim, "count", 3.0)
    vh.push_global(sim, "series", 1.0)
    vh.push_global(sim, "series", 2.0)
    assert vh.get_global(sim, "count") == 3.0
    assert list(vh.global_series(sim, "series")) == [1.0, 2.0]
    sim.close()


def test_bind_param_checks(vh):
    """Binding a transition's parameter slot to a param or global: unknown
    names, transitions, kinds and slots are refused (VG_ERR_ARG) before any
    apply!; rebinding a slot replaces it."""
    m = (vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
         .register_param("beta", 0.1).register_global("eps", 0.3).create_model("bind"))
    sim = vh.create_simulation(m)
    vh.bind_param(sim, "sir", 1, "beta", kind="param")
    vh.bind_param(sim, "sir", 1, "eps")  # rebinding the slot to a global
    vh.bind_param(sim, "bounded_confidence", 1, "eps")
    for bad in [("sir", 1, "nope", "global"), ("sir", 1, "nope", "param"),
                ("no_such_transition", 1, "eps", "global"), ("sir", -1, "eps", "global"),
                ("sir", 64, "eps", "global")]:
        with pytest.raises(vh.VahanaError):
            vh.bind_param(sim, *bad[:3], kind=bad[3])
    assert vh.lib().vg_bind_param(sim._h, b"sir", 1, 2, b"eps") != 0
    vh.unbind_params(sim, "sir")
    vh.unbind_params(sim)
    sim.close()


def test_parametric_type_names(vh):
    """test/parametric_types.jl:1-38: a parametric Julia type is registered
    under its full name; agents of it, a plain agent type and a parametric
    edge type are read back through edges, edgestates and neighborstates
    (here on the staged init-phase edges)."""
    m = (vh.ModelTypes().register_agenttype("PAgent{Float64}", [("t", "f64")])
         .register_agenttype("PAgent2", [("t", "f64")])
         .register_edgetype("PEdge{Float64}", [("t", "f64")]).create_model("parametric types"))
    sim = vh.create_simulation(m)
    id1 = vh.add_agent(sim, "PAgent{Float64}", t=1.0)
    id2 = vh.add_agent(sim, "PAgent2", t=2.0)
    vh.add_edge(sim, id1, id2, "PEdge{Float64}", t=3.0)
    assert vh.edges(sim, id2, "PEdge{Float64}")[0].state == {"t": 3.0}
    assert vh.edgestates(sim, id2, "PEdge{Float64}") == [{"t": 3.0}]
    assert vh.neighborstates(sim, id2, "PEdge{Float64}", "PAgent{Float64}") == [{"t": 1.0}]
    assert vh.type_nr(id1) == m["PAgent{Float64}"].index
    assert vh.type_nr(id2) == m["PAgent2"].index
    sim.close()


def test_neighborstates_iterators(vh):
    """neighborstates_iter (src/EdgeMethods.jl:783-803) and
    neighborstates_flexible_iter (src/Edge.jl:328-335) on staged edges:
    states in insertion order; the :SingleEdge / :IgnoreFrom rules."""
    m = (vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
         .register_edgetype("D", [("foo", "i64")])
         .register_edgetype("SE", [("foo", "i64")], ":SingleEdge")
         .register_edgetype("IF", [("foo", "i64")], ":IgnoreFrom")
         .create_model("iter"))
    sim = vh.create_simulation(m)
    a1, a2, a3 = vh.add_agents(sim, "A", 3, foo=[1, 2, 3])
    vh.add_edge(sim, a2, a3, "D", foo=1)
    vh.add_edge(sim, a1, a3, "D", foo=2)
    vh.add_edge(sim, a2, a3, "SE", foo=1)
    vh.add_edge(sim, a1, a3, "IF", foo=1)
    assert list(vh.neighborstates_iter(sim, a3, "D", "A")) == [{"foo": 2}, {"foo": 1}]
    assert vh.neighborstates_iter(sim, a1, "D", "A") is None
    assert list(vh.neighborstates_flexible_iter(sim, a3, "D")) == [{"foo": 2}, {"foo": 1}]
    assert list(vh.neighborstates_flexible_iter(sim, a3, "SE")) == [{"foo": 2}]
    for T in ("SE", "IF"):
        with pytest.raises(AssertionError):
            vh.neighborstates_iter(sim, a3, T, "A")
    with pytest.raises(AssertionError):
        vh.neighborstates_flexible_iter(sim, a3, "IF")
    sim.close()


def test_null_and_bad_arguments_return_errors(vh):
    """Misuse at the C ABI returns VG_ERR_ARG (2) with a message instead of
    crashing: null handles, names, field arrays and output pointers, and
    unknown type numbers or names."""
    import ctypes as C
    L = vh.lib()
    m = C.c_void_p()
    sim = C.c_void_p()
    nr = C.c_int()
    hints = C.c_uint()
    d = C.c_double()
    assert L.vg_model_create(None) == 2
    assert L.vg_sim_create(None, b"x", None, C.byref(sim)) == 2
    assert b"null model handle" in L.vg_last_error()
    assert L.vg_model_create(C.byref(m)) == 0
    assert L.vg_model_register_agenttype(m, None, 0, None, None, 0, C.byref(nr)) == 2
    assert L.vg_model_register_agenttype(m, b"A", 1, None, None, 0, C.byref(nr)) == 2
    assert L.vg_model_register_agenttype(m, b"A", -1, None, None, 0, C.byref(nr)) == 2
    assert L.vg_model_register_edgetype(m, None, 0, None, None, 0, 0, 0, C.byref(nr)) == 2
    assert L.vg_model_register_param(m, None, 1.0) == 2
    assert L.vg_model_register_global(None, b"g", 1.0) == 2
    assert L.vg_model_edge_hints(m, 99, C.byref(hints)) == 2
    assert L.vg_model_edge_hints(m, 0, None) == 2
    assert L.vg_model_type_by_name(m, b"nope", C.byref(nr)) == 2
    assert L.vg_model_type_by_name(m, None, C.byref(nr)) == 2
    assert L.vg_model_finalize(m, b"bad args") == 0
    assert L.vg_sim_create(m, b"x", None, None) == 2
    assert L.vg_sim_load(m, None, None, C.byref(sim)) == 2
    assert L.vg_num_agents(None, 1, C.byref(C.c_uint64())) == 2
    assert L.vg_get_global(None, b"g", C.byref(d)) == 2
    assert L.vg_finish_init(None) == 2
    assert L.vg_model_finalize(None, b"x") == 2
    L.vg_model_destroy(m)
    # a staged simulation: required output pointers and argument arrays
    mm = (vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
          .register_agenttype("Cell", [("v", "i64")])
          .register_edgetype("D", [("foo", "i64")]).create_model("bad args 2"))
    s = vh.create_simulation(mm)
    vh.add_agents(s, "A", 3, foo=[1, 2, 3])
    vh.add_raster(s, "r", (4, 4), "Cell", v=0)
    h, a, e = s._h, mm["A"].index, mm["D"].index
    u = C.c_uint64()
    nd = C.c_int()
    assert L.vg_num_agents(h, a, None) == 2
    assert L.vg_agent_slots(h, a, None) == 2
    assert L.vg_read_agents(h, a, None, None, 2, None) == 2
    assert L.vg_sim_num_transitions(h, None) == 2
    assert L.vg_sim_device_bytes(h, None) == 2
    assert L.vg_num_edges_total(h, e, 1, None) == 2
    assert L.vg_global_series(h, b"g", None, 0, None) == 2
    assert L.vg_add_edges(h, e, 2, None, None, None) == 2
    assert L.vg_remove_edges(h, e, 2, None, None) == 2
    assert L.vg_cellid(h, b"r", None, C.byref(u)) == 2
    assert L.vg_raster_dims(h, b"r", None, None) == 2
    assert L.vg_raster_dims(h, b"r", None, C.byref(nd)) == 0 and nd.value == 2
    assert L.vg_raster_dims(h, None, None, C.byref(nd)) == 2
    assert L.vg_move_to(h, b"r", 1, None, -1, None, -1, None, 0.0, 0, 1, 0) == 2
    assert L.vg_add_graph(h, a, 2, None, e, 2, None, None, 1, None, None) == 2
    assert L.vg_read_staged_edges(h, e, None, None, None, 0, None) == 2
    assert L.vg_read_edges(h, e, a, None, None, None, None, C.byref(u)) == 2
    assert b"row count pointer" in L.vg_last_error()
    assert L.vg_read_edges(h, e, a, None, None, None, C.byref(u), None) == 2
    # :SingleEdge duplicate check against a staged edge, payload omitted
    mse = (vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
           .register_edgetype("SE", [("foo", "i64")], ":SingleEdge").create_model("se"))
    s2 = vh.create_simulation(mse)
    x = [int(i) for i in vh.add_agents(s2, "A", 2, foo=[1, 2])]
    one = np.array([x[0]], dtype=np.uint64)
    two = np.array([x[1]], dtype=np.uint64)
    P64 = C.POINTER(C.c_uint64)
    se = mse["SE"].index
    assert L.vg_add_edges(s2._h, se, 1, one.ctypes.data_as(P64), two.ctypes.data_as(P64), None) == 0
    assert L.vg_add_edges(s2._h, se, 1, one.ctypes.data_as(P64), two.ctypes.data_as(P64), None) == 0
    vh.add_edge(s2, x[0], x[1], "SE", foo=0)  # identical (zero) value: allowed
    with pytest.raises(AssertionError):
        vh.add_edge(s2, x[0], x[1], "SE", foo=3)
    assert vh.num_edges(s2, "SE", write=True) == 1
    s2.close()
    assert vh.num_agents(s, "A") == 3  # the simulation is still usable
    s.close()
    # serving and batch handles (checked before any device work)
    assert L.vg_serve_create(1 << 20, 1, None) == 2
    assert L.vg_serve_submit(None, None, None) == 2
    assert L.vg_serve_poll(None, None, 0, C.byref(u)) == 2
    assert L.vg_serve_job_state(None, 1, None, 0, C.byref(u)) == 2
    assert L.vg_serve_stats(None, None, None, None, None, None, None) == 2
    assert L.vg_serve_drain(None) == 2
    assert L.vg_serve_destroy(None) == 0
    assert L.vg_batch_create_sir(2, None, None, None, None, None, 10, None, None) == 2
    assert L.vg_batch_step(None, 1, 0) == 2
    # prepared apply!: a null simulation, a null output, a bad list, a null handle
    h = C.c_void_p()
    assert L.vg_apply_prepare(None, b"sir", None, 0, None, 0, None, 0, None, 0, -1, None, 0,
                              C.byref(h)) == 2
    assert L.vg_apply_call_run(None) == 2
    assert L.vg_apply_call_destroy(None) == 0
    assert L.vg_batch_set_launch(None, 0, 256, 0xFFFFFFFF) == 2
    assert L.vg_batch_set_lanes(None, 1, 1) == 2
    assert L.vg_batch_lanes(None, None, None) == 2
    assert L.vg_batch_set_cluster(None, 4, 256, 1) == 2
    assert L.vg_batch_cluster(None, None, None, None, None) == 2
    assert L.vg_batch_tuning(None, None, None, None, None, None, None, None) == 2
    assert L.vg_batch_destroy(None) == 0


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_init_phase_remove_edges_matches_sequential_removal(vh, seed):
    """remove_edges!(sim, to, T) and remove_edges!(sim, from, to, T) in the
    initialization phase (src/EdgeMethods.jl:527-599), many removals in one
    call and calls interleaved with add_edge!: the staged edges equal those
    left by removing one key at a time from the insertion-ordered list."""
    rng = np.random.default_rng(seed)
    m = (vh.ModelTypes().register_agenttype("A", [("foo", "i64")])
         .register_edgetype("D", [("w", "i64")]).create_model("rm"))
    sim = vh.create_simulation(m)
    ids = [int(x) for x in vh.add_agents(sim, "A", 40, foo=np.arange(40))]
    ref = []  # (from, to, w) in insertion order
    w = 0
    for _ in range(6):
        k = int(rng.integers(50, 200))
        frm = [ids[i] for i in rng.integers(0, 40, k)]
        to = [ids[i] for i in rng.integers(0, 40, k)]
        ws = np.arange(w, w + k)
        w += k
        vh.add_edges(sim, "D", frm, to, w=ws)
        ref += list(zip(frm, to, ws.tolist()))
        r = int(rng.integers(1, 15))
        rto = [ids[i] for i in rng.integers(0, 40, r)]
        if rng.integers(0, 2):
            rfrom = [ids[i] for i in rng.integers(0, 40, r)]
            vh.remove_edges(sim, rto, "D", frm=rfrom)
            for a, b in zip(rfrom, rto):
                ref = [x for x in ref if not (x[1] == b and x[0] == a)]
        else:
            vh.remove_edges(sim, rto, "D")
            for b in rto:
                ref = [x for x in ref if x[1] != b]
    from vahana_gb300 import models
    frm, to, pl = models.staged_edges(sim, "D")
    assert list(zip(frm.tolist(), to.tolist(), pl["w"].tolist())) == ref
    assert vh.num_edges(sim, "D", write=True) == len(ref)
    sim.close()


def test_transition_registry_lists_every_named_kernel(vh):
    """apply! binds a transition by name (the reference passes a Julia
    callable, src/Simulation.jl:720-726): the registry names the three test
    models' rules and the generic rules the ported tests use, each once.
    Before finish_init! apply! is refused with the reference's message
    whatever the name (src/Simulation.jl:727)."""
    names = vh.transition_names()
    for n in ("bounded_confidence", "sir", "life", "random_walk", "neighbor_sum",
              "neighbor_or", "count_edges", "die_if", "set_field", "keep", "self_edge",
              "readd_edges", "spawn", "link_neighbors", "remove_edges"):
        assert n in names
    assert len(set(names)) == len(names)
    m = vh.ModelTypes().register_agenttype("A", [("foo", "i64")]).create_model("names")
    sim = vh.create_simulation(m)
    vh.add_agents(sim, "A", 2, foo=[1, 2])
    for rule in ("no_such_rule", "keep"):
        with pytest.raises(AssertionError, match="finish_init"):
            vh.apply_(sim, rule, "A", ["A"], ["A"])
    sim.close()
