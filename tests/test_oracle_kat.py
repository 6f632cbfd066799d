"""The reference's own known-answer tests, run on the oracle (CPU).

These pin the oracle's restatement of Vahana's semantics to the expected
values the reference's test suite asserts (each test cites the reference
test it ports).  The GPU library is then checked against the oracle.
"""
import pytest

from oracle import vahana_ref as V


# ---------------------------------------------------------- test/core.jl
def core_model():
    return (V.ModelTypes()
            .register_agenttype("AMortal", [("foo", "i64")])
            .register_agenttype("AMortalFixed", [("foo", "i64")])
            .register_agenttype("AImm", [("foo", "i64")], ":Immortal")
            .register_agenttype("AImmFixed", [("foo", "i64")], ":Immortal")
            .register_agenttype("AImmFixedOversize", [("foo", "i64")], ":Immortal")
            .register_agenttype("ADefault", [("foo", "i64"), ("bool", "bool")])
            .register_edgetype("ESDict", [("foo", "i64")])
            .register_edgetype("ESLDict1", [])
            .register_edgetype("ESLDict2", [], ":SingleType", target="AImm")
            .create_model("Test Core"))


def add_example_network(sim):
    """test/core.jl:41-69"""
    a1 = V.add_agent(sim, "AMortal", {"foo": 1})
    a2, a3 = V.add_agents(sim, "AMortal", [{"foo": 2}, {"foo": 3}])
    avids = V.add_agents(sim, "AImm", [{"foo": i} for i in range(1, 11)])
    avfids = V.add_agents(sim, "AImmFixed", [{"foo": i} for i in range(1, 11)])
    V.add_agents(sim, "AImmFixedOversize", [{"foo": i} for i in range(1, 11)])
    V.add_agents(sim, "AMortalFixed", [{"foo": i} for i in range(1, 11)])
    V.add_agents(sim, "ADefault", [{"foo": i, "bool": True} for i in range(1, 11)])
    V.add_edge(sim, a2, a1, "ESDict", {"foo": 1})
    V.add_edge(sim, a3, a1, "ESDict", {"foo": 2})
    V.add_edge(sim, avids[0], a1, "ESDict", {"foo": 3})
    V.add_edge(sim, avfids[9], a1, "ESDict", {"foo": 4})
    V.add_edges(sim, a1, [V.Edge(avids[i], {}) for i in range(10)], "ESLDict1")
    for i in range(10):
        V.add_edge(sim, avfids[i], avids[i], "ESLDict2")
    return a1, a2, a3, avids, avfids


def createsim():
    sim = V.create_simulation(core_model())
    ids = add_example_network(sim)
    V.finish_init(sim)
    return (sim,) + ids


ALL = ["AMortal", "AImm", "AImmFixed"]


def test_core_edges_and_neighborids():
    """test/core.jl:177-199"""
    sim, a1, a2, a3, avids, avfids = createsim()
    V.disable_transition_checks(sim, True)
    assert len(V.edges(sim, a1, "ESDict")) == 4
    assert V.edges(sim, a2, "ESDict") is None
    assert len(V.neighborids(sim, avids[0], "ESLDict2")) == 1
    assert V.neighborids(sim, a1, "ESLDict1")[0] == avids[0]
    assert V.neighborids(sim, a1, "ESLDict1")[9] == avids[9]
    assert V.neighborids(sim, avids[9], "ESLDict2")[0] == avfids[9]
    assert {"foo": 3} in V.neighborstates_flexible(sim, a1, "ESDict")
    assert V.num_edges(sim, a1, "ESDict") == 4
    assert V.num_edges(sim, a2, "ESDict") == 0
    assert V.num_edges(sim, avids[0], "ESLDict2") == 1


def test_core_agentstate_checks():
    """test/core.jl:161-175"""
    sim, a1, a2, a3, avids, avfids = createsim()
    with pytest.raises(AssertionError):
        V.agentstate(sim, a2, "AImm")
    V.disable_transition_checks(sim, True)
    assert V.agentstate(sim, a1, "AMortal") == {"foo": 1}
    assert V.agentstate(sim, avfids[9], "AImmFixed") == {"foo": 10}


def test_core_transition_sums():
    """test/core.jl:289-394: neighbour sums over 1-3 steps"""
    sim, a1, a2, a3, avids, avfids = createsim()
    with pytest.raises(AssertionError):  # AImmFixed (a source type) is not readable
        V.apply_(sim, lambda s, id, sim_: V.neighborstates_flexible(sim_, id, "ESLDict2") and s,
                 "AImm", ["ESLDict2"], [])
    sim, a1, a2, a3, avids, avfids = createsim()
    V.disable_transition_checks(sim, True)
    V.add_edge(sim, a1, a1, "ESLDict1")
    V.add_edge(sim, avids[0], avids[0], "ESLDict2")
    V.add_edge(sim, avfids[0], avfids[0], "ESLDict1")
    V.add_edge(sim, avfids[1], avfids[0], "ESLDict1")
    V.add_edge(sim, avfids[1], avfids[1], "ESLDict1")
    V.disable_transition_checks(sim, False)
    f = V.tr_neighbor_sum("ESLDict1", "foo", "foo")
    V.apply_(sim, f, ["AMortal"], ALL + ["ESLDict1"], ["AMortal"])
    V.disable_transition_checks(sim, True)
    assert V.agentstate(sim, a1, "AMortal") == {"foo": sum(range(1, 11)) + 1}
    V.disable_transition_checks(sim, False)
    V.apply_(sim, f, ["AMortal"], ALL + ["ESLDict1"], ["AMortal"])
    V.disable_transition_checks(sim, True)
    assert V.agentstate(sim, a1, "AMortal") == {"foo": 2 * sum(range(1, 11)) + 1}

    sim, a1, a2, a3, avids, avfids = createsim()
    V.disable_transition_checks(sim, True)
    V.add_edge(sim, avids[0], avids[0], "ESLDict2")
    V.disable_transition_checks(sim, False)
    g = V.tr_neighbor_sum("ESLDict2", "foo", "foo")
    for expect in (2, 3, 4):
        V.apply_(sim, g, ["AImm"], ALL + ["ESLDict2"], ["AImm"])
        V.disable_transition_checks(sim, True)
        assert V.agentstate(sim, avids[0], "AImm") == {"foo": expect}
        V.disable_transition_checks(sim, False)

    sim, a1, a2, a3, avids, avfids = createsim()
    V.disable_transition_checks(sim, True)
    V.add_edge(sim, avfids[0], avfids[0], "ESLDict1")
    V.add_edge(sim, avfids[1], avfids[0], "ESLDict1")
    V.add_edge(sim, avfids[1], avfids[1], "ESLDict1")
    V.disable_transition_checks(sim, False)
    for expect in (3, 5, 7):
        V.apply_(sim, f, ["AImmFixed"], ALL + ["ESLDict1"], ["AImmFixed"])
        V.disable_transition_checks(sim, True)
        assert V.agentstate(sim, avfids[0], "AImmFixed") == {"foo": expect}
        V.disable_transition_checks(sim, False)


def test_core_mapreduce_six_ops():
    """test/core.jl:87-107, 396-440"""
    sim = V.create_simulation(core_model())
    add_example_network(sim)
    V.finish_init(sim)
    import functools
    import operator
    for T in ["AImmFixed", "AImmFixedOversize", "AMortalFixed", "ADefault"]:
        assert V.mapreduce(sim, lambda a: a["foo"], "+", T) == sum(range(1, 11))
        assert V.mapreduce(sim, lambda a: a["foo"], "*", T) == functools.reduce(operator.mul, range(1, 11))
        assert V.mapreduce(sim, lambda a: a["foo"], "&", T, datatype="int") == \
            functools.reduce(operator.and_, range(1, 11))
        assert V.mapreduce(sim, lambda a: a["foo"], "|", T, datatype="int") == \
            functools.reduce(operator.or_, range(1, 11))
        assert V.mapreduce(sim, lambda a: a["foo"], "max", T) == 10
        assert V.mapreduce(sim, lambda a: a["foo"], "min", T) == 1
    # all agents of a type removed: mapreduce returns the identity
    V.apply_(sim, V.tr_die_if("always"), ["AMortalFixed"], ["AMortalFixed"], ["AMortalFixed"])
    assert V.mapreduce(sim, lambda a: a["foo"], "+", "AMortalFixed") == 0
    assert V.mapreduce(sim, lambda a: a["bool"], "&", "ADefault") is True
    V.apply_(sim, V.tr_set_field("bool", "const", False), ["ADefault"], ["ADefault"], ["ADefault"])
    assert V.mapreduce(sim, lambda a: a["bool"], "&", "ADefault") is False
    assert V.mapreduce(sim, lambda a: a["bool"], "|", "ADefault") is False
    V.apply_(sim, V.tr_set_field("bool", "id_odd"), ["ADefault"], ["ADefault"], ["ADefault"])
    assert V.mapreduce(sim, lambda a: a["bool"], "&", "ADefault") is False
    assert V.mapreduce(sim, lambda a: a["bool"], "|", "ADefault") is True


def test_core_all_agents_and_deaths():
    """test/core.jl:210-277"""
    sim, *_ = createsim()
    assert len(V.all_agents(sim, "AMortalFixed")) == 10
    assert V.num_agents(sim, "AImm") == 10
    V.apply_(sim, V.tr_die_if("ge", "foo", 6), "AMortalFixed", "AMortalFixed", "AMortalFixed")
    assert V.num_agents(sim, "AMortalFixed") == 5
    assert sorted(a["foo"] for a in V.all_agents(sim, "AMortalFixed")) == [1, 2, 3, 4, 5]
    m = V.ModelTypes().register_agenttype("AMortal", [("foo", "i64")]).create_model("ids")
    s = V.create_simulation(m)
    for i in range(1, 11):
        V.add_agent(s, "AMortal", {"foo": i})
    V.finish_init(s)
    V.apply_(s, V.tr_die_if("mod", "foo", 2), "AMortal", "AMortal", "AMortal")
    assert len(V.all_agentids(s, "AMortal")) == 5


def test_core_with_edge():
    """test/core.jl:133-157"""
    sim = V.create_simulation(core_model())
    aids = [V.add_agent(sim, "AMortal", {"foo": i}) for i in range(1, 101)]
    V.add_edge(sim, aids[0], aids[1], "ESLDict1")
    V.finish_init(sim)
    V.apply_(sim, V.tr_die_if("always"), "AMortal", "AMortal", "AMortal", with_edge="ESLDict1")
    assert V.num_agents(sim, "AMortal") == 99


# ---------------------------------------------------------- test/edges.jl
STATELESS = ["EdgeS", "EdgeSE", "EdgeST", "EdgeSI", "EdgeSEI", "EdgeSTI", "EdgeSETI", "EdgeSTs",
             "EdgeSTsI", "EdgeSETsI"]
STATEFUL = ["EdgeD", "EdgeE", "EdgeT", "EdgeI", "EdgeEI", "EdgeTI", "EdgeTs", "EdgeTsI"]


def hashint(t, h):
    return h in t[4:]


def edges_model():
    """test/edges.jl:42-63"""
    m = (V.ModelTypes().register_agenttype("Agent", [("foo", "i64")])
         .register_agenttype("AgentB", [("foo", "i64")]))
    for t in STATELESS + STATEFUL:
        hints = []
        tag = t[4:]
        if "S" in tag:
            hints.append(":Stateless")
        if "E" in tag:
            hints.append(":SingleEdge")
        if "I" in tag:
            hints.append(":IgnoreFrom")
        kw = {}
        if "T" in tag:
            hints.append(":SingleType")
            kw["target"] = "Agent"
            if "Ts" in tag:
                kw["size"] = 10
        fields = [] if t in STATELESS else [("foo", "i64")]
        m.register_edgetype(t, fields, *hints, **kw)
    return m.create_model("Test Edges")


def st(t, v):
    return {} if t in STATELESS else {"foo": v}


def edges_sim():
    sim = V.create_simulation(edges_model())
    a1, a2, a3 = V.add_agents(sim, "Agent", [{"foo": 1}, {"foo": 2}, {"foo": 3}])
    for t in STATELESS + STATEFUL:
        V.add_edge(sim, a2, a3, t, st(t, 1))
        if hashint(t, "E") and not hashint(t, "T") and not (hashint(t, "S") and hashint(t, "I")):
            with pytest.raises(AssertionError):
                V.add_edge(sim, a1, a3, t, st(t, 2))
        elif not hashint(t, "E"):
            V.add_edge(sim, a1, a3, t, st(t, 2))
        V.add_edges(sim, a1, [V.Edge(a3, st(t, 3))], t)
    V.finish_init(sim)
    return sim, a1, a2, a3


def test_edges_insertion_order_and_hints():
    """test/edges.jl:123-227"""
    sim, a1, a2, a3 = edges_sim()
    V.disable_transition_checks(sim, True)
    for t in ["EdgeD", "EdgeT", "EdgeTs"]:
        e = V.edges(sim, a3, t)
        assert e[0] == V.Edge(a2, {"foo": 1}) and e[1] == V.Edge(a1, {"foo": 2})
        assert V.edges(sim, a2, t) is None
    assert V.edges(sim, a3, "EdgeE") == V.Edge(a2, {"foo": 1})
    for t in ["EdgeD", "EdgeT", "EdgeTs", "EdgeS", "EdgeST", "EdgeSTs"]:
        e = V.neighborids(sim, a3, t)
        assert e[0] == a2 and e[1] == a1
        assert V.neighborids(sim, a2, t) is None
    for t in ["EdgeE", "EdgeSE"]:
        assert V.neighborids(sim, a3, t) == a2
    for t in ["EdgeD", "EdgeT", "EdgeTs", "EdgeI", "EdgeTI", "EdgeTsI"]:
        e = V.edgestates(sim, a3, t)
        assert e[0] == {"foo": 1} and e[1] == {"foo": 2}
    for t in ["EdgeE", "EdgeEI"]:
        assert V.edgestates(sim, a3, t) == {"foo": 1}
    for t in ["EdgeD", "EdgeT", "EdgeTs", "EdgeI", "EdgeTI", "EdgeTsI", "EdgeS", "EdgeST",
              "EdgeSTs", "EdgeSTI", "EdgeSTsI"]:
        assert V.num_edges(sim, a1, t) == 1
        assert V.num_edges(sim, a2, t) == 0
        assert V.num_edges(sim, a3, t) == 2
    for t in STATELESS + STATEFUL:
        assert V.has_edge(sim, a1, t) is True
        assert V.has_edge(sim, a2, t) is False
        assert V.has_edge(sim, a3, t) is True
    V.disable_transition_checks(sim, False)
    for t in ["EdgeI", "EdgeEI", "EdgeTI", "EdgeTsI"] + STATELESS:
        with pytest.raises(AssertionError):
            V.edges(sim, a1, t)
    for t in ["EdgeI", "EdgeTI", "EdgeTsI", "EdgeSI", "EdgeSTI", "EdgeSTsI", "EdgeEI", "EdgeSEI",
              "EdgeSETI", "EdgeSETsI"]:
        with pytest.raises(AssertionError):
            V.neighborids(sim, a1, t)
    for t in STATELESS:
        with pytest.raises(AssertionError):
            V.edgestates(sim, a1, t)
    for t in ["EdgeE", "EdgeEI", "EdgeSE", "EdgeSETI", "EdgeSETsI"]:
        with pytest.raises(AssertionError):
            V.num_edges(sim, a1, t)
    for t in ["EdgeD", "EdgeT", "EdgeI", "EdgeTI", "EdgeTs", "EdgeTsI"]:
        assert V.mapreduce(sim, lambda a: a["foo"], "+", t) == 6
    for t in ["EdgeE", "EdgeEI"]:
        assert V.mapreduce(sim, lambda a: a["foo"], "+", t) == 4
    for t in STATELESS:
        with pytest.raises(AssertionError):
            V.mapreduce(sim, lambda a: a["foo"], "+", t)
    for t in STATELESS + STATEFUL:  # add_edge! after finish_init! outside apply!
        with pytest.raises(AssertionError):
            V.add_edge(sim, 0, 0, t, st(t, 0))


def test_edges_num_edges_write():
    """test/edges.jl:278-316"""
    sim = V.create_simulation(edges_model())
    for t in STATELESS + STATEFUL:
        assert V.num_edges_total(sim, t, write=False) == 0
    id1, id2, id3 = (V.add_agent(sim, "Agent", {"foo": 0}) for _ in range(3))
    for t in STATELESS + STATEFUL:
        V.add_edge(sim, id1, id1, t, st(t, 0))
        V.add_edge(sim, id3, id3, t, st(t, 0))
    for t in STATELESS + STATEFUL:
        assert V.num_edges_total(sim, t, write=True) == 2
        assert V.num_edges_total(sim, t, write=False) == 0
    V.finish_init(sim)
    for t in STATELESS + STATEFUL:
        assert V.num_edges_total(sim, t, write=False) == 2


def test_edges_transition_readd():
    """test/edges.jl:319-389 (one process: nagents = 2)"""
    for ET in ["EdgeD", "EdgeT", "EdgeI", "EdgeTI"]:
        sim = V.create_simulation(edges_model())
        n = 2
        ids = V.add_agents(sim, "Agent", [{"foo": i} for i in range(1, n + 1)])
        for a in range(n):  # complete graph, add_graph! order (GraphsSupport.jl:41-52)
            for b in range(n):
                if a != b:
                    V.add_edge(sim, ids[a], ids[b], ET, {"foo": b + 1})
        V.finish_init(sim)
        counts = []
        check = lambda s, id, sim_: counts.append(V.num_edges(sim_, id, ET))
        V.apply_(sim, check, ["Agent"], [ET], [])
        assert counts == [n - 1] * n
        V.apply_(sim, V.tr_keep, ["Agent"], [], [ET], add_existing=[ET])
        counts.clear()
        V.apply_(sim, check, ["Agent"], [ET], [])
        assert counts == [n - 1] * n
        if ET == "EdgeD":
            V.apply_(sim, V.tr_readd_edges(ET), ["Agent"], [ET], [ET])
            counts.clear()
            V.apply_(sim, check, ["Agent"], [ET], [])
            assert counts == [n - 1] * n
            V.apply_(sim, V.tr_readd_edges(ET), ["Agent"], [ET], [ET], add_existing=[ET])
            counts.clear()
            V.apply_(sim, check, ["Agent"], [ET], [])
            assert counts == [(n - 1) * 2] * n
            V.apply_(sim, V.tr_keep, ["Agent"], [], [ET])
            counts.clear()
            V.apply_(sim, check, ["Agent"], [ET], [])
            assert counts == [0] * n


# ---------------------------------------------------- test/remove_agents.jl
@pytest.mark.parametrize("E", ["DEdge", "DEdgeST"])
def test_dying_agents(E):
    """test/remove_agents.jl:22-112 (one process)"""
    m = (V.ModelTypes().register_agenttype("DAgent", [("idx", "i64")])
         .register_agenttype("DAgentRemove", [])
         .register_edgetype("DEdge", [])
         .register_edgetype("DEdgeState", [("state", "i64")])
         .register_edgetype("DSingleEdge", [], ":SingleEdge")
         .register_edgetype("DEdgeST", [], ":SingleType", target="DAgent")
         .create_model("remove_agents"))
    for twice in (False, True):
        sim = V.create_simulation(m)
        ids = V.add_agents(sim, "DAgent", [{"idx": i} for i in range(1, 4)])
        rids = V.add_agents(sim, "DAgentRemove", [{}])
        reps = 2 if twice else 1
        for _ in range(reps):
            for id in ids:
                V.add_edge(sim, id, ids[1], E)
            for id in rids:
                V.add_edge(sim, id, ids[1], "DEdgeState", {"state": 0})
        for _ in range(reps):
            V.add_edge(sim, ids[1], ids[2], E)
        V.finish_init(sim)
        assert V.num_edges_total(sim, E) == 4 * reps
        assert V.num_edges_total(sim, "DEdgeState") == reps
        V.apply_(sim, V.tr_die_if("always"), ["DAgentRemove"], [], ["DAgentRemove"])
        assert V.num_edges_total(sim, E) == 4 * reps
        if not twice:
            assert V.num_edges_total(sim, "DEdgeState") == 0
        V.apply_(sim, V.tr_die_if("no_edges", E), ["DAgent"], ["DAgent", E], ["DAgent"])
        assert V.num_edges_total(sim, E) == 3 * reps


# --------------------------------------------------- test/edgesiterator.jl
@pytest.mark.parametrize("ET", STATEFUL)
def test_edges_agg(ET):
    """test/edgesiterator.jl:55-109"""
    sim = V.create_simulation(edges_model())
    assert V.mapreduce(sim, lambda e: e["foo"], "+", ET) == 0
    aids = V.add_agents(sim, "Agent", [{"foo": i} for i in range(1, 11)])
    for id in aids:
        V.add_edge(sim, aids[0], id, ET, {"foo": V.agent_nr(id)})
    V.finish_init(sim)
    assert V.mapreduce(sim, lambda e: e["foo"], "+", ET) == 55 if not hashint(ET, "E") else True
    V.apply_(sim, V.tr_die_if("always"), ["Agent"], [], ["Agent"])
    assert V.mapreduce(sim, lambda e: e["foo"], "+", ET) == 0
    sim = V.create_simulation(edges_model())
    aids = V.add_agents(sim, "Agent", [{"foo": i} for i in range(1, 11)])
    bids = V.add_agents(sim, "AgentB", [{"foo": i} for i in range(1, 11)])
    for i in range(10):
        V.add_edge(sim, bids[i], aids[i], ET, {"foo": i + 1})
    V.finish_init(sim)
    assert V.mapreduce(sim, lambda e: e["foo"], "+", ET) == 55
    V.apply_(sim, V.tr_die_if("always"), ["Agent"], [], ["Agent"])
    assert V.mapreduce(sim, lambda e: e["foo"], "+", ET) == 0


@pytest.mark.parametrize("ET", STATEFUL + STATELESS)
def test_remove_edges_of_died(ET):
    """test/edgesiterator.jl:111-217"""
    m = edges_model()
    sim = V.create_simulation(m)
    aids = V.add_agents(sim, "Agent", [{"foo": i} for i in range(1, 11)])
    bids = V.add_agents(sim, "AgentB", [{"foo": i} for i in range(1, 11)])
    h = m.etypes[ET]["hints"]
    for i in range(10):
        V.add_edge(sim, bids[i], aids[i], ET, st(ET, i + 1))
    V.finish_init(sim)
    assert V.num_edges_total(sim, ET) == 10
    V.apply_(sim, V.tr_die_if("always"), ["Agent"], [], ["Agent"])
    assert V.num_edges_total(sim, ET) == 0
    if ":IgnoreFrom" in h:
        return
    sim = V.create_simulation(m)
    aids = V.add_agents(sim, "Agent", [{"foo": i} for i in range(1, 11)])
    bids = V.add_agents(sim, "AgentB", [{"foo": i} for i in range(1, 11)])
    for i in range(10):
        if ":SingleEdge" not in h:
            V.add_edge(sim, aids[i], aids[i], ET, st(ET, i + 1))      # a -> a
            if ":SingleType" not in h:
                V.add_edge(sim, aids[i], bids[i], ET, st(ET, i + 1))  # a -> b
        V.add_edges(sim, aids[i], [V.Edge(bids[i], st(ET, i + 1))], ET)  # b -> a
        if ":SingleType" not in h:
            V.add_edges(sim, bids[i], [V.Edge(bids[i], st(ET, i + 1))], ET)  # b -> b
    V.finish_init(sim)
    V.apply_(sim, V.tr_die_if("mod", "foo", 2), "AgentB", "AgentB", "AgentB")
    count = 5
    if ":SingleEdge" not in h:
        count += 10
    if ":SingleType" not in h:
        count += 5
    if ":SingleEdge" not in h and ":SingleType" not in h:
        count += 5
    assert V.num_edges_total(sim, ET) == count


# --------------------------------------------------------- test/raster.jl
def raster_model():
    return (V.ModelTypes()
            .register_agenttype("GridA", [("pos", "x"), ("active", "bool")])
            .register_agenttype("Grid3D", [("pos", "x"), ("active", "bool")])
            .register_edgetype("GridE", [])
            .register_agenttype("Position", [("ids_sum", "i64")])
            .register_agenttype("MovingAgent", [("value", "i64")])
            .register_edgetype("OnPosition", [])
            .create_model("Raster_Test"))


@pytest.mark.parametrize("dims,start,T,kw,counts", [
    ((10, 8), (10, 8), "GridA", {}, (1, 9, 25)),
    ((7, 9), (3, 5), "GridA", {}, (1, 9, 25)),
    ((17, 6), (9, 1), "GridA", {}, (1, 9, 25)),
    ((6, 7), (1, 1), "GridA", {}, (1, 9, 25)),
    ((6, 7, 6), (1, 1, 1), "Grid3D", {}, (1, 27, 125)),
    ((6, 7, 6), (1, 1, 1), "Grid3D", {"periodic": False}, (1, 8, 27)),
    ((6, 7, 6), (1, 1, 1), "Grid3D", {"periodic": False, "distance": 2}, (1, 27, 125)),
    ((6, 7, 6), (1, 1, 1), "Grid3D", {"distance": 1.5, "metric": "euclidean"}, (1, 27 - 8)),
    ((6, 7, 6), (1, 1, 1), "Grid3D", {"distance": 1.5, "metric": "manhatten"}, (1, 7)),
    ((6, 7, 6), (1, 1, 1), "Grid3D", {"periodic": False, "distance": 2, "metric": "manhatten"},
     (1, 10)),
])
def test_raster_diffusion(dims, start, T, kw, counts):
    """test/raster.jl:34-289"""
    sim = V.create_simulation(raster_model())
    V.add_raster(sim, "grid", dims, T, lambda p: {"pos": p, "active": p == start})
    V.connect_raster_neighbors(sim, "grid", "GridE", lambda a, b: {}, **kw)
    V.finish_init(sim)
    f = V.tr_neighbor_or("GridE", "active")
    assert V.mapreduce(sim, lambda a: a["active"], "+", T) == counts[0]
    for c in counts[1:]:
        V.apply_(sim, f, [T], [T, "GridE"], [T])
        assert V.mapreduce(sim, lambda a: a["active"], "+", T) == c


def test_raster_move_to_counts():
    """test/raster.jl:374-436"""
    sim = V.create_simulation(raster_model())
    V.add_raster(sim, "raster", (10, 10), "Position", lambda p: {"ids_sum": 0})
    p = [V.add_agent(sim, "MovingAgent", {"value": 1}) for _ in range(3)]
    V.move_to(sim, "raster", p[0], (4, 4), ("OnPosition", {}), None, distance=2)
    V.move_to(sim, "raster", p[1], (4, 4), ("OnPosition", {}), None, distance=2, metric="manhatten")
    V.move_to(sim, "raster", p[2], (4, 4), ("OnPosition", {}), None, distance=2.5,
              metric="euclidean")
    V.finish_init(sim)
    V.disable_transition_checks(sim, True)
    assert [V.num_edges(sim, x, "OnPosition") for x in p] == [25, 13, 21]
    sim = V.create_simulation(raster_model())
    V.add_raster(sim, "raster", (10, 10, 10, 10), "Position", lambda p: {"ids_sum": 0})
    p = [V.add_agent(sim, "MovingAgent", {"value": 1}) for _ in range(2)]
    V.move_to(sim, "raster", p[0], (4, 4, 4, 4), ("OnPosition", {}), None, distance=1)
    V.move_to(sim, "raster", p[1], (4, 4, 4, 4), ("OnPosition", {}), None, distance=1,
              metric="manhatten")
    V.finish_init(sim)
    V.disable_transition_checks(sim, True)
    assert [V.num_edges(sim, x, "OnPosition") for x in p] == [81, 9]


# ---------------------------------------------------------- test/graphs.jl
def test_complete_graph_sum():
    """test/graphs.jl:237-266"""
    m = (V.ModelTypes().register_agenttype("GraphA", [("id", "i64"), ("sum", "i64")])
         .register_edgetype("GraphE", []).create_model("g"))
    sim = V.create_simulation(m)
    n = 4
    ids = V.add_agents(sim, "GraphA", [{"id": i, "sum": 0} for i in range(1, n + 1)])
    for a in range(n):  # undirected complete graph: both directions
        for b in range(a + 1, n):
            V.add_edge(sim, ids[a], ids[b], "GraphE")
            V.add_edge(sim, ids[b], ids[a], "GraphE")
    V.finish_init(sim)
    V.apply_(sim, V.tr_neighbor_sum("GraphE", "id", "sum"), ["GraphA"], ["GraphA", "GraphE"],
             ["GraphA"])
    assert V.mapreduce(sim, lambda a: a["sum"], "+", "GraphA") == sum(range(1, n + 1)) * (n - 1)


# ------------------------------------------------------ test/independent.jl
def test_independent_equivalence():
    """test/independent.jl:31-216: the same model under :Independent, without
    it, and the second :Independent type (named Immortal in the reference)
    gives equal agent and edge counts after each of the three transitions:
    agents with foo == 1 die while the others link to and from their
    neighbours, then foo == 2, then every agent adds two agents (foo + 10,
    foo + 20) linked both ways with add_existing."""
    counts = {}
    for T, hints in (("AIndependent", [":Independent"]), ("ANotIndependent", []),
                     ("AIndependentImmortal", [":Independent"])):
        m = (V.ModelTypes().register_agenttype(T, [("foo", "i64")], *hints)
             .register_edgetype("AFooEdge", [("foo", "i64")]).register_edgetype("AEdge", [])
             .create_model("Test Independent"))
        sim = V.create_simulation(m)
        ids = [V.add_agent(sim, T, {"foo": i}) for i in range(1, 11)]
        for a in ids:
            for b in ids:
                V.add_edge(sim, a, b, "AEdge")
        V.finish_init(sim)
        assert V.num_agents(sim, T) == 10
        assert V.num_edges_total(sim, "AEdge") == 100
        c = []
        for foo in (1, 2):
            V.apply_(sim, V.tr_link_neighbors("AEdge", "AFooEdge", foo), T, [T, "AEdge"],
                     [T, "AFooEdge"])
            c.append((V.num_agents(sim, T), V.num_edges_total(sim, "AEdge"),
                      V.num_edges_total(sim, "AFooEdge")))
        V.apply_(sim, V.tr_spawn([10, 20], "AFooEdge"), T, [T, "AEdge"], [T, "AFooEdge"],
                 add_existing="AFooEdge")
        c.append((V.num_agents(sim, T), V.num_edges_total(sim, "AEdge"),
                  V.num_edges_total(sim, "AFooEdge")))
        counts[T] = c
    assert counts["AIndependent"] == counts["ANotIndependent"] == counts["AIndependentImmortal"]
    assert counts["ANotIndependent"] == [(9, 81, 162), (8, 64, 128), (24, 64, 160)]


# ------------------------------------------------- test/parametric_types.jl
def test_parametric_types():
    """test/parametric_types.jl:1-38: a parametric type is one more type
    name; an agent type, a non-parametric agent type and a parametric edge
    type are read back through edges, edgestates and neighborstates"""
    m = (V.ModelTypes().register_agenttype("PAgent{Float64}", [("t", "f64")])
         .register_agenttype("PAgent2", [("t", "f64")])
         .register_edgetype("PEdge{Float64}", [("t", "f64")]).create_model("parametric types"))
    sim = V.create_simulation(m)
    id1 = V.add_agent(sim, "PAgent{Float64}", {"t": 1.0})
    id2 = V.add_agent(sim, "PAgent2", {"t": 2.0})
    V.add_edge(sim, id1, id2, "PEdge{Float64}", {"t": 3.0})
    V.finish_init(sim)
    seen = []

    def f(state, id, sim_):
        assert V.edges(sim_, id, "PEdge{Float64}")[0].state["t"] == 3.0
        assert V.edgestates(sim_, id, "PEdge{Float64}") == [{"t": 3.0}]
        assert V.neighborstates(sim_, id, "PEdge{Float64}", "PAgent{Float64}") == [{"t": 1.0}]
        seen.append(id)
        return state
    V.apply_(sim, f, "PAgent2", ["PAgent{Float64}", "PAgent2", "PEdge{Float64}"], "PAgent2")
    assert seen == [id2]
    assert V.type_nr(id1) != V.type_nr(id2)


# ------------------------------------------------------ test/addexisting.jl
def test_add_existing_reset():
    """test/addexisting.jl:127-184 (the parts without add_agent! in a transition)"""
    m = (V.ModelTypes().register_agenttype("ComputeAgent", [])
         .register_agenttype("ConstructedAgent", []).register_edgetype("Connection", [])
         .create_model("Test add_existing"))
    sim = V.create_simulation(m)
    c = V.add_agent(sim, "ComputeAgent", {})
    k = V.add_agent(sim, "ConstructedAgent", {})
    V.add_edge(sim, k, c, "Connection")
    V.finish_init(sim)
    assert len(sim.E["Connection"]["aot"][k]) == 1
    V.apply_(sim, lambda s, id, sim_: None, "ComputeAgent", [], "Connection",
             add_existing="Connection")
    assert len(sim.E["Connection"]["aot"][k]) == 1
    V.apply_(sim, lambda s, id, sim_: None, ["ComputeAgent"], [],
             ["ConstructedAgent", "Connection"])
    assert len(sim.E["Connection"]["aot"]) == 0
    assert V.num_agents(sim, "ComputeAgent") == 1
    assert V.num_agents(sim, "ConstructedAgent") == 0
    assert V.num_edges_total(sim, "Connection") == 0
    m2 = (V.ModelTypes().register_agenttype("ComputeAgent", [])
          .register_agenttype("ConstructedAgent", [], ":Immortal")
          .register_edgetype("Connection", []).create_model("imm"))
    sim = V.create_simulation(m2)
    V.add_agent(sim, "ComputeAgent", {})
    V.finish_init(sim)
    with pytest.raises(AssertionError):
        V.apply_(sim, lambda s, id, sim_: s, ["ComputeAgent"], [],
                 ["ConstructedAgent", "Connection"])
