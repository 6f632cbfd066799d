"""Differential test of the generic engine: seeded random sequences of the
library's named transitions run on the GPU (through the C ABI) and on the
oracle's sequential restatement of Vahana's state machine, compared after
every apply! -- agent ids (died slots and their LIFO reuse included),
states, and every agent's edges in insertion order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TYPES = [("A", []), ("B", []), ("C", [":Immortal"])]
EDGES = [("E1", [("foo", "i64")], []), ("E2", [], [":Stateless"])]


def _model(M):
    mt = M.ModelTypes()
    for name, hints in TYPES:
        mt = mt.register_agenttype(name, [("foo", "i64")], *hints)
    for name, fields, hints in EDGES:
        mt = mt.register_edgetype(name, fields, *hints)
    return mt.create_model("differential")


def _snap(M, sim, oracle):
    M.disable_transition_checks(sim, True)
    out = {}
    for T, _ in TYPES:
        ids = [int(i) for i in M.all_agentids(sim, T)]
        st = [M.agentstate(sim, i, T)["foo"] for i in ids]
        e1 = [[(int(e.frm), e.state["foo"]) for e in (M.edges(sim, i, "E1") or [])] for i in ids]
        e2 = [[int(x) for x in (M.neighborids(sim, i, "E2") or [])] for i in ids]
        out[T] = (ids, st, e1, e2)
    out["counts"] = ((M.num_edges_total(sim, "E1"), M.num_edges_total(sim, "E2")) if oracle
                     else (M.num_edges(sim, "E1"), M.num_edges(sim, "E2")))
    M.disable_transition_checks(sim, False)
    return out


def _steps(rng, n):
    seq = []
    for _ in range(n):
        T = ["A", "B", "C"][rng.integers(0, 3)]
        k = rng.integers(0, 8)
        if k == 0:
            seq.append(("keep", T, None))
        elif k == 1 and T != "C":
            seq.append(("die_mod", T, int(rng.integers(2, 5))))
        elif k == 2:
            seq.append(("neighbor_sum", T, ["E1", "E2"][rng.integers(0, 2)]))
        elif k == 3:
            seq.append(("self_edge", T, None))
        elif k == 4:
            seq.append(("readd", T, bool(rng.integers(0, 2))))
        elif k == 5:
            seq.append(("spawn", T, int(rng.integers(1, 3))))
        elif k == 6:
            seq.append(("link", T, int(rng.integers(1, 12)) if T != "C" else None))
        else:
            seq.append(("remove", T, (int(rng.integers(0, 3)), int(rng.integers(2, 5)),
                                      int(rng.integers(0, 2)), bool(rng.integers(0, 4)))))
    return seq


def _apply(eng, M, m, sim, step):
    kind, T, arg = step
    R = M
    if kind == "keep":
        if eng == "p":
            M.apply_(sim, "keep", T, [T], [T])
        else:
            M.apply_(sim, R.tr_keep, T, [T], [T])
    elif kind == "die_mod":
        if eng == "p":
            M.apply_(sim, "die_if", T, [T], [T], params=[2, 0, arg])
        else:
            M.apply_(sim, R.tr_die_if("mod", "foo", arg), T, [T], [T])
    elif kind == "neighbor_sum":
        read = ["A", "B", "C", arg]
        if eng == "p":
            M.apply_(sim, "neighbor_sum", T, read, [T], params=[m[arg].index, 0, 0])
        else:
            M.apply_(sim, R.tr_neighbor_sum(arg, "foo", "foo"), T, read, [T])
    elif kind == "self_edge":
        if eng == "p":
            M.apply_(sim, "self_edge", T, [T], [T, "E1"], add_existing=["E1"],
                     params=[m["E1"].index, 7])
        else:
            M.apply_(sim, R.tr_self_edge("E1", {"foo": 7}), T, [T], [T, "E1"],
                     add_existing=["E1"])
    elif kind == "readd":
        ae = ["E1"] if arg else []
        if eng == "p":
            M.apply_(sim, "readd_edges", T, [T, "E1"], [T, "E1"], add_existing=ae,
                     params=[m["E1"].index])
        else:
            M.apply_(sim, R.tr_readd_edges("E1"), T, [T, "E1"], [T, "E1"], add_existing=ae)
    elif kind == "spawn":
        offs = [100, 200][:arg]
        if eng == "p":
            M.apply_(sim, "spawn", T, [T], [T, "E1"], add_existing=["E1"],
                     params=[arg] + offs + [m["E1"].index])
        else:
            M.apply_(sim, R.tr_spawn(offs, "E1"), T, [T], [T, "E1"], add_existing=["E1"])
    elif kind == "remove":
        fk, farg, mode, aex = arg
        read = ["A", "B", "C", "E1"]
        ae = ["E1"] if aex else []
        if eng == "p":
            M.apply_(sim, "remove_edges", T, read, [T, "E1"], add_existing=ae,
                     params=[m["E1"].index, fk, farg, mode])
        else:
            M.apply_(sim, R.tr_remove_edges("E1", fk, farg, mode), T, read, [T, "E1"],
                     add_existing=ae)
    elif kind == "link":
        read = [T, "E2"]
        if eng == "p":
            M.apply_(sim, "link_neighbors", T, read, [T, "E1"], add_existing=["E1"],
                     params=[m["E2"].index, m["E1"].index] + ([arg] if arg is not None else []))
        else:
            M.apply_(sim, R.tr_link_neighbors("E2", "E1", arg), T, read, [T, "E1"],
                     add_existing=["E1"])


@pytest.mark.parametrize("seed", [1, 2, 6, 7, 9, 22, 25, 28, 34, 35])
def test_random_transition_sequences(vh, seed):
    from oracle import vahana_ref as R
    rng = np.random.default_rng(seed)
    sizes = {"A": int(rng.integers(5, 30)), "B": int(rng.integers(5, 30)),
             "C": int(rng.integers(5, 30))}
    foo = {T: rng.integers(1, 50, sizes[T]) for T in sizes}
    n_e1, n_e2 = int(rng.integers(20, 120)), int(rng.integers(20, 120))
    pick = [(T, int(rng.integers(0, sizes[T]))) for T in rng.choice(["A", "B", "C"], 2 * (n_e1 + n_e2))]
    seq = _steps(rng, 14)
    sims = {}
    for eng, M in (("p", vh), ("o", R)):
        m = _model(M)
        sim = M.create_simulation(m)
        ids = {}
        for T, _ in TYPES:
            if eng == "p":
                ids[T] = [int(x) for x in vh.add_agents(sim, T, sizes[T], foo=foo[T])]
            else:
                ids[T] = [R.add_agent(sim, T, {"foo": int(v)}) for v in foo[T]]
        ends = [ids[T][i] for T, i in pick]
        for k in range(n_e1):
            f, t = ends[2 * k], ends[2 * k + 1]
            if eng == "p":
                vh.add_edge(sim, f, t, "E1", foo=k)
            else:
                R.add_edge(sim, f, t, "E1", {"foo": k})
        for k in range(n_e1, n_e1 + n_e2):
            f, t = ends[2 * k], ends[2 * k + 1]
            if eng == "p":
                vh.add_edge(sim, f, t, "E2")
            else:
                R.add_edge(sim, f, t, "E2")
        M.finish_init(sim)
        sims[eng] = (M, m, sim)
    for n, step in enumerate(seq):
        for eng in ("p", "o"):
            M, m, sim = sims[eng]
            _apply(eng, M, m, sim, step)
        sp = _snap(vh, sims["p"][2], False)
        so = _snap(R, sims["o"][2], True)
        assert sp == so, "after step %d %r" % (n, step)
    sims["p"][2].close()
