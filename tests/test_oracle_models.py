"""The C restatement of the three test models (oracle/models.c) agrees with
the same models written as ordinary transition functions on the generic
oracle (oracle/vahana_ref.py, which the reference's own known-answer tests
pin), on small seeded graphs.  Exact equality, Float64 included.
"""
import numpy as np

from oracle import models as om
from oracle import vahana_ref as V

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85


def philox(c, seed):
    """Philox4x32-10 in plain Python (Salmon et al., SC'11)."""
    c = list(c)
    k0, k1 = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
    for _ in range(10):
        p0, p1 = M0 * c[0], M1 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k0, p1 & 0xFFFFFFFF, (p0 >> 32) ^ c[3] ^ k1, p0 & 0xFFFFFFFF]
        k0, k1 = (k0 + W0) & 0xFFFFFFFF, (k1 + W1) & 0xFFFFFFFF
    return c


def unit(o):
    return float(((o[1] << 32 | o[0]) >> 11)) * 2.0 ** -53


def test_philox_matches_c():
    for ctr in [(0, 0, 0, 0), (1, 2, 3, 4), (0xFFFFFFFF, 7, 9, 3)]:
        assert philox(ctr, 0x123456789ABCDEF) == list(om.philox(*ctr, 0x123456789ABCDEF))


def test_sir_generic_vs_c():
    n, k, beta, rec, seed, steps = 300, 6, 0.2, 4, 3, 12
    frm, to = om.gen_uniform_out(n, k, seed)
    state = np.zeros(n, np.uint8)
    state[[5, 77, 140]] = 1
    days = np.zeros(n, np.int32)
    m = (V.ModelTypes().register_agenttype("Person", [("state", "u8"), ("days", "i32")],
                                           ":Immortal")
         .register_edgetype("Contact", [], ":Stateless", target="Person").create_model("SIR"))
    sim = V.create_simulation(m)
    ids = V.add_agents(sim, "Person", [{"state": int(s), "days": 0} for s in state])
    for f, t in zip(frm, to):
        V.add_edge(sim, ids[V.agent_nr(int(f)) - 1], ids[V.agent_nr(int(t)) - 1], "Contact")
    V.finish_init(sim)

    def sir(a, id, s):
        st, d = a["state"], a["days"]
        if st == 0:
            ns = V.neighborstates(s, id, "Contact", "Person") or []
            kk = 0
            for x in ns:  # explicit loop, no sum()
                kk += x["state"] == 1
            if kk > 0:
                q = 1.0
                for _ in range(kk):
                    q = q * (1.0 - beta)
                if unit(philox((V.agent_nr(id), 0, s.num_transitions, 3), seed)) < 1.0 - q:
                    st, d = 1, 0
        elif st == 1:
            d = d + 1
            if d >= rec:
                st = 2
        return {"state": st, "days": d}
    for _ in range(steps):
        V.apply_(sim, sir, "Person", ["Person", "Contact"], "Person")
    gen = V.all_agents(sim, "Person")
    s_c, d_c = om.run_sir(n, frm, to, state, days, beta, rec, seed, steps)
    assert [a["state"] for a in gen] == list(s_c)
    assert [a["days"] for a in gen] == list(d_c)
    assert 2 in list(s_c)


def test_opinion_generic_vs_c():
    n, E, seed, steps = 400, 5000, 5, 6
    frm, to, w = om.gen_chung_lu(n, E, 12.5, 2.5, 60.0, seed)
    x0 = [unit(philox((i, 0, 0, 1), seed)) for i in range(1, n + 1)]
    m = (V.ModelTypes().register_agenttype("Opinion", [("x", "f64")], ":Immortal")
         .register_edgetype("Weight", [("w", "f64")], target="Opinion").create_model("HK"))
    sim = V.create_simulation(m)
    ids = V.add_agents(sim, "Opinion", [{"x": v} for v in x0])
    for f, t, ww in zip(frm, to, w):
        V.add_edge(sim, ids[V.agent_nr(int(f)) - 1], ids[V.agent_nr(int(t)) - 1], "Weight",
                   {"w": float(ww)})
    V.finish_init(sim)

    def bc(a, id, s):
        xi = a["x"]
        es = V.edges(s, id, "Weight") or []
        sw = swx = 0.0
        cnt = 0
        for e in es:
            xj = V.agentstate(s, e.frm, "Opinion")["x"]
            if abs(xj - xi) < 0.3:
                sw = sw + e.state["w"]
                swx = swx + e.state["w"] * xj
                cnt += 1
        return {"x": 0.5 * xi + 0.5 * (swx / sw) if cnt else xi}
    for _ in range(steps):
        V.apply_(sim, bc, "Opinion", ["Opinion", "Weight"], "Opinion")
    gen = np.array([a["x"] for a in V.all_agents(sim, "Opinion")])
    ref = om.run_opinion(n, frm, to, w, np.array(x0), 0.3, steps)
    np.testing.assert_array_equal(gen.view(np.uint64), ref.view(np.uint64))


def test_life_walkers_generic_vs_c():
    W, H, nw, seed, steps = 9, 7, 12, 8, 4
    alive = np.array([unit(philox((c, 0, 0, 1), seed)) < 0.35 for c in range(1, W * H + 1)])
    wx = [philox((i, 0, 1, 1), seed) for i in range(1, nw + 1)]
    x0 = np.array([((o[0] * W) >> 32) + 1 for o in wx], np.int32)
    y0 = np.array([((o[1] * H) >> 32) + 1 for o in wx], np.int32)
    m = (V.ModelTypes().register_agenttype("Cell", [("alive", "bool")], ":Immortal")
         .register_agenttype("Walker", [("x", "i32"), ("y", "i32")], ":Immortal")
         .register_edgetype("Neighbor", [], ":Stateless", target="Cell")
         .register_edgetype("OnCell", [], ":Stateless", target="Cell").create_model("Life"))
    sim = V.create_simulation(m)
    flat = alive.reshape((H, W)).T  # column-major: cell (x, y) at index (x-1) + (y-1) W
    V.add_raster(sim, "raster", (W, H), "Cell", lambda p: {"alive": bool(flat[p[0] - 1, p[1] - 1])})
    V.connect_raster_neighbors(sim, "raster", "Neighbor", lambda a, b: None)
    wids = V.add_agents(sim, "Walker", [{"x": int(a), "y": int(b)} for a, b in zip(x0, y0)])
    for i, wid in enumerate(wids):
        V.move_to(sim, "raster", wid, (int(x0[i]), int(y0[i])), None, ("OnCell", None))
    V.finish_init(sim)
    moore = [(-1, -1), (0, -1), (1, -1), (-1, 0), (1, 0), (-1, 1), (0, 1), (1, 1)]

    def life(a, id, s):
        ns = V.neighborstates(s, id, "Neighbor", "Cell") or []
        c = 0
        for x in ns:
            c += 1 if x["alive"] else 0
        return {"alive": c == 3 or (a["alive"] and c == 2)}

    def walk(a, id, s):
        o = philox((V.agent_nr(id), 0, s.num_transitions, 4), seed)
        dx, dy = moore[(o[0] * 8) >> 32]
        nx = (a["x"] + dx - 1) % W + 1
        ny = (a["y"] + dy - 1) % H + 1
        V.move_to(s, "raster", id, (nx, ny), None, ("OnCell", None))
        return {"x": nx, "y": ny}
    for _ in range(steps):
        V.apply_(sim, life, "Cell", ["Cell", "Neighbor"], "Cell")
        V.apply_(sim, walk, "Walker", "Walker", ["Walker", "OnCell"])
    a_c, x_c, y_c, rp_c, src_c = om.run_life_walkers(alive, x0, y0, W, H, seed, steps)
    cells = V.all_agents(sim, "Cell")
    assert [bool(c["alive"]) for c in cells] == [bool(v) for v in a_c]
    walkers = V.all_agents(sim, "Walker")
    assert [w["x"] for w in walkers] == list(x_c)
    assert [w["y"] for w in walkers] == list(y_c)
    V.disable_transition_checks(sim, True)
    grid = sim.rasters["raster"][1]
    for c in range(W * H):
        pos = (c % W + 1, c // W + 1)
        ids = V.neighborids(sim, grid[pos], "OnCell") or []
        assert [V.agent_nr(i) for i in ids] == list(src_c[int(rp_c[c]):int(rp_c[c + 1])])


def test_life_bounded_generic_vs_c():
    """The C restatement's Life on a bounded raster (positions outside are
    dropped, src/Raster.jl:479-499) equals Life written as a transition on
    the generic oracle with connect_raster_neighbors!(periodic = false)."""
    W, H, steps = 8, 6, 5
    rng = np.random.default_rng(4)
    alive = rng.random(W * H) < 0.4
    m = (V.ModelTypes().register_agenttype("Cell", [("alive", "bool")], ":Immortal")
         .register_edgetype("Neighbor", [], ":Stateless", target="Cell").create_model("LifeB"))
    sim = V.create_simulation(m)
    flat = alive.reshape((H, W)).T
    V.add_raster(sim, "raster", (W, H), "Cell", lambda p: {"alive": bool(flat[p[0] - 1, p[1] - 1])})
    V.connect_raster_neighbors(sim, "raster", "Neighbor", lambda a, b: None, periodic=False)
    V.finish_init(sim)

    def life(a, id, s):
        c = sum(1 for x in (V.neighborstates(s, id, "Neighbor", "Cell") or []) if x["alive"])
        return {"alive": c == 3 or (a["alive"] and c == 2)}
    ref = alive.astype(np.uint8)
    for _ in range(steps):
        V.apply_(sim, life, "Cell", ["Cell", "Neighbor"], "Cell")
        ref = om.life_step(ref, W, H, periodic=False)
    assert [bool(c["alive"]) for c in V.all_agents(sim, "Cell")] == [bool(v) for v in ref]
