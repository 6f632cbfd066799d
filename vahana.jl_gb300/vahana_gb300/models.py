"""The three test models of the transition step, written against the API.

Each builder returns a `Run` with the simulation, its types and a `step()`
that performs one model step (one or more apply! calls).  Initial states are
drawn with Philox4x32-10 on the host; graphs come from the device
generators (the add_edge! loops of the model scripts).

  sir:      Person{state::UInt8, days::Int32} (:Immortal), Contact
            (:Stateless, :SingleType target=Person); k uniform out-edges per
            agent; transition "sir".
  opinion:  Opinion{x::Float64} (:Immortal), Weight{w::Float64}
            (:SingleType target=Opinion); directed Chung-Lu graph;
            transition "bounded_confidence".
  life:     Cell{alive::Bool} raster with implicit Moore edges (Neighbor),
            Walker{x::Int32, y::Int32} moving by Philox Moore offsets and
            rebuilding walker -> cell edges (OnCell, :Stateless, :SingleType
            target=Cell) every step; transitions "life" and "random_walk".
"""
import ctypes as C

import numpy as np

from . import api, philox
from ._lib import check, lib


class Run:
    def __init__(self, sim, **kw):
        self.sim = sim
        self.__dict__.update(kw)

    def close(self):
        self.sim.close()


# ------------------------------------------------------------------- SIR
def sir_model(name="SIR"):
    return (api.ModelTypes()
            .register_agenttype("Person", [("state", "u8"), ("days", "i32")], ":Immortal")
            .register_edgetype("Contact", [], ":Stateless", target="Person")
            .create_model(name))


def sir_initial_state(n, seed, n_infected=None):
    """0.1 % of the agents (the n_infected with the smallest init draw, ties
    by index) start infected with days = 0."""
    if n_infected is None:
        n_infected = max(1, int(round(n / 1000)))
    d = philox.to_u64(philox.draw(seed, np.arange(1, n + 1, dtype=np.uint64), 0, philox.TAG_INIT))
    order = np.lexsort((np.arange(n), d))
    state = np.zeros(n, dtype=np.uint8)
    state[order[:n_infected]] = 1
    return state, np.zeros(n, dtype=np.int32)


def build_sir(n=100_000, degree=10, beta=0.05, recovery=7, seed=1, stream=None,
              n_infected=None):
    model = sir_model()
    sim = api.create_simulation(model, stream=stream)
    state, days = sir_initial_state(n, seed, n_infected)
    ids = api.add_agents(sim, "Person", n, state=state, days=days)
    check(lib().vg_gen_uniform_out_edges(sim._h, model["Contact"].index, model["Person"].index,
                                         int(degree), int(seed)))
    run = Run(sim, model=model, ids=ids, beta=beta, recovery=recovery, seed=seed, n=n,
              degree=degree)

    run.step = api.prepare_apply(sim, "sir", ["Person"], ["Person", "Contact"], ["Person"],
                                 params=[model["Contact"].index, beta, recovery, seed])
    run.edges_per_step = lambda: n * degree
    return run


# ---------------------------------------------------------------- opinion
def opinion_model(name="Opinion"):
    return (api.ModelTypes()
            .register_agenttype("Opinion", [("x", "f64")], ":Immortal")
            .register_edgetype("Weight", [("w", "f64")], target="Opinion")
            .create_model(name))


def opinion_initial_state(n, seed):
    return philox.unit(philox.to_u64(philox.draw(seed, np.arange(1, n + 1, dtype=np.uint64), 0,
                                                 philox.TAG_INIT)))


# rows above this in-degree are split across a warp (1e-12 relative), the
# others fold in order (bit-exact); the library's default as well
OPINION_HUB_THRESHOLD = 1536


def build_opinion(n=10_000_000, mean_degree=20, gamma=2.5, wmax=1e4, eps=0.3, seed=1,
                  stream=None, hub_threshold=OPINION_HUB_THRESHOLD):
    model = opinion_model()
    sim = api.create_simulation(model, stream=stream)
    x = opinion_initial_state(n, seed)
    ids = api.add_agents(sim, "Opinion", n, x=x)
    nedges = int(round(mean_degree * n))
    check(lib().vg_gen_chung_lu_edges(sim._h, model["Weight"].index, model["Opinion"].index,
                                      nedges, float(mean_degree), float(gamma), float(wmax),
                                      int(seed), 0))
    run = Run(sim, model=model, ids=ids, eps=eps, seed=seed, n=n, nedges=nedges)

    run.step = api.prepare_apply(sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                                 ["Opinion"],
                                 params=[model["Weight"].index, eps, 0.5, 0.5, hub_threshold])
    run.edges_per_step = lambda: nedges
    return run


def staged_edges(sim, E):
    """Edge records staged before finish_init!, in call order: (from, to, payload)."""
    t = sim.T(E)
    n = C.c_uint64()
    check(lib().vg_read_staged_edges(sim._h, t.index, None, None, None, 0, C.byref(n)))
    frm = np.zeros(n.value, dtype=np.uint64)
    to = np.zeros(n.value, dtype=np.uint64)
    cols = [np.zeros(n.value, dtype=t.dtype(f)) for f in range(len(t.fields))]
    ptrs = (C.c_void_p * max(len(cols), 1))(*[c.ctypes.data for c in cols])
    check(lib().vg_read_staged_edges(sim._h, t.index, frm.ctypes.data_as(C.POINTER(C.c_uint64)),
                                     to.ctypes.data_as(C.POINTER(C.c_uint64)),
                                     ptrs if cols else None, n.value, C.byref(n)))
    return frm, to, {f[0]: c for f, c in zip(t.fields, cols)}


# -------------------------------------------------------- batched SIR
def batch_params(n_instances, n_lo=1_000, n_hi=100_000, deg_lo=5, deg_hi=30, beta_lo=0.01,
                 beta_hi=0.1, rec_lo=5, rec_hi=10):
    """Per-instance parameters drawn from Philox(seed = instance index):
    N log-uniform in [n_lo, n_hi], out-degree uniform in [deg_lo, deg_hi],
    beta uniform in [beta_lo, beta_hi], recovery uniform in [rec_lo, rec_hi]."""
    i = np.arange(n_instances, dtype=np.uint64)
    N = np.empty(n_instances, np.int64)
    deg = np.empty(n_instances, np.int32)
    beta = np.empty(n_instances, np.float64)
    rec = np.empty(n_instances, np.int32)
    for k in range(n_instances):
        w = philox.draw(k, 0, 0, philox.TAG_PARAM)
        u = philox.unit(philox.to_u64(w))
        N[k] = int(np.floor(n_lo * (n_hi / n_lo) ** float(u)))
        deg[k] = deg_lo + int(philox.bounded32(w[2], deg_hi - deg_lo + 1))
        w2 = philox.draw(k, 1, 0, philox.TAG_PARAM)
        beta[k] = beta_lo + (beta_hi - beta_lo) * float(philox.unit(philox.to_u64(w2)))
        rec[k] = rec_lo + int(philox.bounded32(w2[2], rec_hi - rec_lo + 1))
    return N, deg, beta, rec, i.copy()


class Batch:
    """Batched SIR ensemble (vg_batch_*): every instance is also kept as its
    own simulation for the one-at-a-time path."""

    def __init__(self, N, deg, beta, rec, seeds, infected_per_1000=1, stream=None):
        self.n = len(N)
        self.N = np.ascontiguousarray(N, np.int64)
        h = C.c_void_p()
        arr = lambda a, t: np.ascontiguousarray(a, t)
        self._keep = [arr(N, np.int64), arr(deg, np.int32), arr(beta, np.float64),
                      arr(rec, np.int32), arr(seeds, np.uint64)]
        k = self._keep
        check(lib().vg_batch_create_sir(
            self.n, k[0].ctypes.data_as(C.POINTER(C.c_int64)),
            k[1].ctypes.data_as(C.POINTER(C.c_int32)), k[2].ctypes.data_as(C.POINTER(C.c_double)),
            k[3].ctypes.data_as(C.POINTER(C.c_int32)), k[4].ctypes.data_as(C.POINTER(C.c_uint64)),
            int(infected_per_1000), C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h

    def step(self, steps, mode=1):
        check(lib().vg_batch_step(self._h, int(steps), int(mode)))

    def step_one(self, i, steps):
        check(lib().vg_batch_step_one(self._h, int(i), int(steps)))

    def states(self, i, which=0):
        n = int(self.N[i])
        s = np.zeros(n, np.uint8)
        d = np.zeros(n, np.int32)
        out = C.c_uint64()
        check(lib().vg_batch_read_states2(self._h, int(i), int(which),
                                          s.ctypes.data_as(C.POINTER(C.c_uint8)),
                                          d.ctypes.data_as(C.POINTER(C.c_int32)), n,
                                          C.byref(out)))
        return s, d

    def graph(self, i):
        nr, ne = C.c_uint64(), C.c_uint64()
        check(lib().vg_batch_read_graph(self._h, int(i), None, None, C.byref(nr), C.byref(ne)))
        rp = np.zeros(nr.value + 1, np.uint32)
        src = np.zeros(max(ne.value, 1), np.uint32)
        check(lib().vg_batch_read_graph(self._h, int(i), rp.ctypes.data_as(C.POINTER(C.c_uint32)),
                                        src.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(nr),
                                        C.byref(ne)))
        return rp, src[:ne.value]

    def info(self):
        a, e, db = C.c_uint64(), C.c_uint64(), C.c_uint64()
        t, p = C.c_int(), C.c_int()
        check(lib().vg_batch_info(self._h, C.byref(a), C.byref(e), C.byref(t), C.byref(p),
                                  C.byref(db)))
        return {"agents": a.value, "edges": e.value, "tpb": t.value, "apt": p.value,
                "device_bytes": db.value}

    def set_launch(self, persistent, tpb=256, bucket_threshold=0xFFFFFFFF):
        """Form of mode 3: 0 graph replay, 1 persistent grid launch (block
        size tpb, warps for agents above bucket_threshold in-edges), 2
        persistent cluster launch."""
        check(lib().vg_batch_set_launch(self._h, int(persistent), int(tpb), int(bucket_threshold)))

    def set_lanes(self, per_step=0, persistent=0):
        """Agents per lane (1, 2, 4) of the per-step and persistent grid
        launches; 0 keeps the autotuner's value."""
        check(lib().vg_batch_set_lanes(self._h, int(per_step), int(persistent)))

    def lanes(self):
        a, p = C.c_int(), C.c_int()
        check(lib().vg_batch_lanes(self._h, C.byref(a), C.byref(p)))
        return {"per_step": a.value, "persistent": p.value}

    def set_cluster(self, ctas, tpb, ilp):
        """Shape of the cluster launch: CTAs per cluster, threads per CTA,
        agents per lane."""
        check(lib().vg_batch_set_cluster(self._h, int(ctas), int(tpb), int(ilp)))

    def cluster(self):
        c, t, i, g = C.c_int(), C.c_int(), C.c_int(), C.c_uint()
        check(lib().vg_batch_cluster(self._h, C.byref(c), C.byref(t), C.byref(i), C.byref(g)))
        return {"ctas": c.value, "tpb": t.value, "ilp": i.value, "clusters": g.value}

    FORMS = ("graph", "persistent_grid", "persistent_cluster")

    def tuning(self):
        p, t, n = C.c_int(), C.c_int(), C.c_uint64()
        thr = C.c_uint32()
        gm, pm, cm = C.c_double(), C.c_double(), C.c_double()
        check(lib().vg_batch_tuning(self._h, C.byref(p), C.byref(t), C.byref(thr), C.byref(n),
                                    C.byref(gm), C.byref(pm), C.byref(cm)))
        return {"form": self.FORMS[p.value], "persistent_tpb": t.value,
                "bucket_threshold": thr.value, "heavy_agents": n.value,
                "trial_ms_per_step_graph": gm.value, "trial_ms_per_step_persistent": pm.value,
                "trial_ms_per_step_cluster": cm.value}

    def close(self):
        if self._h:
            check(lib().vg_batch_destroy(self._h))
            self._h = None


# ------------------------------------------------------- Life + walkers
def life_model(name="Life"):
    return (api.ModelTypes()
            .register_agenttype("Cell", [("alive", "bool")], ":Immortal")
            .register_agenttype("Walker", [("x", "i32"), ("y", "i32")], ":Immortal")
            .register_edgetype("Neighbor", [], ":Stateless", target="Cell")
            .register_edgetype("OnCell", [], ":Stateless", target="Cell")
            .create_model(name))


def life_initial_state(width, height, n_walkers, density, seed):
    c = width * height
    alive = philox.unit(philox.to_u64(philox.draw(seed, np.arange(1, c + 1, dtype=np.uint64), 0,
                                                  philox.TAG_INIT))) < density
    w = philox.draw(seed, np.arange(1, n_walkers + 1, dtype=np.uint64), 1, philox.TAG_INIT)
    x = (philox.bounded32(w[0], width) + 1).astype(np.int32)
    y = (philox.bounded32(w[1], height) + 1).astype(np.int32)
    return alive, x, y


def build_life(width=4096, height=4096, n_walkers=1_000_000, density=0.3, seed=1, stream=None):
    model = life_model()
    sim = api.create_simulation(model, stream=stream)
    alive, x, y = life_initial_state(width, height, n_walkers, density, seed)
    api.add_raster(sim, "raster", (width, height), "Cell", alive=alive)
    api.connect_raster_neighbors(sim, "raster", "Neighbor", implicit=True)
    wids = api.add_agents(sim, "Walker", n_walkers, x=x, y=y)
    # initial walker -> cell edges (move_to! in the init phase)
    cells = (np.uint64(model["Cell"].index) << np.uint64(56)) | (
        (x.astype(np.uint64) - 1) + (y.astype(np.uint64) - 1) * np.uint64(width) + np.uint64(1))
    if n_walkers:
        api.add_edges(sim, "OnCell", wids, cells)
    run = Run(sim, model=model, width=width, height=height, n_walkers=n_walkers, seed=seed)

    life = api.prepare_apply(sim, "life", ["Cell"], ["Cell", "Neighbor"], ["Cell"],
                             params=[model["Neighbor"].index])
    walk = api.prepare_apply(sim, "random_walk", ["Walker"], ["Walker"], ["Walker", "OnCell"],
                             params=[model["OnCell"].index, 0, seed])

    def step():
        life()
        walk()
    run.step = step
    run.edges_per_step = lambda: 8 * width * height + n_walkers
    return run
