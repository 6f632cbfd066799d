"""move_to! inside a transition (src/Raster.jl:437-499) on the GPU ("move_to"
kernel), through the C ABI, against the generic oracle calling move_to! in
the same transition: every edge container, per target in insertion order,
must be identical (tolerance 0).

  test/raster.jl:291-370 (Raster_NodeID): agents move to the cell named by
      their cell's state, with edges cell -> agent and agent -> cell of one
      edge type; the raster sums after each step.
  option sweep: distance 0 / 1 / 2 / 2.5, the chebyshev, euclidean and
      manhatten stencils, periodic and bounded rasters (positions on the
      border), only_surrounding, edge_from only, edge_to only, both of one
      type and of two types; 2-D and 3-D rasters.
"""
import itertools

import numpy as np
import pytest

from oracle import vahana_ref as V

pytestmark = pytest.mark.gpu

METRIC = {"chebyshev": 0, "euclidean": 1, "manhatten": 2}


def containers_equal(vh, sim, osim, E, T):
    """The library's CSR of edge type E over target type T against the
    oracle's neighborids, row by row in insertion order."""
    rp, frm, _ = vh.read_edges(sim, E, T)
    V.disable_transition_checks(osim, True)
    try:
        for r, oid in enumerate(V.all_agentids(osim, T)):
            want = V.neighborids(osim, oid, E) or []
            got = [int(x) for x in frm[int(rp[r]):int(rp[r + 1])]] if r + 1 < len(rp) else []
            assert got == [int(x) for x in want], (E, T, r)
    finally:
        V.disable_transition_checks(osim, False)


def test_raster_nodeid_in_apply(vh):
    """test/raster.jl:291-370, value_on_pos as the "move_to" kernel (mode 1)"""
    m = (vh.ModelTypes()
         .register_agenttype("Position", [("ids_sum", "i64")])
         .register_agenttype("MovingAgent", [("value", "i64")])
         .register_edgetype("GridE", [])
         .register_edgetype("OnPosition", [])
         .create_model("Raster_Test"))
    sim = vh.create_simulation(m)
    vh.add_raster(sim, "raster", (10, 10), "Position", ids_sum=0)
    vh.connect_raster_neighbors(sim, "raster", "GridE")
    p = vh.add_agents(sim, "MovingAgent", 3, value=[1, 2, 3])
    for pid, pos in zip(p, [(1, 1), (2, 2), (2, 2)]):
        vh.move_to(sim, "raster", pid, pos, "OnPosition", "OnPosition")
    vh.finish_init(sim)
    E = m["OnPosition"].index

    def sum_on_pos():
        vh.apply_(sim, "neighbor_sum", ["Position"], ["MovingAgent", "OnPosition"], ["Position"],
                  params=[E, 0, 0])
        return vh.rastervalues(sim, "raster", "ids_sum")

    r = sum_on_pos()
    assert (r[0, 0], r[0, 1], r[1, 1], r[1, 2]) == (1, 0, 5, 0)
    vh.apply_(sim, "move_to", ["MovingAgent"], ["Position", "OnPosition"],
              ["OnPosition", "MovingAgent"], params=[0, E, E, 0, 0, 1, 0, 1, E, 0])
    r = sum_on_pos()
    assert (r[0, 0], r[0, 1], r[1, 1], r[4, 4]) == (1, 0, 0, 10)
    assert list(vh.read_agents(sim, "MovingAgent")[0]["value"]) == [1, 5, 5]
    sim.close()


def _sweep_case(vh, dims, dist, metric, periodic, only_sur, dirs, seed):
    rng = np.random.default_rng(seed)
    nd = len(dims)
    fields = [("x", "i64"), ("y", "i64"), ("z", "i64")][:nd]
    m = (vh.ModelTypes()
         .register_agenttype("Cell", [("v", "i64")])
         .register_agenttype("Mover", fields)
         .register_edgetype("In", [])
         .register_edgetype("Out", [])
         .create_model("Move"))
    om_ = V.ModelTypes().register_agenttype("Cell", [("v", "i64")])
    om_ = om_.register_agenttype("Mover", fields).register_edgetype("In", []).register_edgetype(
        "Out", [])
    om_ = om_.create_model("Move")
    n = 40
    sim = vh.create_simulation(m)
    osim = V.create_simulation(om_)
    vh.add_raster(sim, "r", dims, "Cell", v=0)
    V.add_raster(osim, "r", dims, "Cell", lambda pos: {"v": 0})
    start = {f[0]: np.ones(n, np.int64) for f in fields}
    vh.add_agents(sim, "Mover", n, **start)
    V.add_agents(osim, "Mover", [{f[0]: 1 for f in fields} for _ in range(n)])
    vh.finish_init(sim)
    V.finish_init(osim)
    ef = {"from": "In", "to": None, "same": "In", "two": "In"}[dirs]
    et = {"from": None, "to": "Out", "same": "In", "two": "Out"}[dirs]
    write = ["Mover"] + sorted({e for e in (ef, et) if e})
    for step in range(3):
        # positions on the border and inside, drawn per step
        pos = np.stack([rng.choice([1, 2, d // 2 + 1, d - 1, d], n) for d in dims], axis=1)
        vh.write_agents(sim, "Mover", **{f[0]: pos[:, k] for k, f in enumerate(fields)})
        params = [0, m[ef].index if ef else -1, m[et].index if et else -1, dist, METRIC[metric],
                  int(periodic), int(only_sur), 0]
        vh.apply_(sim, "move_to", ["Mover"], ["Mover"], write, params=params)

        def mv(state, id, s, pos=pos):
            nr = V.agent_nr(id) - 1
            p = tuple(int(v) for v in pos[nr])
            V.move_to(s, "r", id, p, (ef, None) if ef else None, (et, None) if et else None,
                      distance=dist, metric=metric, periodic=periodic, only_surrounding=only_sur)
            return {f[0]: p[k] for k, f in enumerate(fields)}
        V.apply_(osim, mv, "Mover", "Mover", write)
        for E in sorted({e for e in (ef, et) if e}):
            for T in ("Cell", "Mover"):
                containers_equal(vh, sim, osim, E, T)
    sim.close()


@pytest.mark.parametrize("dist,metric", [(0, "chebyshev"), (1, "chebyshev"), (2, "chebyshev"),
                                         (2, "manhatten"), (2.5, "euclidean")])
@pytest.mark.parametrize("periodic", [True, False])
def test_move_to_options_2d(vh, dist, metric, periodic):
    for k, (only_sur, dirs) in enumerate(itertools.product([False, True],
                                                           ["from", "to", "same", "two"])):
        if only_sur and dist == 0:
            continue  # nothing to add
        _sweep_case(vh, (7, 5), dist, metric, periodic, only_sur, dirs, seed=k)


@pytest.mark.parametrize("periodic", [True, False])
def test_move_to_3d(vh, periodic):
    _sweep_case(vh, (4, 5, 3), 1, "chebyshev", periodic, False, "two", seed=7)
    _sweep_case(vh, (4, 5, 3), 1.5, "euclidean", periodic, True, "same", seed=8)
