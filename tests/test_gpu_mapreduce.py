"""mapreduce over Float64 fields (src/AgentMethods.jl:533-565,
src/EdgeMethods.jl:972-1001): the reference folds sequentially,
reduced = op(f(x), reduced), starting from val4empty (src/Helpers.jl:44-81).

  Float + and * (default): the sequential fold in index order, bit-exact
      (tolerance 0) over 10^6 agents of which about 30 % died.
  the tree form (ordered=False): within the stated bound
      |tree - sequential| <= 2 (n - 1) 2^-53 sum |f(x)|.
  Float max / min: Julia's semantics (a NaN gives NaN, +0.0 > -0.0), any
      order.
  edges of a :SingleType type: the reference iterates the Vector container
      in target index order, each target's edges in insertion order; the
      sequential fold over the same order is bit-exact.
"""
import numpy as np
import pytest

from oracle import models as om

pytestmark = pytest.mark.gpu


def val_model(vh):
    return (vh.ModelTypes()
            .register_agenttype("Val", [("x", "f64"), ("u", "f64")])
            .register_edgetype("Link", [("w", "f64")], target="Val")
            .create_model("Reduce"))


def seq(op, init, xs):
    """The reference's loop: reduced = op(x, reduced) for x in order."""
    vals = np.concatenate([[init], xs]).astype(np.float64)
    acc = np.add.accumulate if op == "+" else np.multiply.accumulate
    return float(acc(vals)[-1])


def test_float_mapreduce_agents_with_deaths(vh):
    rng = np.random.default_rng(31)
    n = 1_000_000
    m = val_model(vh)
    sim = vh.create_simulation(m)
    # mixed signs and magnitudes: the fold order shows in the last bits
    x = rng.standard_normal(n) * np.exp(rng.uniform(-20, 20, n))
    u = rng.random(n)
    vh.add_agents(sim, "Val", n, x=x, u=u)
    vh.finish_init(sim)
    vh.apply_(sim, "die_if", ["Val"], ["Val"], ["Val"], params=[1, 1, 0.7])  # u >= 0.7 dies
    alive = u < 0.7
    assert 0.25 < 1 - alive.mean() < 0.35
    xs = x[alive]
    got = vh.mapreduce(sim, "x", "+", "Val")
    ref = seq("+", 0.0, xs)
    assert np.float64(got).view(np.uint64) == np.float64(ref).view(np.uint64)
    got = vh.mapreduce(sim, "x", "+", "Val", init=1.5)
    assert np.float64(got).view(np.uint64) == np.float64(seq("+", 1.5, xs)).view(np.uint64)
    tree = vh.mapreduce(sim, "x", "+", "Val", ordered=False)
    bound = 2 * (xs.size - 1) * 2.0 ** -53 * np.abs(xs).sum()
    assert abs(tree - ref) <= bound
    # a product of factors near 1 (no overflow), sequential
    vh.write_agents(sim, "Val", x=1.0 + (x / np.abs(x).max()) * 1e-3, u=u)
    y = 1.0 + (x / np.abs(x).max()) * 1e-3
    got = vh.mapreduce(sim, "x", "*", "Val")
    assert np.float64(got).view(np.uint64) == np.float64(seq("*", 1.0, y[alive])).view(np.uint64)
    assert vh.mapreduce(sim, "x", "max", "Val") == y[alive].max()
    assert vh.mapreduce(sim, "x", "min", "Val") == y[alive].min()
    sim.close()


def test_float_max_min_julia_semantics(vh):
    m = val_model(vh)
    sim = vh.create_simulation(m)
    vh.add_agents(sim, "Val", 3, x=np.array([-0.0, 0.0, -0.0]), u=np.zeros(3))
    vh.finish_init(sim)
    mx = vh.mapreduce(sim, "x", "max", "Val")
    mn = vh.mapreduce(sim, "x", "min", "Val")
    assert mx == 0.0 and not np.signbit(mx)
    assert mn == 0.0 and np.signbit(mn)
    vh.write_agents(sim, "Val", x=np.array([1.0, np.nan, 3.0]), u=np.zeros(3))
    assert np.isnan(vh.mapreduce(sim, "x", "max", "Val"))
    assert np.isnan(vh.mapreduce(sim, "x", "min", "Val"))
    sim.close()


def test_float_mapreduce_singletype_edges(vh):
    rng = np.random.default_rng(7)
    n, E = 50_000, 2_000_000
    m = val_model(vh)
    sim = vh.create_simulation(m)
    ids = vh.add_agents(sim, "Val", n, x=np.zeros(n), u=np.zeros(n))
    frm = ids[rng.integers(0, n, E)]
    to = ids[rng.integers(0, n, E)]
    w = rng.standard_normal(E) * np.exp(rng.uniform(-10, 10, E))
    vh.add_edges(sim, "Link", frm, to, w=w)
    vh.finish_init(sim)
    g = om.build_inedges(n, frm, to)  # per target in add_edge! order
    ref = seq("+", 0.0, w[g[2]])
    got = vh.mapreduce(sim, "w", "+", "Link")
    assert np.float64(got).view(np.uint64) == np.float64(ref).view(np.uint64)
    tree = vh.mapreduce(sim, "w", "+", "Link", ordered=False)
    assert abs(tree - ref) <= 2 * (E - 1) * 2.0 ** -53 * np.abs(w).sum()
    sim.close()
