"""Checkpoint and restore (the role of write_snapshot / read_snapshot!,
src/HDF5.jl): a simulation saved between transitions and loaded into the
same model holds the same agents, died flags, reuse stack, edges and
rasters, and continues bit-identically to the original."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same_x(vh, a, b, T, field):
    xa = vh.read_agents(a, T)[0][field]
    xb = vh.read_agents(b, T)[0][field]
    assert xa.dtype == xb.dtype
    np.testing.assert_array_equal(xa.view(np.uint8), xb.view(np.uint8))


def test_opinion_checkpoint_continues_bit_identically(vh, tmp_path):
    from vahana_gb300 import models
    run = models.build_opinion(n=20000, mean_degree=20, gamma=2.5, wmax=2000, eps=0.3, seed=4)
    vh.finish_init(run.sim)
    for _ in range(3):
        run.step()
    path = os.fspath(tmp_path / "opinion.vgsnap")
    vh.save_simulation(run.sim, path)
    loaded = vh.load_simulation(run.model, path)
    _same_x(vh, run.sim, loaded, "Opinion", "x")
    E = run.model["Weight"].index
    assert vh.num_edges(loaded, "Weight") == vh.num_edges(run.sim, "Weight")
    for _ in range(4):
        run.step()
        vh.apply_(loaded, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"], ["Opinion"],
                  params=[E, 0.3, 0.5, 0.5, models.OPINION_HUB_THRESHOLD])
    _same_x(vh, run.sim, loaded, "Opinion", "x")
    loaded.close()
    run.close()


def test_life_walkers_checkpoint(vh, tmp_path):
    """implicit raster edges, rebuilt walker edges and raster dims survive"""
    from vahana_gb300 import models
    run = models.build_life(64, 48, 300, 0.3, 9)
    vh.finish_init(run.sim)
    for _ in range(4):
        run.step()
    path = os.fspath(tmp_path / "life.vgsnap")
    vh.save_simulation(run.sim, path)
    loaded = vh.load_simulation(run.model, path)
    np.testing.assert_array_equal(vh.rastervalues(loaded, "raster", "alive"),
                                  vh.rastervalues(run.sim, "raster", "alive"))
    m = run.model
    for _ in range(5):
        run.step()
        vh.apply_(loaded, "life", ["Cell"], ["Cell", "Neighbor"], ["Cell"],
                  params=[m["Neighbor"].index])
        vh.apply_(loaded, "random_walk", ["Walker"], ["Walker"], ["Walker", "OnCell"],
                  params=[m["OnCell"].index, 0, 9])
    _same_x(vh, run.sim, loaded, "Cell", "alive")
    _same_x(vh, run.sim, loaded, "Walker", "x")
    _same_x(vh, run.sim, loaded, "Walker", "y")
    a = vh.read_edges(run.sim, "OnCell", "Cell")
    b = vh.read_edges(loaded, "OnCell", "Cell")
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    loaded.close()
    run.close()


def test_mortal_agents_reuse_and_edges_checkpoint(vh, tmp_path):
    """deaths, the LIFO reuse stack, mixed-type and stateless edges: the
    seeded transition sequence continued on the original and the restored
    simulation gives the same ids, states and edges after every step"""
    from tests import test_gpu_differential as D
    rng = np.random.default_rng(7)
    sizes = {"A": int(rng.integers(5, 30)), "B": int(rng.integers(5, 30)),
             "C": int(rng.integers(5, 30))}
    foo = {T: rng.integers(1, 50, sizes[T]) for T in sizes}
    n_e1, n_e2 = int(rng.integers(20, 120)), int(rng.integers(20, 120))
    pick = [(T, int(rng.integers(0, sizes[T]))) for T in rng.choice(["A", "B", "C"],
                                                                  2 * (n_e1 + n_e2))]
    seq = D._steps(rng, 14)
    m = D._model(vh)
    sim = vh.create_simulation(m)
    ids = {T: [int(x) for x in vh.add_agents(sim, T, sizes[T], foo=foo[T])] for T, _ in D.TYPES}
    ends = [ids[T][i] for T, i in pick]
    for k in range(n_e1):
        vh.add_edge(sim, ends[2 * k], ends[2 * k + 1], "E1", foo=k)
    for k in range(n_e1, n_e1 + n_e2):
        vh.add_edge(sim, ends[2 * k], ends[2 * k + 1], "E2")
    vh.finish_init(sim)
    for step in seq[:7]:
        D._apply("p", vh, m, sim, step)
    path = os.fspath(tmp_path / "mortal.vgsnap")
    vh.save_simulation(sim, path)
    loaded = vh.load_simulation(m, path)
    assert D._snap(vh, loaded, False) == D._snap(vh, sim, False)
    for n, step in enumerate(seq[7:]):
        D._apply("p", vh, m, sim, step)
        D._apply("p", vh, m, loaded, step)
        assert D._snap(vh, loaded, False) == D._snap(vh, sim, False), "step %d %r" % (n, step)
    loaded.close()
    sim.close()


def test_checkpoint_rules(vh, tmp_path):
    from vahana_gb300 import models
    m = models.sir_model()
    sim = vh.create_simulation(m)
    vh.add_agents(sim, "Person", 10, state=0, days=0)
    with pytest.raises(Exception):  # before finish_init!
        vh.save_simulation(sim, os.fspath(tmp_path / "early.vgsnap"))
    vh.finish_init(sim)
    path = os.fspath(tmp_path / "sir.vgsnap")
    vh.save_simulation(sim, path)
    with pytest.raises(AssertionError):  # another model
        vh.load_simulation(models.opinion_model(), path)
    with open(os.fspath(tmp_path / "junk"), "wb") as f:
        f.write(b"not a snapshot at all")
    with pytest.raises(Exception):
        vh.load_simulation(m, os.fspath(tmp_path / "junk"))
    sim.close()
