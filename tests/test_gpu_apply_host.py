"""apply! with the called type's state in host memory (vg_apply_host),
through the C ABI: the result equals vg_write_agents + vg_apply +
vg_read_agents bit for bit (tolerance 0), for the bounded-confidence gather
(run in row-range chunks whose downloads overlap the kernel; hub rows split
across warps, several degree windows per chunk) and for a transition without
chunking (SIR); the simulation's own state afterwards is the downloaded one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_apply_host_opinion_matches_apply(vh):
    import torch
    from vahana_gb300 import models
    n = 300_000
    run = models.build_opinion(n=n, mean_degree=20, gamma=2.5, wmax=4000, eps=0.3, seed=13)
    twin = models.build_opinion(n=n, mean_degree=20, gamma=2.5, wmax=4000, eps=0.3, seed=13)
    vh.finish_init(run.sim)
    vh.finish_init(twin.sim)
    m = run.model
    params = [m["Weight"].index, 0.3, 0.5, 0.5, 256]  # many hub rows
    rng = np.random.default_rng(3)
    pinned_in = torch.empty(n, dtype=torch.float64).pin_memory()
    pinned_out = torch.empty(n, dtype=torch.float64).pin_memory()
    for k in range(4):
        x = rng.random(n) if k % 2 == 0 else vh.read_agents(twin.sim, "Opinion")[0]["x"]
        pinned_in.numpy()[:] = x
        out = vh.apply_host(run.sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                            ["Opinion"], "Opinion", {"x": pinned_in.numpy()},
                            out={"x": pinned_out.numpy()}, params=params)
        vh.write_agents(twin.sim, "Opinion", x=x)
        vh.apply_(twin.sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"], ["Opinion"],
                  params=params)
        ref = vh.read_agents(twin.sim, "Opinion")[0]["x"]
        np.testing.assert_array_equal(out["x"].view(np.uint64), ref.view(np.uint64))
        np.testing.assert_array_equal(
            vh.read_agents(run.sim, "Opinion")[0]["x"].view(np.uint64), ref.view(np.uint64))
        assert not np.array_equal(out["x"], x)
    assert vh.num_transitions(run.sim) == vh.num_transitions(twin.sim)
    # unpinned numpy buffers: the same values
    x = rng.random(n)
    got = vh.apply_host(run.sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                        ["Opinion"], "Opinion", {"x": x}, params=params)["x"]
    vh.write_agents(twin.sim, "Opinion", x=x)
    vh.apply_(twin.sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"], ["Opinion"],
              params=params)
    np.testing.assert_array_equal(got.view(np.uint64),
                                  vh.read_agents(twin.sim, "Opinion")[0]["x"].view(np.uint64))
    run.close()
    twin.close()


def test_apply_host_sir_matches_apply(vh):
    from vahana_gb300 import models
    run = models.build_sir(n=20_000, degree=10, beta=0.2, recovery=5, seed=4, n_infected=200)
    twin = models.build_sir(n=20_000, degree=10, beta=0.2, recovery=5, seed=4, n_infected=200)
    vh.finish_init(run.sim)
    vh.finish_init(twin.sim)
    m = run.model
    params = [m["Contact"].index, 0.2, 5, 4]
    st = vh.read_agents(run.sim, "Person")[0]
    state, days = st["state"].copy(), st["days"].copy()
    for _ in range(6):
        out = vh.apply_host(run.sim, "sir", ["Person"], ["Person", "Contact"], ["Person"],
                            "Person", {"state": state, "days": days}, params=params)
        vh.apply_(twin.sim, "sir", ["Person"], ["Person", "Contact"], ["Person"], params=params)
        ref = vh.read_agents(twin.sim, "Person")[0]
        np.testing.assert_array_equal(out["state"], ref["state"])
        np.testing.assert_array_equal(out["days"], ref["days"])
        state, days = out["state"], out["days"]
    assert (state == 2).sum() > 0
    run.close()
    twin.close()


def test_apply_host_ordered_path_and_partial_n(vh):
    """No hub split (no hub warps: every range reports on its own) and a
    host exchange of the first n agents only: equal to write + apply! + read
    of the same agents."""
    from vahana_gb300 import models
    n = 200_000
    run = models.build_opinion(n=n, mean_degree=15, gamma=2.5, wmax=3000, eps=0.3, seed=23)
    twin = models.build_opinion(n=n, mean_degree=15, gamma=2.5, wmax=3000, eps=0.3, seed=23)
    vh.finish_init(run.sim)
    vh.finish_init(twin.sim)
    params = [run.model["Weight"].index, 0.3, 0.5, 0.5, 4294967295]
    rng = np.random.default_rng(8)
    for m in (n, n // 3):
        x = rng.random(m)
        got = vh.apply_host(run.sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                            ["Opinion"], "Opinion", {"x": x}, params=params)["x"]
        vh.write_agents(twin.sim, "Opinion", x=x)
        vh.apply_(twin.sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                  ["Opinion"], params=params)
        ref = vh.read_agents(twin.sim, "Opinion")[0]["x"]
        assert got.size == m
        np.testing.assert_array_equal(got.view(np.uint64), ref[:m].view(np.uint64))
        np.testing.assert_array_equal(vh.read_agents(run.sim, "Opinion")[0]["x"].view(np.uint64),
                                      ref.view(np.uint64))
    run.close()
    twin.close()
