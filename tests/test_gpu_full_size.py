"""Parity at the workloads' stated sizes and step counts (GPU, through the
C ABI) against the oracle's C restatement on the same seeded inputs.

  SIR            N = 10^5, 10 out-edges per agent, 100 steps: bit-exact.
  opinion        N = 10^7, E = 2*10^8 (Chung-Lu, exponent 2.5, mean 20,
                 expected degree capped at 10^4), 50 steps.  With the
                 default hub threshold (1536 in-edges): after one step every
                 row up to the threshold bit-exact and the hub rows within
                 1e-12 relative; after 50 steps every row within 1e-12
                 relative (hub differences reach their neighbours).  On the
                 ordered path (no split): bit-exact after 50 steps.
  Life + walkers 4096 x 4096 periodic cells, 10^6 walkers, 1000 steps:
                 cells, walkers and the rebuilt walker -> cell containers
                 bit-exact.
  ensemble       512 SIR instances, 200 steps: every instance bit-identical
                 batched, stepped alone with the plain kernels, and in the
                 oracle.

The oracle builds its own per-target containers from the edge records staged
before finish_init! (add_edge! call order), never from the library's CSR.
"""
import numpy as np
import pytest

from oracle import models as om

pytestmark = pytest.mark.gpu

NO_SPLIT = 4294967295
RTOL = 1e-12


def _max_rel(got, ref):
    diff = got.view(np.uint64) != ref.view(np.uint64)
    if not diff.any():
        return 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.abs(got[diff] - ref[diff]) / np.abs(ref[diff])
    rel[~np.isfinite(rel)] = np.inf
    return float(rel.max())


def test_sir_full_size(vh):
    from vahana_gb300 import models
    run = models.build_sir(n=100_000, degree=10, beta=0.05, recovery=7, seed=1)
    frm, to, _ = models.staged_edges(run.sim, "Contact")
    st0, d0 = vh.read_agents(run.sim, "Person")[0].values()
    st0, d0 = st0.copy(), d0.copy()
    assert int((st0 == 1).sum()) == 100  # 0.1 % start infected
    vh.finish_init(run.sim)
    for _ in range(100):
        run.step()
    cols = vh.read_agents(run.sim, "Person")[0]
    s_ref, d_ref = om.run_sir(run.n, frm, to, st0, d0, 0.05, 7, 1, 100, first_step=1)
    np.testing.assert_array_equal(cols["state"], s_ref)
    np.testing.assert_array_equal(cols["days"], d_ref)
    assert (s_ref == 2).sum() > 1000  # the epidemic spread
    run.close()


def test_opinion_full_size(vh):
    from vahana_gb300 import models
    run = models.build_opinion(n=10_000_000, mean_degree=20, gamma=2.5, wmax=1e4, eps=0.3,
                               seed=1)
    sim, m = run.sim, run.model
    x0 = vh.read_agents(sim, "Opinion")[0]["x"].copy()
    frm, to, pl = models.staged_edges(sim, "Weight")
    assert frm.size == 200_000_000
    g = om.build_inedges(run.n, frm, to)
    del frm, to
    w = np.ascontiguousarray(pl["w"][g[2]])
    del pl
    vh.finish_init(sim)
    ref1 = om.opinion_step(g, w, x0, 0.3)
    ref = ref1
    for _ in range(49):
        ref = om.opinion_step(g, w, ref, 0.3)
    deg = np.diff(g[0].astype(np.int64))
    hub = deg > models.OPINION_HUB_THRESHOLD
    assert 1000 < hub.sum() < 10000 and deg.max() > 5000

    def steps(thr, k):
        for _ in range(k):
            vh.apply_(sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                      ["Opinion"], params=[m["Weight"].index, 0.3, 0.5, 0.5, thr])
        return vh.read_agents(sim, "Opinion")[0]["x"].copy()

    x1 = steps(models.OPINION_HUB_THRESHOLD, 1)
    np.testing.assert_array_equal(x1[~hub].view(np.uint64), ref1[~hub].view(np.uint64))
    assert _max_rel(x1[hub], ref1[hub]) <= RTOL
    x50 = steps(models.OPINION_HUB_THRESHOLD, 49)
    assert _max_rel(x50, ref) <= RTOL
    vh.write_agents(sim, "Opinion", x=x0)
    xo = steps(NO_SPLIT, 50)
    np.testing.assert_array_equal(xo.view(np.uint64), ref.view(np.uint64))
    assert not np.array_equal(xo, x0)
    run.close()


def test_life_walkers_full_size(vh):
    from vahana_gb300 import models
    W = H = 4096
    nw, seed, K = 1_000_000, 1, 1000
    run = models.build_life(W, H, nw, 0.3, seed)
    sim = run.sim
    a0 = vh.read_agents(sim, "Cell")[0]["alive"].copy()
    wc = vh.read_agents(sim, "Walker")[0]
    x0, y0 = wc["x"].copy(), wc["y"].copy()
    vh.finish_init(sim)
    vh.set_async(sim, True)
    for _ in range(K):
        run.step()
    vh.synchronize(sim)
    a = vh.read_agents(sim, "Cell")[0]["alive"]
    wk = vh.read_agents(sim, "Walker")[0]
    a_ref, x_ref, y_ref, rp_ref, src_ref = om.run_life_walkers(a0, x0, y0, W, H, seed, K)
    np.testing.assert_array_equal(a.astype(np.uint8), a_ref)
    np.testing.assert_array_equal(wk["x"], x_ref)
    np.testing.assert_array_equal(wk["y"], y_ref)
    rp, frm, _ = vh.read_edges(sim, "OnCell", "Cell")
    np.testing.assert_array_equal(rp, rp_ref)
    np.testing.assert_array_equal(frm & np.uint64((1 << 36) - 1), src_ref)
    assert 0 < a_ref.sum() < W * H
    run.close()


def test_ensemble_full_size(vh):
    from vahana_gb300 import models
    N, deg, beta, rec, seeds = models.batch_params(512)
    b = models.Batch(N, deg, beta, rec, seeds)
    b.step(200, mode=3)  # the autotuner's form
    for i in range(b.n):
        b.step_one(i, 200)
    bad = []
    for i in range(b.n):
        sb, db = b.states(i, which=0)
        sp, dp = b.states(i, which=1)
        if not (np.array_equal(sb, sp) and np.array_equal(db, dp)):
            bad.append(("plain", i))
        n_i = int(N[i])
        frm, to = om.gen_uniform_out(n_i, int(deg[i]), int(seeds[i]))
        st0, d0 = models.sir_initial_state(n_i, int(seeds[i]), max(1, int(round(n_i / 1000))))
        s_ref, d_ref = om.run_sir(n_i, frm, to, st0, d0, float(beta[i]), int(rec[i]),
                                  int(seeds[i]), 200, first_step=1)
        if not (np.array_equal(sb, s_ref) and np.array_equal(db, d_ref)):
            bad.append(("oracle", i))
    # the persistent cluster form from the same initial state
    bc = models.Batch(N, deg, beta, rec, seeds)
    bc.step(200, mode=4)
    for i in range(b.n):
        sc, dc = bc.states(i, which=0)
        sp, dp = b.states(i, which=1)
        if not (np.array_equal(sc, sp) and np.array_equal(dc, dp)):
            bad.append(("cluster", i))
    bc.close()
    assert bad == []
    b.close()
