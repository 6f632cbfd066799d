"""Parity of the three test models' transition steps (GPU, through the C ABI)
against the oracle's C restatement, on the same seeded inputs.

Integer, Bool and UInt8 state must be bit-exact; Float64 state of the
bounded-confidence model is bit-exact too (the kernels fold in container
order with separately rounded operations), so the tolerance is 0.
"""
import numpy as np
import pytest

from oracle import models as om

pytestmark = pytest.mark.gpu


def test_sir_bit_exact(vh):
    from vahana_gb300 import models
    run = models.build_sir(n=3000, degree=10, beta=0.05, recovery=7, seed=7, n_infected=30)
    sim = run.sim
    frm, to, _ = models.staged_edges(sim, "Contact")
    st0, d0 = vh.read_agents(sim, "Person")[0].values()
    vh.finish_init(sim)
    steps = 40
    for _ in range(steps):
        run.step()
    cols, died = vh.read_agents(sim, "Person")
    s_ref, d_ref = om.run_sir(run.n, frm, to, st0, d0, 0.05, 7, 7, steps, first_step=1)
    assert not died.any()
    np.testing.assert_array_equal(cols["state"], s_ref)
    np.testing.assert_array_equal(cols["days"], d_ref)
    assert (s_ref == 2).sum() > 0  # the epidemic ran
    run.close()


def test_sir_steps_around_contact_rebuilds(vh):
    """SIR steps run with programmatic dependent launch (the next step reads
    its contact rows before waiting for the previous one) only while no edge
    container was rewritten since the previous step: steps around an
    identical rebuild of the contacts (add_existing) and around the removal
    of every contact equal the oracle's steps on the graph of that moment."""
    from vahana_gb300 import models
    run = models.build_sir(n=3000, degree=10, beta=0.05, recovery=7, seed=11, n_infected=60)
    sim, m = run.sim, run.model
    frm, to, _ = models.staged_edges(sim, "Contact")
    st0, d0 = vh.read_agents(sim, "Person")[0].values()
    vh.finish_init(sim)
    full = om.build_inedges(run.n, frm, to)
    empty = om.build_inedges(run.n, np.zeros(0, np.int64), np.zeros(0, np.int64))
    s_ref, d_ref = np.ascontiguousarray(st0, np.uint8), np.ascontiguousarray(d0, np.int32)
    g, t = full, 1
    plan = ["sir"] * 4 + ["rebuild"] + ["sir"] * 4 + ["remove"] + ["sir"] * 4
    for what in plan:
        if what == "sir":
            run.step()
            s_ref, d_ref = om.sir_step(g, s_ref, d_ref, 0.05, 7, 11, t)
        elif what == "rebuild":  # the same contacts, a new container
            vh.apply_(sim, "keep", ["Person"], ["Person"], ["Contact"], add_existing=["Contact"])
        else:  # every Person removes its contacts
            vh.apply_(sim, "remove_edges", ["Person"], ["Person"], ["Contact"],
                      params=[m["Contact"].index, 0, 0, 0])
            g = empty
        t += 1
        cols = vh.read_agents(sim, "Person")[0]
        np.testing.assert_array_equal(cols["state"], s_ref)
        np.testing.assert_array_equal(cols["days"], d_ref)
    assert vh.num_edges(sim, "Contact") == 0
    run.close()


def test_sir_changing_beta_between_steps(vh):
    """The infection table (1 - (1 - beta)^k per infected-neighbour count)
    is uploaded once per content: a beta that changes between apply! calls
    is picked up at the next call, and going back reuses nothing stale."""
    from vahana_gb300 import models
    run = models.build_sir(n=3000, degree=10, beta=0.05, recovery=7, seed=9, n_infected=30)
    sim, m = run.sim, run.model
    frm, to, _ = models.staged_edges(sim, "Contact")
    st0, d0 = vh.read_agents(sim, "Person")[0].values()
    vh.finish_init(sim)
    g = om.build_inedges(run.n, frm, to)
    s_ref, d_ref = np.ascontiguousarray(st0, np.uint8), np.ascontiguousarray(d0, np.int32)
    betas = [0.05, 0.05, 0.2, 0.2, 0.05, 0.11, 0.2, 0.05] * 3
    for t, beta in enumerate(betas):
        vh.apply_(sim, "sir", ["Person"], ["Person", "Contact"], ["Person"],
                  params=[m["Contact"].index, beta, 7, 9])
        s_ref, d_ref = om.sir_step(g, s_ref, d_ref, beta, 7, 9, t + 1)
    cols = vh.read_agents(sim, "Person")[0]
    np.testing.assert_array_equal(cols["state"], s_ref)
    np.testing.assert_array_equal(cols["days"], d_ref)
    run.close()


def test_sir_beta_bound_to_a_global(vh):
    """The "sir" transition's beta slot bound to a global of the simulation
    (get_global inside the transition, src/Global.jl:10): set_global!
    between apply! calls reaches the kernel; equals the oracle with the same
    beta sequence."""
    from vahana_gb300 import api
    m = (api.ModelTypes()
         .register_agenttype("Person", [("state", "u8"), ("days", "i32")], ":Immortal")
         .register_edgetype("Contact", [], ":Stateless", target="Person")
         .register_global("beta", 0.05)
         .create_model("SIRg"))
    from vahana_gb300 import models
    sim = api.create_simulation(m)
    st, dy = models.sir_initial_state(3000, 9, 30)
    api.add_agents(sim, "Person", 3000, state=st, days=dy)
    from vahana_gb300._lib import check, lib
    check(lib().vg_gen_uniform_out_edges(sim._h, m["Contact"].index, m["Person"].index, 10, 9))
    frm, to, _ = models.staged_edges(sim, "Contact")
    vh.finish_init(sim)
    vh.bind_param(sim, "sir", 1, "beta")
    g = om.build_inedges(3000, frm, to)
    s_ref, d_ref = st.copy(), dy.copy()
    betas = [0.05, 0.2, 0.2, 0.01, 0.11, 0.3] * 3
    for t, beta in enumerate(betas):
        vh.set_global(sim, "beta", beta)
        vh.apply_(sim, "sir", ["Person"], ["Person", "Contact"], ["Person"],
                  params=[m["Contact"].index, 0.0, 7, 9])  # slot 1 comes from the global
        s_ref, d_ref = om.sir_step(g, s_ref, d_ref, beta, 7, 9, t + 1)
    cols = vh.read_agents(sim, "Person")[0]
    np.testing.assert_array_equal(cols["state"], s_ref)
    np.testing.assert_array_equal(cols["days"], d_ref)
    assert (s_ref == 2).sum() > 0
    sim.close()


NO_SPLIT = 4294967295  # hub threshold that keeps every row on the ordered path


def test_opinion_bit_exact(vh):
    """Ordered path (no hub split): tolerance 0, bit-identical binary64."""
    from vahana_gb300 import models
    run = models.build_opinion(n=20000, mean_degree=20, gamma=2.5, wmax=2000, eps=0.3, seed=11,
                               hub_threshold=NO_SPLIT)
    sim = run.sim
    frm, to, pl = models.staged_edges(sim, "Weight")
    x0 = vh.read_agents(sim, "Opinion")[0]["x"].copy()
    vh.finish_init(sim)
    steps = 12
    for _ in range(steps):
        run.step()
    x = vh.read_agents(sim, "Opinion")[0]["x"]
    x_ref = om.run_opinion(run.n, frm, to, pl["w"], x0, 0.3, steps)
    np.testing.assert_array_equal(x.view(np.uint64), x_ref.view(np.uint64))
    assert not np.array_equal(x, x0)
    run.close()


def test_opinion_bit_exact_arbitrary_weights(vh):
    """Weights that are not multiples of 2^-53 take the kernel's binary64
    add path for sw; still bit-identical to the sequential fold."""
    from vahana_gb300 import models
    rng = np.random.default_rng(5)
    n, E = 3000, 60000
    m = models.opinion_model()
    sim = vh.create_simulation(m)
    x0 = rng.random(n)
    ids = vh.add_agents(sim, "Opinion", n, x=x0)
    frm = ids[rng.integers(0, n, E)]
    to = ids[np.minimum(rng.zipf(1.8, E) - 1, n - 1)]  # skewed in-degrees
    w = rng.random(E) * 0.7 + 1e-3                      # off the 2^-53 grid
    vh.add_edges(sim, "Weight", frm, to, w=w)
    vh.finish_init(sim)
    for _ in range(8):
        vh.apply_(sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"], ["Opinion"],
                  params=[m["Weight"].index, 0.3, 0.5, 0.5, NO_SPLIT])
    x = vh.read_agents(sim, "Opinion")[0]["x"]
    ref = om.run_opinion(n, frm, to, w, x0, 0.3, 8)
    np.testing.assert_array_equal(x.view(np.uint64), ref.view(np.uint64))
    sim.close()


@pytest.mark.parametrize("hub", [256, 16])
def test_opinion_hub_split(vh, hub):
    """Hub rows (in-degree > hub) are summed in split chunks: within 1e-12
    relative of the sequential fold; every other row stays bit-exact after
    one step, and all rows stay within 1e-12 over several steps."""
    from vahana_gb300 import models
    run = models.build_opinion(n=20000, mean_degree=20, gamma=2.5, wmax=2000, eps=0.3, seed=11,
                               hub_threshold=hub)
    sim = run.sim
    frm, to, pl = models.staged_edges(sim, "Weight")
    x0 = vh.read_agents(sim, "Opinion")[0]["x"].copy()
    vh.finish_init(sim)
    run.step()
    x1 = vh.read_agents(sim, "Opinion")[0]["x"].copy()
    ref1 = om.run_opinion(run.n, frm, to, pl["w"], x0, 0.3, 1)
    deg = np.bincount((to & np.uint64((1 << 36) - 1)).astype(np.int64) - 1, minlength=run.n)
    hubs = deg > hub
    assert hubs.any()
    np.testing.assert_array_equal(x1[~hubs].view(np.uint64), ref1[~hubs].view(np.uint64))
    np.testing.assert_allclose(x1[hubs], ref1[hubs], rtol=1e-12, atol=0)
    for _ in range(5):
        run.step()
    x = vh.read_agents(sim, "Opinion")[0]["x"]
    ref = om.run_opinion(run.n, frm, to, pl["w"], x0, 0.3, 6)
    np.testing.assert_allclose(x, ref, rtol=1e-12, atol=0)
    run.close()


@pytest.mark.parametrize("weights", ["grid", "arbitrary"])
def test_opinion_block_hubs(vh, weights):
    """With a block threshold of 2048 (parameter 5), rows above it take a
    whole block, their edges staged in shared memory by bulk copies in
    chunks of 512 (unaligned row starts, a row of tens of chunks, tails of
    1-3 edges): within 1e-12 relative of the sequential fold; rows below the
    hub threshold stay bit-exact."""
    from vahana_gb300 import models
    rng = np.random.default_rng(17)
    if weights == "grid":
        run = models.build_opinion(n=60000, mean_degree=20, gamma=2.5, wmax=1e4, eps=0.3,
                                   seed=21, hub_threshold=256)
        sim, m, n = run.sim, run.model, run.n
        frm, to, pl = models.staged_edges(sim, "Weight")
        w = pl["w"]
    else:
        n, E = 8000, 120000
        m = models.opinion_model()
        sim = vh.create_simulation(m)
        ids = vh.add_agents(sim, "Opinion", n, x=rng.random(n))
        frm = ids[rng.integers(0, n, E)]
        to = ids[np.minimum(rng.zipf(1.6, E) - 1, n - 1)]
        w = rng.random(E) * 0.7 + 1e-3
        vh.add_edges(sim, "Weight", frm, to, w=w)
        run = None
    x0 = vh.read_agents(sim, "Opinion")[0]["x"].copy()
    deg = np.bincount((to & np.uint64((1 << 36) - 1)).astype(np.int64) - 1, minlength=n)
    assert (deg > 2048).sum() >= 2 and deg.max() > 8 * 512
    vh.finish_init(sim)
    step = lambda: vh.apply_(sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                             ["Opinion"], params=[m["Weight"].index, 0.3, 0.5, 0.5, 256, 2048])
    step()
    x1 = vh.read_agents(sim, "Opinion")[0]["x"].copy()
    ref1 = om.run_opinion(n, frm, to, w, x0, 0.3, 1)
    hubs = deg > 256
    np.testing.assert_array_equal(x1[~hubs].view(np.uint64), ref1[~hubs].view(np.uint64))
    np.testing.assert_allclose(x1[hubs], ref1[hubs], rtol=1e-12, atol=0)
    for _ in range(4):
        step()
    x = vh.read_agents(sim, "Opinion")[0]["x"]
    np.testing.assert_allclose(x, om.run_opinion(n, frm, to, w, x0, 0.3, 5), rtol=1e-12, atol=0)
    if run is not None:
        run.close()
    else:
        sim.close()


def test_fp64_integer_arithmetic_matches_hardware(vh):
    """The integer-pipe binary64 add/mul/div used by the gather kernels
    equal the hardware instructions on 4M operand pairs (random, ties,
    carries, exponent gaps); out-of-range cases fall back."""
    import ctypes as C
    from vahana_gb300._lib import check, lib
    counts = (C.c_uint64 * 6)()
    check(lib().vg_selftest_fp64(4 << 20, 12345, counts))
    add_bad, mul_bad, div_bad, add_fb, mul_fb, div_fb = list(counts)
    assert (add_bad, mul_bad, div_bad) == (0, 0, 0)
    assert add_fb < (4 << 20) // 4 and mul_fb < (4 << 20) // 4


def test_generators_match_host_restatement(vh):
    """The device graph generators emit the same records, in the same call
    order, as the oracle's host restatement."""
    from vahana_gb300 import models
    run = models.build_opinion(n=50000, mean_degree=20, gamma=2.5, wmax=1e4, seed=9)
    frm, to, pl = models.staged_edges(run.sim, "Weight")
    f2, t2, w2 = om.gen_chung_lu(50000, 1_000_000, 20, 2.5, 1e4, 9)
    np.testing.assert_array_equal(frm, f2)
    np.testing.assert_array_equal(to, t2)
    np.testing.assert_array_equal(pl["w"].view(np.uint64), w2.view(np.uint64))
    run.close()
    run = models.build_sir(n=4000, degree=10, seed=4)
    frm, to, _ = models.staged_edges(run.sim, "Contact")
    f2, t2 = om.gen_uniform_out(4000, 10, 4)
    np.testing.assert_array_equal(frm, f2)
    np.testing.assert_array_equal(to, t2)
    run.close()


def test_prepared_apply_equals_apply(vh):
    """A prepared apply! (vg_apply_prepare, vg_apply_call_run) runs the same
    call as apply!: ten SIR steps either way from the same state end in the
    same state, and before finish_init! the prepared call is refused with the
    reference's message."""
    from vahana_gb300 import models
    r1 = models.build_sir(n=3000, degree=8, seed=4)
    r2 = models.build_sir(n=3000, degree=8, seed=4)
    with pytest.raises(AssertionError, match="finish_init"):
        r1.step()
    vh.finish_init(r1.sim)
    vh.finish_init(r2.sim)
    m = r2.model
    for _ in range(10):
        r1.step()
        vh.apply_(r2.sim, "sir", ["Person"], ["Person", "Contact"], ["Person"],
                  params=[m["Contact"].index, r2.beta, r2.recovery, r2.seed])
    a1 = vh.read_agents(r1.sim, "Person")[0]
    a2 = vh.read_agents(r2.sim, "Person")[0]
    np.testing.assert_array_equal(a1["state"], a2["state"])
    np.testing.assert_array_equal(a1["days"], a2["days"])
    assert int((a1["state"] != 0).sum()) > 3  # the epidemic moved
    r1.close()
    r2.close()


@pytest.mark.parametrize("W,H,nw,crowd", [(64, 48, 1500, 1000), (8, 8, 300, 0), (40, 40, 900, 800)])
def test_walker_rebuild_step_by_step(vh, W, H, nw, crowd):
    """The walker -> cell containers after every step equal the oracle's, in
    walker order per cell.  `crowd` walkers start on cell (1, 1), so the
    first rebuilds hold rows of more than 64 records that then spread out;
    with more walkers than cells (8 x 8) most rows hold several records."""
    from vahana_gb300 import models
    seed = 11
    a0, x0, y0 = models.life_initial_state(W, H, nw, 0.3, seed)
    x0[:crowd] = 1
    y0[:crowd] = 1
    m = models.life_model()
    sim = vh.create_simulation(m)
    vh.add_raster(sim, "raster", (W, H), "Cell", alive=a0)
    vh.connect_raster_neighbors(sim, "raster", "Neighbor", implicit=True)
    wids = vh.add_agents(sim, "Walker", nw, x=x0, y=y0)
    cells = (np.uint64(m["Cell"].index) << np.uint64(56)) | (
        (x0.astype(np.uint64) - 1) + (y0.astype(np.uint64) - 1) * np.uint64(W) + np.uint64(1))
    vh.add_edges(sim, "OnCell", wids, cells)
    vh.finish_init(sim)
    for step in range(1, 9):
        vh.apply_(sim, "life", ["Cell"], ["Cell", "Neighbor"], ["Cell"],
                  params=[m["Neighbor"].index])
        vh.apply_(sim, "random_walk", ["Walker"], ["Walker"], ["Walker", "OnCell"],
                  params=[m["OnCell"].index, 0, seed])
        a_ref, x_ref, y_ref, rp_ref, src_ref = om.run_life_walkers(a0, x0, y0, W, H, seed, step)
        w = vh.read_agents(sim, "Walker")[0]
        np.testing.assert_array_equal(w["x"], x_ref)
        np.testing.assert_array_equal(w["y"], y_ref)
        rp, frm, _ = vh.read_edges(sim, "OnCell", "Cell")
        np.testing.assert_array_equal(rp, rp_ref)
        np.testing.assert_array_equal(frm & np.uint64((1 << 36) - 1), src_ref)
        if step == 1 and crowd > 64:
            assert int(np.diff(rp_ref).max()) > 64
    sim.close()


def test_life_walkers_bit_exact(vh):
    from vahana_gb300 import models
    W, H, nw, seed = 96, 80, 700, 5
    run = models.build_life(W, H, nw, 0.3, seed)
    sim = run.sim
    a0 = vh.read_agents(sim, "Cell")[0]["alive"].copy()
    wc = vh.read_agents(sim, "Walker")[0]
    x0, y0 = wc["x"].copy(), wc["y"].copy()
    vh.finish_init(sim)
    steps = 15
    for _ in range(steps):
        run.step()
    a = vh.read_agents(sim, "Cell")[0]["alive"]
    w = vh.read_agents(sim, "Walker")[0]
    a_ref, x_ref, y_ref, rp_ref, src_ref = om.run_life_walkers(a0, x0, y0, W, H, seed, steps)
    np.testing.assert_array_equal(a.astype(np.uint8), a_ref)
    np.testing.assert_array_equal(w["x"], x_ref)
    np.testing.assert_array_equal(w["y"], y_ref)
    # walker -> cell edges rebuilt every step, in call (walker) order per cell
    rp, frm, _ = vh.read_edges(sim, "OnCell", "Cell")
    np.testing.assert_array_equal(rp, rp_ref)
    np.testing.assert_array_equal(frm & np.uint64((1 << 36) - 1), src_ref)
    run.close()
