"""Batched SIR ensemble: every instance bit-identical between the batched
arena (one launch per step, or a CUDA graph of the step loop) and the same
instance stepped alone with the plain kernels through apply!, and equal to
the oracle's CPU run of the instance."""
import numpy as np
import pytest

from oracle import models as om

pytestmark = pytest.mark.gpu


def small_params(n):
    from vahana_gb300 import models
    return models.batch_params(n, n_lo=500, n_hi=4000)


def test_batch_equals_plain_and_oracle(vh):
    from vahana_gb300 import models
    N, deg, beta, rec, seeds = small_params(24)
    b = models.Batch(N, deg, beta, rec, seeds)
    # 10 steps as a CUDA graph, 10 more replaying it, 7 plain launches, 3 graph
    b.step(10, mode=1)
    b.step(10, mode=1)
    b.step(7, mode=0)
    b.step(3, mode=1)
    for i in range(b.n):
        b.step_one(i, 30)
    for i in range(b.n):
        sb, db = b.states(i, which=0)
        sp, dp = b.states(i, which=1)
        np.testing.assert_array_equal(sb, sp)
        np.testing.assert_array_equal(db, dp)
    for i in (0, 5, 17):  # the CPU oracle from its own generator and initial state
        n_i = int(N[i])
        frm, to = om.gen_uniform_out(n_i, int(deg[i]), int(seeds[i]))
        st0, d0 = models.sir_initial_state(n_i, int(seeds[i]),
                                           max(1, int(round(n_i / 1000))))
        s_ref, d_ref = om.run_sir(n_i, frm, to, st0, d0, float(beta[i]), int(rec[i]),
                                  int(seeds[i]), 30, first_step=1)
        sb, db = b.states(i, which=0)
        np.testing.assert_array_equal(sb, s_ref)
        np.testing.assert_array_equal(db, d_ref)
    info = b.info()
    assert info["agents"] == int(N.sum()) and info["tpb"] in (128, 256, 512)
    b.close()


def test_batch_persistent_equals_plain(vh):
    """The persistent launch (all steps in one cooperative launch, a block
    ticket of step t waiting for its instances' step t - 1), with and without
    the warp-per-agent bucket for agents above 8 in-edges, interleaved with
    the other forms,
    with 1, 2 and 4 agents per lane in both forms: every instance
    bit-identical to its plain apply! run."""
    from vahana_gb300 import models
    N, deg, beta, rec, seeds = small_params(20)
    b = models.Batch(N, deg, beta, rec, seeds)
    t = b.tuning()
    assert t["persistent_tpb"] in (256, 512)
    total = 0
    for mode, steps, forced, lanes in ((2, 6, None, (1, 1)), (2, 5, None, (2, 4)),
                                       (1, 4, None, (4, 2)), (3, 7, (1, 256, 8), (1, 1)),
                                       (2, 3, (1, 512, 8), (2, 4)), (0, 2, None, (4, 2)),
                                       (3, 5, (0, 256, 8), (2, 2)), (2, 4, (1, 256, 8), (4, 4))):
        if forced:
            b.set_launch(*forced)
        b.set_lanes(*lanes)
        assert b.lanes() == {"per_step": lanes[0], "persistent": lanes[1]}
        b.step(steps, mode=mode)
        total += steps
    assert b.tuning()["heavy_agents"] > 0  # threshold 8: the bucket path ran
    for i in range(b.n):
        b.step_one(i, total)
    for i in range(b.n):
        sb, db = b.states(i, which=0)
        sp, dp = b.states(i, which=1)
        np.testing.assert_array_equal(sb, sp)
        np.testing.assert_array_equal(db, dp)
    b.close()


def test_batch_cluster_equals_plain(vh):
    """The persistent cluster launch (clusters take packs of instances from
    a counter, masks in distributed shared memory, a cluster barrier between
    steps) in several shapes, interleaved with the other forms: every
    instance bit-identical to its plain apply! run."""
    from vahana_gb300 import models
    N, deg, beta, rec, seeds = small_params(24)
    b = models.Batch(N, deg, beta, rec, seeds)
    assert b.tuning()["form"] in models.Batch.FORMS
    total = 0
    for shape, mode, steps in (((8, 512, 1), 4, 7), ((4, 256, 2), 4, 6), ((1, 128, 1), 4, 3),
                               ((2, 256, 2), 1, 2), ((2, 256, 2), 4, 5), ((8, 128, 2), 2, 3),
                               ((8, 128, 2), 4, 4)):
        b.set_cluster(*shape)
        c = b.cluster()
        assert (c["ctas"], c["tpb"], c["ilp"]) == shape and c["clusters"] >= 1
        b.step(steps, mode=mode)
        total += steps
    b.set_launch(2)
    b.step(5, mode=3)
    total += 5
    for i in range(b.n):
        b.step_one(i, total)
    for i in range(b.n):
        sb, db = b.states(i, which=0)
        sp, dp = b.states(i, which=1)
        np.testing.assert_array_equal(sb, sp)
        np.testing.assert_array_equal(db, dp)
    b.close()


def test_batch_tiny_instances_every_form(vh):
    """Three hundred instances of 2..39 agents (one infected each, beta 0.2..0.9):
    a block ticket of the persistent launch spans many instances, a cluster
    pack holds dozens, and mask words straddle instance boundaries.  Every
    form, with every lane count, bit-identical to the plain path."""
    from vahana_gb300 import models
    N, deg, beta, rec, seeds = models.batch_params(300, n_lo=2, n_hi=40, deg_lo=1, deg_hi=8,
                                                   beta_lo=0.2, beta_hi=0.9, rec_lo=2, rec_hi=4)
    b = models.Batch(N, deg, beta, rec, seeds)
    total = 0
    for mode, lanes, forced in ((2, (1, 1), (1, 256, 0xFFFFFFFF)), (1, (2, 2), None),
                                (4, (4, 4), None), (2, (1, 4), (1, 512, 2)),
                                (0, (4, 2), None), (2, (2, 2), (1, 128, 0xFFFFFFFF))):
        if forced:
            b.set_launch(*forced)
        b.set_lanes(*lanes)
        b.step(5, mode=mode)
        total += 5
    for i in range(b.n):
        b.step_one(i, total)
    moved = 0
    for i in range(b.n):
        sb, db = b.states(i, which=0)
        sp, dp = b.states(i, which=1)
        np.testing.assert_array_equal(sb, sp)
        np.testing.assert_array_equal(db, dp)
        moved += int((sb == 2).sum())
    assert moved > 300  # the epidemics ran
    b.close()


def test_step_barrier_wait_gives_up_with_a_status(vh):
    """The persistent launch's step waits are bounded: two blocks waiting
    for an instance counter that nothing advances record 0x5e04 and end;
    the GPU stays usable (a batch steps correctly afterwards)."""
    import ctypes as C
    from vahana_gb300 import models
    from vahana_gb300._lib import check, lib
    st, ms = C.c_int(), C.c_double()
    check(lib().vg_selftest_barrier_timeout(C.byref(st), C.byref(ms)))
    assert st.value == 0x5e04 and ms.value < 5000
    N, deg, beta, rec, seeds = small_params(4)
    b = models.Batch(N, deg, beta, rec, seeds)
    b.set_launch(1, 256, 0xFFFFFFFF)
    b.step(3, mode=2)
    for i in range(b.n):
        b.step_one(i, 3)
        np.testing.assert_array_equal(b.states(i, 0)[0], b.states(i, 1)[0])
    b.close()
