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
