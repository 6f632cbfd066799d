"""Serving loop: jobs stepped together in one launch per model per tick
finish in exactly the state they reach when each is built and stepped alone
through apply! (bit-identical, both models), whatever the admission budget."""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(600)]


def _alone(spec):
    from vahana_gb300 import models, serve
    if spec.model == serve.SIR:
        run = models.build_sir(n=spec.n, degree=int(spec.mean_degree), beta=spec.beta,
                               recovery=spec.recovery, seed=spec.seed)
        T = "Person"
    else:
        run = models.build_opinion(n=spec.n, mean_degree=spec.mean_degree, gamma=2.5,
                                   wmax=spec.wmax, eps=spec.eps, seed=spec.seed,
                                   hub_threshold=models.OPINION_HUB_THRESHOLD)
        T = "Opinion"
    import vahana_gb300 as vh
    vh.finish_init(run.sim)
    for _ in range(spec.steps):
        run.step()
    cols = vh.read_agents(run.sim, T)[0]
    run.close()
    return cols


def _specs():
    from vahana_gb300 import serve
    return [serve.sir_job(4000, degree=8, steps=30, seed=3, beta=0.08, keep_state=True),
            serve.opinion_job(6000, mean_degree=12, steps=7, seed=5, eps=0.25, wmax=800,
                              keep_state=True),
            serve.sir_job(2500, degree=12, steps=11, seed=9, beta=0.03, recovery=4,
                          keep_state=True),
            serve.opinion_job(3000, mean_degree=20, steps=15, seed=8, eps=0.4, wmax=300,
                              keep_state=True),
            serve.sir_job(1000, degree=5, steps=0, seed=2, keep_state=True)]


@pytest.mark.parametrize("budget", [1 << 34, 1])
def test_serving_matches_alone(vh, budget):
    """budget 16 GiB: all five jobs resident together; budget 1 byte: one
    job at a time (each admitted only into an empty server)."""
    from vahana_gb300 import serve
    specs = _specs()
    with serve.Server(budget_bytes=budget) as S:
        ids = [S.submit(s) for s in specs]
        S.drain()
        res = {r["id"]: r for r in S.poll()}
        assert sorted(res) == sorted(ids)
        st = S.stats()
        assert st["done"] == len(specs) and st["active"] == 0 and st["queued"] == 0
        assert st["sim_steps"] == sum(s.steps for s in specs)
        if budget == 1:
            assert st["ticks"] >= st["sim_steps"]
        else:  # jobs overlapped
            assert max(s.steps for s in specs) <= st["ticks"] < st["sim_steps"]
        for i, spec in zip(ids, specs):
            got = S.job_state(i, spec)
            ref = _alone(spec)
            if spec.model == serve.SIR:
                np.testing.assert_array_equal(got[0], ref["state"])
                np.testing.assert_array_equal(got[1], ref["days"])
            else:
                np.testing.assert_array_equal(got.view(np.uint64), ref["x"].view(np.uint64))
            r = res[i]
            assert r["admit_s"] >= r["arrival_s"] and r["finish_s"] >= r["admit_s"]


def test_serving_rejects_bad_jobs(vh):
    from vahana_gb300 import serve
    with serve.Server() as S:
        bad = serve.sir_job(1, steps=3)
        with pytest.raises(vh.VahanaError):
            S.submit(bad)
        spec = serve.sir_job(100, steps=2)
        spec.model = 7
        with pytest.raises(vh.VahanaError):
            S.submit(spec)


def test_failed_build_retires_only_that_job(vh):
    """A job whose build raises on the host after admission (failure
    injected after its simulation and agents exist) is retired with an error
    status; the jobs resident beside it finish bit-identical to their alone
    runs, and the server keeps accepting jobs."""
    import time
    from vahana_gb300 import serve
    specs = _specs()[:4]
    bad = serve.sir_job(3000, degree=6, steps=9, seed=4)
    bad.fail_build = 1
    with serve.Server(budget_bytes=1 << 34) as S:
        ids = [S.submit(specs[0]), S.submit(specs[1]), S.submit(bad), S.submit(specs[2]),
               S.submit(specs[3])]
        res = {}
        deadline = time.time() + 300
        while len(res) < len(ids) and time.time() < deadline:
            for r in S.poll():
                res[r["id"]] = r
            time.sleep(0.01)
        assert sorted(res) == sorted(ids)
        failed = res[ids[2]]
        assert failed["status"] != 0 and "injected" in failed["error"]
        good = [i for k, i in enumerate(ids) if k != 2]
        assert all(res[i]["status"] == 0 for i in good)
        for i, spec in zip(good, specs):
            got = S.job_state(i, spec)
            ref = _alone(spec)
            if spec.model == serve.SIR:
                np.testing.assert_array_equal(got[0], ref["state"])
                np.testing.assert_array_equal(got[1], ref["days"])
            else:
                np.testing.assert_array_equal(got.view(np.uint64), ref["x"].view(np.uint64))
        late = serve.sir_job(1500, degree=7, steps=5, seed=12, keep_state=True)
        j = S.submit(late)
        S.drain()
        r = {x["id"]: x for x in S.poll()}
        assert r[j]["status"] == 0
        got = S.job_state(j, late)
        np.testing.assert_array_equal(got[0], _alone(late)["state"])
        st = S.stats()
        assert st["done"] == len(ids) + 1 and st["bytes_in_use"] == 0
