"""The ensemble and serving workloads' inputs, on the CPU: the 512-instance
SIR ensemble's parameters (Philox(seed = instance index)) and the serving
stream's jobs stay within the stated ranges, are deterministic in their
seed and have the stated mixes."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_ensemble_parameters_in_range(vh):
    from vahana_gb300 import models
    N, deg, beta, rec, seeds = models.batch_params(512)
    assert N.min() >= 1_000 and N.max() <= 100_000
    assert deg.min() >= 5 and deg.max() <= 30
    assert beta.min() >= 0.01 and beta.max() <= 0.1
    assert rec.min() >= 5 and rec.max() <= 10
    assert np.array_equal(seeds, np.arange(512, dtype=np.uint64))
    # log-uniform N: log10(N) spreads over [3, 5) with mean near 4; the sum
    # is near 512 x E[N] = 512 x 99000 / ln(100) = 1.1e7
    assert abs(np.log10(N).mean() - 4.0) < 0.1
    assert 0.9e7 < N.sum() < 1.3e7
    # every degree and recovery value occurs
    assert set(deg.tolist()) == set(range(5, 31))
    assert set(rec.tolist()) == set(range(5, 11))
    again = models.batch_params(512)
    for a, b in zip((N, deg, beta, rec, seeds), again):
        assert np.array_equal(a, b)
    # the first instances of a larger ensemble are the same instances
    first = models.batch_params(8)
    assert np.array_equal(first[0], N[:8]) and np.array_equal(first[2], beta[:8])


def test_serving_stream_jobs(vh):
    import bench
    from vahana_gb300 import serve
    specs = bench.serve_jobs(4096, 1)
    n = np.array([s.n for s in specs])
    steps = np.array([s.steps for s in specs])
    model = np.array([s.model for s in specs])
    deg = np.array([s.mean_degree for s in specs])
    assert n.min() >= 1_000 and n.max() <= 1_000_000
    assert steps.min() >= 50 and steps.max() <= 500
    assert deg.min() >= 5 and deg.max() <= 30
    assert abs((model == serve.SIR).mean() - 0.5) < 0.03
    assert abs(np.log10(n).mean() - 4.5) < 0.05
    sir = [s for s in specs if s.model == serve.SIR]
    op = [s for s in specs if s.model == serve.OPINION]
    assert all(0.01 <= s.beta <= 0.1 and 5 <= s.recovery <= 10 for s in sir)
    assert all(s.eps == 0.3 and s.wmax == min(1e4, s.n / 10) for s in op)
    # each job's seed is its index + 1; the stream repeats for its seed
    assert [s.seed for s in specs] == list(range(1, 4097))
    again = bench.serve_jobs(4096, 1)
    assert all((a.model, a.n, a.steps, a.mean_degree, a.beta, a.recovery) ==
               (b.model, b.n, b.steps, b.mean_degree, b.beta, b.recovery)
               for a, b in zip(specs, again))
    other = bench.serve_jobs(64, 2)
    assert any(a.n != b.n for a, b in zip(specs[:64], other))
