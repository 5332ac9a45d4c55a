"""Serving: continuous batching with per-slot clocks.  A request's result is
the same alone and in a mix of concurrent requests of several grid sizes and
both backgrounds (quiet Sun, magnetohydrostatic flux tube) that join running
batches at different times."""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRIDS = {(32, 32, 48): 3, (64, 64, 64): 2}


def engine(precision):
    from sparc_gb300.serving import Engine
    return Engine(precision=precision, hbm_budget=8e9, slots=GRIDS, max_steps=300)


def mix():
    from sparc_gb300.serving import TUBE, Request
    return [
        Request(0, (32, 32, 48), "fwd+adj", 60, 3.0, -5.0, 0.00),
        Request(1, (64, 64, 64), "fwd", 90, -20.0, 10.0, 0.00),
        Request(2, (32, 32, 48), "fwd", 45, -8.0, 2.0, 0.01),
        Request(3, (32, 32, 48), "fwd+adj", 75, 12.0, 4.0, 0.02),
        Request(4, (64, 64, 64), "fwd+adj", 60, 5.0, 5.0, 0.05),
        Request(5, (32, 32, 48), "fwd", 30, 0.0, 0.0, 0.10),
        Request(6, (64, 64, 64), "fwd+adj", 45, 30.0, -10.0, 0.02, background=TUBE),
        Request(7, (64, 64, 64), "fwd", 60, -15.0, 25.0, 0.04, background=TUBE),
    ]


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_result_same_alone_and_in_mix(gpu_lib, precision):
    eng = engine(precision)
    done = {r.rid: r for r in eng.run(mix())}
    eng.close()
    assert sorted(done) == list(range(8))
    for rid in (0, 3, 4, 6):
        alone = copy.deepcopy([r for r in mix() if r.rid == rid][0])
        alone.arrival = 0.0
        e2 = engine(precision)
        (a,) = e2.run([alone])
        e2.close()
        m = done[rid]
        assert m.records.shape == a.records.shape == (m.nsteps // 15, m.grid[1], m.grid[0])
        assert np.abs(a.records).max() > 0
        np.testing.assert_array_equal(m.records, a.records)
        np.testing.assert_array_equal(m.adj_records, a.adj_records)
        assert np.isfinite(m.records).all() and np.isfinite(m.adj_records).all()


def test_latency_stats_and_stream(gpu_lib):
    from sparc_gb300.serving import latency_stats, poisson_stream
    reqs = poisson_stream(12, rate=20.0, seed=1, mix=[((32, 32, 48), 0.7), ((64, 64, 64), 0.3)],
                          compress=240.0)
    assert all(r.nsteps % 15 == 0 for r in reqs)
    eng = engine("f32")
    done = eng.run(reqs)
    eng.close()
    st = latency_stats(done)
    assert st["n"] == 12 and 0 < st["p50_s"] <= st["p95_s"] <= st["p99_s"]
    for r in done:
        assert r.finished >= r.admitted >= r.arrival - 1e-6
