"""Host logic of the continuous-batching engine, with a fake pool (no GPU):
admission by footprint, idle-pool eviction, no livelock, bounded pools."""
import numpy as np
import pytest

from sparc_gb300 import serving


class FakePool:
    created = 0

    def __init__(self, p, table, role, slots, max_records, background="quiet", tube_cache=None, priority=0):
        FakePool.created += 1
        self.role = role
        self.background = background
        self.p = p.replace(nsrc=slots)
        self.requests = [None] * slots
        self.clock = [0] * slots
        self.bytes = slots * (p.nx // 2 + 1) * p.ny * p.nz * 8 * 15
        self.closed = False

    free = serving.Pool.free
    busy = serving.Pool.busy

    def admit(self, req, planes=None):
        slot = self.free[0]
        self.requests[slot] = req
        self.clock[slot] = 0
        return slot

    def advance(self, n):
        for i, r in enumerate(self.requests):
            if r is not None:
                self.clock[i] += n
        return self.busy

    def collect(self):
        out = []
        for i, r in enumerate(self.requests):
            if r is not None and self.clock[i] >= r.nsteps:
                out.append((r, np.zeros((2, 1, 1))))
                self.requests[i] = None
        return out

    def close(self):
        self.closed = True


@pytest.fixture
def fake(monkeypatch):
    FakePool.created = 0
    monkeypatch.setattr(serving, "Pool", FakePool)
    monkeypatch.setattr(serving.Engine, "_adjoint_planes", lambda self, pl, req: None)
    monkeypatch.setattr(serving, "polytrope_table", lambda nz, **kw: None)
    return FakePool


def test_idle_pools_are_evicted_when_the_budget_blocks(fake):
    # a budget that holds one large pool or a few small ones, never both
    grids = [(128, 128, 150), (256, 256, 300), (512, 512, 300)]
    reqs = [serving.Request(i, grids[i % 3], ("fwd", "fwd+adj")[i % 2], 30 * (1 + i % 4), 0.0, 0.0, 0.01 * i)
            for i in range(24)]
    eng = serving.Engine("f32", hbm_budget=14e9,
                         slots={(128, 128, 150): 8, (256, 256, 300): 4, (512, 512, 300): 2},
                         max_steps=max(r.nsteps for r in reqs))
    done = eng.run(reqs, max_wall=30.0)
    assert sorted(r.rid for r in done) == list(range(24))
    assert all(r.finished >= r.arrival for r in done)
    assert fake.created > len(eng.pools)                     # some pools were released on the way


def test_pool_count_per_grid_is_bounded(fake):
    reqs = [serving.Request(i, (128, 128, 150), "fwd", 30, 0.0, 0.0, 0.0) for i in range(40)]
    eng = serving.Engine("f32", hbm_budget=1e12, slots={(128, 128, 150): 4}, max_steps=30)
    done = eng.run(reqs, max_wall=30.0)
    assert len(done) == 40 and len(eng.pools) <= eng.max_pools_per_key


def test_a_pool_above_the_budget_is_an_error(fake):
    reqs = [serving.Request(0, (512, 512, 300), "fwd", 30, 0.0, 0.0, 0.0)]
    eng = serving.Engine("f64", hbm_budget=1e9, slots={(512, 512, 300): 2}, max_steps=30)
    with pytest.raises(RuntimeError, match="above the HBM budget"):
        eng.run(reqs, max_wall=30.0)


def test_flux_tube_requests_get_their_own_pools(fake):
    """Requests on the flux tube and on the quiet Sun of the same grid never
    share a pool: the background belongs to the pool."""
    reqs = [serving.Request(i, (128, 128, 150), "fwd", 30, 0.0, 0.0, 0.0,
                            background=(serving.TUBE if i % 2 else serving.QUIET)) for i in range(8)]
    eng = serving.Engine("f32", hbm_budget=1e12, slots={(128, 128, 150): 8}, max_steps=30)
    done = eng.run(reqs, max_wall=30.0)
    assert len(done) == 8
    kinds = sorted(pl.background for pl in eng.pools)
    assert kinds == [serving.QUIET, serving.TUBE]
    for pl in eng.pools:
        assert pl.p.option == (10 if pl.background == serving.TUBE else 4)


def test_stream_mixes_backgrounds():
    reqs = serving.poisson_stream(200, seed=3, p_tube=0.25)
    n_tube = sum(r.background == serving.TUBE for r in reqs)
    assert 30 < n_tube < 70


def test_pool_priorities_follow_the_cost_of_a_step():
    """Cheaper configurations get more urgent streams: 128^2 quiet first,
    the 512^2 flux tube last (level 0)."""
    eng = serving.Engine("f32", hbm_budget=1e12,
                         slots={(128, 128, 150): 8, (256, 256, 300): 4, (512, 512, 300): 2}, max_steps=30)
    Q, T = serving.QUIET, serving.TUBE
    order = [((128, 128, 150), Q), ((256, 256, 300), Q), ((128, 128, 150), T), ((512, 512, 300), Q),
             ((256, 256, 300), T), ((512, 512, 300), T)]
    levels = [eng._priority(g, bg) for g, bg in order]
    assert levels == sorted(levels, reverse=True) and levels[-1] == 0 and len(set(levels)) == len(levels)


def test_warm_creates_pools_within_the_budget_without_eviction(fake):
    """Engine.warm: one pool per (grid, background, role), cheapest first,
    stopping at the HBM budget; the stream then runs on them."""
    slots = {(128, 128, 150): 8, (256, 256, 300): 4, (512, 512, 300): 2}
    eng = serving.Engine("f32", hbm_budget=1e12, slots=slots, max_steps=30)
    assert eng.warm() == 12 and fake.created == 12
    reqs = [serving.Request(i, (128, 128, 150), "fwd+adj", 30, 0.0, 0.0, 0.0) for i in range(4)]
    done = eng.run(reqs, max_wall=30.0)
    assert len(done) == 4 and fake.created == 12            # served by the warmed pools
    small = serving.Engine("f32", hbm_budget=14e9, slots=slots, max_steps=30)
    n = small.warm()
    assert 0 < n < 12 and sum(pl.bytes for pl in small.pools) <= 14e9
    assert all(not pl.closed for pl in small.pools)          # nothing released on the way
