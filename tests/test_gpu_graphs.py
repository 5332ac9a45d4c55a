"""Captured step sequences (CUDA graphs, replayed at any time from the device
clock) and the autotuner: both must leave results bit-for-bit unchanged."""
import os

import numpy as np
import pytest

from cases import gaussian_plane, random_state, small_params, table_for

pytestmark = pytest.mark.gpu


def _solver(p, tab, graphs: bool):
    from sparc_gb300.solver import Solver
    if not graphs:
        os.environ["SPARC_NO_GRAPHS"] = "1"
    try:
        return Solver(p, tab)
    finally:
        os.environ.pop("SPARC_NO_GRAPHS", None)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_graph_replay_equals_direct_launches(gpu_lib, prec):
    from sparc_gb300 import sources
    p = small_params(precision=prec, nsrc=2)
    tab = table_for(p)
    a0, pml0 = random_state(p)
    plane = gaussian_plane(p)
    series = sources.ricker_series(p, 400) * 1e3
    out = []
    for graphs in (True, False):
        s = _solver(p, tab, graphs)
        for slot in range(2):
            s.set_state(a0 * (slot + 1), pml0, slot=slot)
            s.set_source_series(plane, series, slot=slot)
        s.record_surface(8)
        for n in (7, 15, 15, 3, 15):          # replays of one graph at different times, and new counts
            s.step(n)
        s.slot_reset(1)                       # device-side clock change between replays
        s.step(15)
        out.append(([s.state(slot=k)[0] for k in range(2)], [s.records(slot=k) for k in range(2)], s.time))
    (sa, ra, ta), (sb, rb, tb) = out
    assert ta == tb == 70
    for k in range(2):
        assert np.array_equal(sa[k], sb[k]), k
        assert np.array_equal(ra[k], rb[k]), k


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_autotune_keeps_results(gpu_lib, prec):
    from sparc_gb300.solver import Solver
    p = small_params(precision=prec)
    tab = table_for(p)
    a0, pml0 = random_state(p)
    s1, s2 = Solver(p, tab), Solver(p, tab)
    for s in (s1, s2):
        s.set_state(a0, pml0)
    pick = s1.autotune(2)                      # 2 warm + 2 timed ordinary steps per candidate
    assert list(pick.values())[0] in (2, 4, 8, 32, 64, 128) and pick["ms_per_step"] > 0
    n_auto = s1.time
    assert n_auto == 12                        # three candidates
    s1.step(3)
    s2.step(n_auto + 3)
    assert s1.time == s2.time == n_auto + 3
    assert np.array_equal(s1.state()[0], s2.state()[0])


@pytest.mark.parametrize("nz", [48, 200])
def test_fused_cta_shapes_agree(gpu_lib, nz, monkeypatch):
    """The fused FP32 step with 2, 4 and 8 modes per CTA (one and two warps
    per pencil) gives bitwise the same state."""
    from sparc_gb300 import sources
    from sparc_gb300.solver import Solver
    p = small_params(precision="f32", nz=nz, nsrc=2)
    tab = table_for(p)
    out = {}
    for P in ("2", "4", "8"):
        monkeypatch.setenv("SPARC_FUSED_MODES", P)
        with Solver(p, tab) as s:
            s.set_source_series(sources.gaussian_plane(p, 2.0), sources.ricker_series(p, 80, delay=20.0), slot=0)
            s.set_source_series(sources.gaussian_plane(p, 2.0, 5.0), sources.ricker_series(p, 80, delay=30.0), slot=1)
            s.step(37)
            out[P] = [s.state(k) for k in range(2)]
    for P in ("2", "8"):
        for k in range(2):
            assert np.array_equal(out[P][k][0], out["4"][k][0]) and np.array_equal(out[P][k][1], out["4"][k][1])
    assert np.abs(out["4"][0][0]).max() > 0


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_rhs_output_off_keeps_the_state_and_guards_the_snapshot(gpu_lib, prec):
    """sparc_gpu_set_rhs_output(ctx, 0): the state after several step calls
    is bit for bit that of the default context; the forward snapshot, which
    reads scr, is refused with SPARC_ESTATE until the output is back on."""
    from sparc_gb300 import sources
    from sparc_gb300.native import SPARC_ESTATE, SparcError
    from sparc_gb300.solver import Solver
    p = small_params(precision=prec, nsrc=2)
    tab = table_for(p)
    a0, pml0 = random_state(p)
    plane = gaussian_plane(p)
    series = sources.ricker_series(p, 400) * 1e3
    out = []
    for on in (True, False):
        g = Solver(p, tab)
        g.set_rhs_output(on)
        for s in range(p.nsrc):
            g.set_state(a0 * (s + 1), pml0, slot=s)
            g.set_source_series(plane, series, slot=s)
        for n in (3, 1, 5):
            g.step(n)
        g.sync(check_finite=True)
        out.append([g.state(slot=s) for s in range(p.nsrc)])
        if not on:
            with pytest.raises(SparcError) as e:
                g.snapshot(0, 2)
            assert e.value.status == SPARC_ESTATE
            g.set_rhs_output(True)
            g.step(1)
            g.snapshot(0, 2)
            g.sync()
        g.close()
    for s in range(p.nsrc):
        assert np.array_equal(out[0][s][0], out[1][s][0])
        assert np.array_equal(out[0][s][1], out[1][s][1])


def test_stream_priority_and_query(gpu_lib):
    """sparc_gpu_set_stream_priority moves the context to new streams between
    steps without changing results; sparc_gpu_query reports the queued work
    finished once the context is synchronised."""
    from sparc_gb300 import sources
    from sparc_gb300.solver import Solver
    p = small_params(precision="f32", nsrc=2)
    tab = table_for(p)
    a0, pml0 = random_state(p)
    plane = gaussian_plane(p)
    series = sources.ricker_series(p, 400) * 1e3
    out = []
    for level in (0, 3):
        g = Solver(p, tab)
        for s in range(p.nsrc):
            g.set_state(a0, pml0, slot=s)
            g.set_source_series(plane, series, slot=s)
        g.step(4)
        if level:
            g.set_stream_priority(level)      # between steps: waits for the queued work
        g.step(5)
        g.sync()
        assert g.busy() is False
        out.append(g.state(slot=1))
        g.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
