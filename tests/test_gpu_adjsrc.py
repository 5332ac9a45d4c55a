"""The adjoint source of a 2-D run on the GPU (ADJOINT_SOURCE_FILT,
driver.f90:1262-1686) against the numpy restatement in the oracle, FP64
<= 1e-10 relative L2; windows, measurement count and line-search reuse
identical."""
import numpy as np
import pytest

from adjsrc_cases import CASE, delayed, ridge_field
from cases import gaussian_plane, rel_l2, small_params_2d, table_for

pytestmark = pytest.mark.gpu


def _ctx():
    from sparc_gb300.solver import Solver
    p = small_params_2d(nx=CASE["nx"], nz=48, xlength=CASE["xlength"], ylength=CASE["xlength"],
                        outputcad=CASE["outputcad"])
    return p, Solver(p, table_for(p))


def test_adjoint_source_matches_oracle(gpu_lib):
    from oracle import adjoint_source as A
    c = CASE
    p, s = _ctx()
    t = np.arange(c["nt"]) * 0.5
    acc = ridge_field(c["nx"], c["nt"], c["xlength"], c["outputcad"], seed=5)
    dat = delayed(acc, 9.0, c["outputcad"])
    adj_g, mis_g, n_g, win_g = s.adjoint_source(dat, c["x00"], t[0], 0.5, c["ridges"], c["bands"], synth=acc)
    adj_o, mis_o, n_o, win_o, _ = A.adjoint_source_filt(acc, dat, c["xlength"], c["outputcad"], c["x00"], t,
                                                        c["ridges"], c["bands"])
    assert n_g == n_o and n_g > 20
    assert win_g == win_o
    assert abs(mis_g - mis_o) <= 1e-10 * mis_o
    assert rel_l2(adj_g, adj_o) < 1e-10, rel_l2(adj_g, adj_o)
    # line search: the windows of sets 0 and 1 are read back (windows.0/1)
    dat2 = delayed(acc, -6.0, c["outputcad"])
    adj_g2, mis_g2, _, _ = s.adjoint_source(dat2, c["x00"], t[0], 0.5, c["ridges"], c["bands"], windows=win_g,
                                            synth=acc)
    adj_o2, mis_o2, _, _, _ = A.adjoint_source_filt(acc, dat2, c["xlength"], c["outputcad"], c["x00"], t,
                                                    c["ridges"], c["bands"], windows_in=win_o)
    assert abs(mis_g2 - mis_o2) <= 1e-10 * mis_o2
    assert rel_l2(adj_g2, adj_o2) < 1e-10


def test_adjoint_source_from_device_records(gpu_lib):
    """The synthetic taken from the context's surface records on the device
    equals the same computation from the records read back to the host."""
    from sparc_gb300 import sources
    c = CASE
    p, s = _ctx()
    s.set_source_series(gaussian_plane(p, sigma_mm=1.0, x0_mm=c["x00"]), sources.ricker_series(p, 4000))
    s.record_surface(c["nt"])
    s.step(c["nt"] * p.steps)
    rec = s.records()[:, 0, :]
    assert rec.shape == (c["nt"], c["nx"]) and np.abs(rec).max() > 0
    dat = delayed(rec, 9.0, c["outputcad"])
    ridges = {0: (10.0, 30.0, 20.0), 1: (15.0, 40.0, 15.0)}
    got = s.adjoint_source(dat, c["x00"], 0.0, 0.5, ridges, c["bands"])
    ref = s.adjoint_source(dat, c["x00"], 0.0, 0.5, ridges, c["bands"], synth=rec)
    assert np.array_equal(got[0], ref[0]) and got[1] == ref[1] and got[2] == ref[2] and got[3] == ref[3]
    assert got[2] > 0


def test_adjoint_source_refuses_3d(gpu_lib):
    from cases import small_params
    from sparc_gb300.native import SparcError
    from sparc_gb300.solver import Solver
    p = small_params()
    s = Solver(p, table_for(p))
    with pytest.raises(SparcError):
        s.adjoint_source(np.zeros((20, p.nx)), 0.0, 0.0, 0.5, {0: (1, 2, 3)}, {}, synth=np.zeros((20, p.nx)))


def test_misfit_all_matches_oracle(gpu_lib):
    from oracle import adjoint_source as A
    c = CASE
    p, s = _ctx()
    t = np.arange(c["nt"]) * 0.5
    acc = ridge_field(c["nx"], c["nt"], c["xlength"], c["outputcad"], seed=7)
    dat = delayed(acc, -9.0, c["outputcad"])
    mg, ng, wg = s.misfit_all(dat, c["x00"], t[0], 0.5, c["ridges"], synth=acc)
    mo, no, wo = A.misfit_all(acc, dat, c["xlength"], c["outputcad"], c["x00"], t, c["ridges"])
    assert np.array_equal(ng, no) and wg == wo
    assert np.all(np.abs(mg - mo) <= 1e-10 * mo)
    # line search on the stored windows (windows.all.N)
    dat2 = delayed(acc, 15.0, c["outputcad"])
    mg2, ng2, _ = s.misfit_all(dat2, c["x00"], t[0], 0.5, c["ridges"], windows=wg, synth=acc)
    mo2, no2, _ = A.misfit_all(acc, dat2, c["xlength"], c["outputcad"], c["x00"], t, c["ridges"], windows_in=wo)
    assert np.array_equal(ng2, no2) and np.all(np.abs(mg2 - mo2) <= 1e-10 * mo2)
