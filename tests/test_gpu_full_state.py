"""Checkpoint and resume through the reference's full-state files
(WRITE_OUT_FULL_STATE / READ_IN_INITIAL_CONDITION, all_modules.f90:530-694):
a run resumed from the files continues as the original one."""
import numpy as np
import pytest

from cases import rel_l2, small_params, table_for

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_resume_from_full_state_files(gpu_lib, tmp_path, prec):
    from sparc_gb300 import io, sources
    from sparc_gb300.solver import Solver
    p = small_params(precision=prec)
    tab = table_for(p)
    se = sources.ricker_series(p, 200, delay=20.0)
    pl = sources.gaussian_plane(p, 2.0)
    with Solver(p, tab) as s:
        s.set_source_series(pl, se)
        s.step(40)
        io.write_full_state(str(tmp_path), s, s.time)
        t0 = s.time
        s.step(20)
        ref = s.state()[0]
        with Solver(p, tab) as r:
            r.set_source_series(pl, se)
            io.read_full_state(str(tmp_path), r, t0)
            r.time = t0
            r.step(20)
            got = r.state()[0]
    assert np.abs(ref).max() > 0
    tol = 1e-12 if prec == "f64" else 1e-5
    assert rel_l2(got, ref) < tol, rel_l2(got, ref)
