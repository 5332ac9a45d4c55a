"""The bounded device wait of the fused FP32 step, made to run out on purpose.

With SPARC_TEST_FUSED_NO_TABLE_COPY set when the context is created, the fused
step issues no z-table bulk copy, so its mbarrier never completes and every
CTA's wait gives up after a short limit with nothing in flight.  The library
must report SPARC_ETIMEDOUT from the next sync, clear the flag (the sync after
that succeeds), and leave the state of the CTAs that gave up untouched."""
import os

import numpy as np
import pytest

from cases import random_state, small_params, table_for

pytestmark = pytest.mark.gpu


def test_fused_table_wait_times_out_and_recovers(gpu_lib):
    from sparc_gb300.native import SPARC_ETIMEDOUT, SparcError
    from sparc_gb300.solver import Solver
    p = small_params(precision="f32")
    os.environ["SPARC_TEST_FUSED_NO_TABLE_COPY"] = "1"
    try:
        s = Solver(p, table_for(p))
    finally:
        os.environ.pop("SPARC_TEST_FUSED_NO_TABLE_COPY", None)
    a0, pml0 = random_state(p)
    s.set_state(a0, pml0)
    s.sync()
    before, _ = s.state()
    s.step(1)
    with pytest.raises(SparcError) as e:
        s.sync()
    assert e.value.status == SPARC_ETIMEDOUT
    s.sync()                                   # the flag was cleared
    after, _ = s.state()
    assert np.array_equal(before, after)       # no CTA computed or stored
    s.close()


def test_fused_step_without_the_switch_does_not_time_out(gpu_lib):
    from sparc_gb300.solver import Solver
    p = small_params(precision="f32")
    s = Solver(p, table_for(p))
    a0, pml0 = random_state(p)
    s.set_state(a0, pml0)
    before, _ = s.state()
    s.step(1)
    s.sync()
    after, _ = s.state()
    assert not np.array_equal(before, after)
    s.close()
