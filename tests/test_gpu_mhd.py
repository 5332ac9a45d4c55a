"""Option 10 (MP_MHD_PML_3D_DISPL) on a flux-tube background: the CUDA path
(physical-space state, 21 derivatives per stage) against the FP64 oracle and
the committed fixture.  Tolerance: FP64 <= 1e-10 relative L2 per field."""
import os
import sys

import numpy as np
import pytest

from cases import gaussian_plane, rel_l2, table_for

pytestmark = pytest.mark.gpu
TOL64 = 1e-10


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def _case(prec="f64", **kw):
    sys.path.insert(0, os.path.dirname(__file__))
    from golden.make_golden import golden_mhd_background, golden_params_mhd
    p = golden_params_mhd().replace(precision=prec, **kw)
    return p, table_for(p), golden_mhd_background(p)


def _state(p, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((6, p.nz, p.ny, p.nx)) * 1e-6
    pml = rng.standard_normal((6, p.nzpml, p.ny, p.nx)) * 1e-8
    return a, pml


@pytest.mark.parametrize("nsteps,mode", [(1, 1), (5, 1), (5, 2)])
def test_mhd_matches_oracle(gpu_lib, oracle_mod, nsteps, mode):
    from sparc_gb300.solver import Solver
    p, tab, bg = _case()
    g, o = Solver(p, tab), oracle_mod.Oracle(p, tab)
    g.set_mhd_background(*bg)
    o.set_mhd(*bg)
    a0, pml0 = _state(p, 31)
    g.set_state(a0, pml0)
    o.set_state(a0, pml0)
    if mode == 1:
        plane = gaussian_plane(p)
        series = oracle_mod.forward_source(p, 200) * 1e3
        g.set_source_series(plane, series)
        o.set_source(1, plane[None].copy(), series)
    else:
        planes = np.random.default_rng(6).standard_normal((12, p.ny, p.nx)) * 1e-4
        g.set_source_lagrange(planes)
        o.set_source(2, planes, None)
    g.step(nsteps)
    o.step(nsteps)
    ag, pg = g.state()
    ao, _, po = o.state()
    for f in range(6):
        assert rel_l2(ag[f], ao[f]) < TOL64, (f, rel_l2(ag[f], ao[f]))
    for f in range(6):
        assert rel_l2(pg[f], po[f]) < TOL64, ("pml", f, rel_l2(pg[f], po[f]))


def test_mhd_matches_committed_fixture(gpu_lib):
    from sparc_gb300.solver import Solver
    from golden.make_golden import golden_inputs
    p, tab, bg = _case()
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))
    s = Solver(p, tab)
    s.set_mhd_background(*bg)
    a, pml, plane, series = golden_inputs(p, 48)
    s.set_state(a * 1e-3, pml)
    s.set_source_series(plane, series)
    s.step(5)
    st, pm = s.state()
    for f in range(6):
        assert rel_l2(st[f], g["step5_mhd_a"][f]) < TOL64, f
    assert rel_l2(pm, g["step5_mhd_pml"]) < TOL64


def test_mhd_fp32_and_records(gpu_lib, oracle_mod):
    """FP32 against FP64 on the same inputs, and the surface records (v_z on
    the observation plane of each pixel, the plane of a(:,:,orad_2d,6))."""
    from sparc_gb300.solver import Solver
    out = []
    for prec in ("f64", "f32"):
        p, tab, bg = _case(prec)
        s = Solver(p, tab)
        s.set_mhd_background(*bg)
        a0, pml0 = _state(p, 32)
        s.set_state(a0, pml0)
        s.set_source_series(gaussian_plane(p), oracle_mod.forward_source(p, 200) * 1e3)
        s.record_surface(3)
        s.step(16)
        out.append((s.state()[0], s.records(), s.info()["o_rad"]))
    (a64, r64, orad), (a32, r32, _) = out
    for f in range(6):
        assert rel_l2(a32[f], a64[f]) < 1e-4, (f, rel_l2(a32[f], a64[f]))
    assert r64.shape[0] == 2
    assert rel_l2(r32, r64) < 1e-4
    assert np.abs(r64[1]).max() > 0
    assert rel_l2(r64[1], a64[5, int(orad) - 1]) < 1e-15     # record 1 = v_z after the step at time 15
