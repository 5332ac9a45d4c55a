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


# ---- option 18: MP_MHD_PML_2D_DISPL (physics2d.f90:724-943) on a flux sheet ----

def _case2d(prec="f64", **kw):
    sys.path.insert(0, os.path.dirname(__file__))
    from golden.make_golden import golden_mhd2d_background, golden_params_mhd2d
    p = golden_params_mhd2d().replace(precision=prec, **kw)
    return p, table_for(p), golden_mhd2d_background(p)


def _state2d(p, seed):
    """A state the reference can reach: no y components, psi_p zero on the
    bottom plane (ddz's bc 2 reads it as the caller-set value, which the
    reference leaves at 0), the 3-D-only auxiliaries zero."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((6, p.nz, 1, p.nx)) * 1e-6
    a[1] = 0.0
    a[4] = 0.0
    pml = rng.standard_normal((6, p.nzpml, 1, p.nx)) * 1e-8
    pml[1, 0] = 0.0
    pml[3] = 0.0
    pml[5] = 0.0
    return a, pml


@pytest.mark.parametrize("nsteps,mode,adjoint", [(1, 1, False), (31, 1, False), (31, 2, True)])
def test_mhd2d_matches_oracle(gpu_lib, oracle_mod, nsteps, mode, adjoint):
    from sparc_gb300.solver import Solver
    p, tab, bg = _case2d(compute_adjoint=adjoint, compute_forward=not adjoint)
    g, o = Solver(p, tab), oracle_mod.Oracle(p, tab)
    g.set_mhd2d_background(*bg)
    o.set_mhd2d(*bg)
    a0, pml0 = _state2d(p, 33)
    g.set_state(a0, pml0)
    o.set_state(a0, pml0)
    if mode == 1:
        plane = gaussian_plane(p, sigma_mm=8.0)
        series = oracle_mod.forward_source(p, 200) * 1e3
        g.set_source_series(plane, series)
        o.set_source(1, plane[None].copy(), series)
    else:
        planes = np.random.default_rng(7).standard_normal((12, 1, p.nx)) * 1e-4
        g.set_source_lagrange(planes)
        o.set_source(2, planes, None)
    g.step(nsteps)
    o.step(nsteps)
    ag, pg = g.state()
    ao, _, po = o.state()
    for f in (0, 2, 3, 5):
        assert rel_l2(ag[f], ao[f]) < TOL64, (f, rel_l2(ag[f], ao[f]))
    assert np.abs(ag[1]).max() == 0 and np.abs(ag[4]).max() == 0
    for f in (0, 1, 2, 4):
        assert rel_l2(pg[f], po[f]) < TOL64, ("pml", f, rel_l2(pg[f], po[f]))
    assert np.abs(pg[3]).max() == 0 and np.abs(pg[5]).max() == 0


def test_mhd2d_matches_committed_fixture(gpu_lib):
    from sparc_gb300.solver import Solver
    from golden.make_golden import golden_inputs
    p, tab, bg = _case2d()
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))
    s = Solver(p, tab)
    s.set_mhd2d_background(*bg)
    a, pml, plane, series = golden_inputs(p, 49)
    s.set_state(a * 1e-3, pml)
    s.set_source_series(plane, series)
    s.step(31)
    st, pm = s.state()
    for f in (0, 2, 3, 5):
        assert rel_l2(st[f], g["step31_mhd2d_a"][f]) < TOL64, f
    assert rel_l2(pm, g["step31_mhd2d_pml"]) < TOL64


def test_mhd2d_fp32_and_records(gpu_lib, oracle_mod):
    from sparc_gb300.solver import Solver
    out = []
    for prec in ("f64", "f32"):
        p, tab, bg = _case2d(prec)
        s = Solver(p, tab)
        s.set_mhd2d_background(*bg)
        a0, pml0 = _state2d(p, 34)
        s.set_state(a0, pml0)
        s.set_source_series(gaussian_plane(p, sigma_mm=8.0), oracle_mod.forward_source(p, 200) * 1e3)
        s.record_surface(4)
        s.step(31)
        out.append((s.state()[0], s.records(), s.info()["o_rad"]))
    (a64, r64, orad), (a32, r32, _) = out
    for f in (0, 2, 3, 5):
        assert rel_l2(a32[f], a64[f]) < 1e-4, (f, rel_l2(a32[f], a64[f]))
    assert r64.shape[0] == 3                                    # times 0, 15, 30
    assert rel_l2(r32, r64) < 1e-4
    assert rel_l2(r64[2], a64[5, int(orad) - 1]) < 1e-15     # record 2 = v_z after the step at time 30


def test_mhd2d_needs_its_background(gpu_lib):
    from sparc_gb300.native import SparcError
    from sparc_gb300.solver import Solver
    p, tab, bg = _case2d()
    s = Solver(p, tab)
    with pytest.raises(SparcError):
        s.step(1)
    with pytest.raises(SparcError):
        s.set_mhd_background(*bg[:3], bg[3], bg[3], bg[3])      # the 3-D call belongs to option 10


# ---- option 8: MP_MHD_PML_3D (pml.f90:80-208), the MHD velocity form ----------

def _case8(prec="f64", **kw):
    sys.path.insert(0, os.path.dirname(__file__))
    from golden.make_golden import golden_mhd_background, golden_params_mhd8
    p = golden_params_mhd8().replace(precision=prec, **kw)
    return p, table_for(p), golden_mhd_background(p)


def _state8(p, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros((8, p.nz, p.ny, p.nx))
    a[1:4] = rng.standard_normal((3, p.nz, p.ny, p.nx)) * 1e-6
    a[5:] = rng.standard_normal((3, p.nz, p.ny, p.nx)) * 1e-9
    pml = rng.standard_normal((6, p.nzpml, p.ny, p.nx)) * 1e-8
    return a, pml


@pytest.mark.parametrize("nsteps,mode", [(1, 1), (31, 1), (31, 2)])
def test_mhd8_matches_oracle(gpu_lib, oracle_mod, nsteps, mode):
    from sparc_gb300.solver import Solver
    p, tab, bg = _case8()
    g, o = Solver(p, tab), oracle_mod.Oracle(p, tab)
    g.set_mhd_background(*bg)
    o.set_mhd(*bg)
    a0, pml0 = _state8(p, 35)
    g.set_state(a0, pml0)
    o.set_state(a0, pml0)
    if mode == 1:
        plane = gaussian_plane(p)
        series = oracle_mod.forward_source(p, 200) * 1e3
        g.set_source_series(plane, series)
        o.set_source(1, plane[None].copy(), series)
    else:
        planes = np.random.default_rng(8).standard_normal((12, p.ny, p.nx)) * 1e-4
        g.set_source_lagrange(planes)
        o.set_source(2, planes, None)
    g.step(nsteps)
    o.step(nsteps)
    ag, pg = g.state()
    ao, _, po = o.state()
    assert ag.shape[0] == 8
    for f in range(8):
        assert rel_l2(ag[f], ao[f]) < TOL64, (f, rel_l2(ag[f], ao[f]))
    for f in range(6):
        assert rel_l2(pg[f], po[f]) < TOL64, ("pml", f, rel_l2(pg[f], po[f]))


def test_mhd8_matches_committed_fixture(gpu_lib):
    from sparc_gb300.solver import Solver
    from golden.make_golden import golden_inputs
    p, tab, bg = _case8()
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))
    s = Solver(p, tab)
    s.set_mhd_background(*bg)
    a, pml, plane, series = golden_inputs(p, 50)
    s.set_state(a * 1e-3, pml)
    s.set_source_series(plane, series)
    s.step(31)
    st, pm = s.state()
    for f in range(8):
        assert rel_l2(st[f], g["step31_mhd8_a"][f]) < TOL64, f
    assert rel_l2(pm, g["step31_mhd8_pml"]) < TOL64


def test_mhd8_fp32_and_records(gpu_lib, oracle_mod):
    """FP32 against FP64, and the surface records: v_z (field 4 of the
    velocity form) on the observation plane."""
    from sparc_gb300.solver import Solver
    out = []
    for prec in ("f64", "f32"):
        p, tab, bg = _case8(prec)
        s = Solver(p, tab)
        s.set_mhd_background(*bg)
        a0, pml0 = _state8(p, 36)
        s.set_state(a0, pml0)
        s.set_source_series(gaussian_plane(p), oracle_mod.forward_source(p, 200) * 1e3)
        s.record_surface(3)
        s.step(16)
        out.append((s.state()[0], s.records(), s.info()["o_rad"]))
    (a64, r64, orad), (a32, r32, _) = out
    for f in range(8):
        assert rel_l2(a32[f], a64[f]) < 1e-4, (f, rel_l2(a32[f], a64[f]))
    assert r64.shape[0] == 2
    assert rel_l2(r32, r64) < 1e-4
    assert rel_l2(r64[1], a64[3, int(orad) - 1]) < 1e-15


def test_mhd8_state_shape_and_fields(gpu_lib):
    from sparc_gb300.native import SparcError
    from sparc_gb300.solver import Solver
    p, tab, bg = _case8()
    s = Solver(p, tab)
    with pytest.raises(SparcError):
        s.step(1)                                       # no magnetic background yet
    s.set_mhd_background(*bg)
    a0, pml0 = _state8(p, 37)
    s.set_state(a0, pml0)
    assert np.array_equal(s.field(7), a0[7])           # b_z, the eighth field
    with pytest.raises(ValueError):
        s.set_state(a0[:6], pml0)
    with pytest.raises(SparcError):
        s.field(16)


# ---- the register-FFT derivative kernels (horizontal sizes 64 and 256) ------

@pytest.mark.parametrize("option,nx,ny,nz,nsteps", [(10, 64, 64, 32, 5), (8, 64, 64, 32, 3),
                                                     (10, 256, 256, 24, 1), (18, 64, 1, 32, 31),
                                                     (18, 256, 1, 32, 5)])
def test_mhd_register_fft_derivatives(gpu_lib, oracle_mod, option, nx, ny, nz, nsteps):
    """The x and y derivatives of the physical-space path at nx, ny = 64 and
    256 (R x R two-pass register DFTs) against the oracle's FFTs, through
    whole steps of each MHD form, FP64 <= 1e-10."""
    from cases import small_params, small_params_2d
    from sparc_gb300.background import flux_sheet_background, flux_tube_background
    from sparc_gb300.solver import Solver
    if option == 18:
        p = small_params_2d(nx=nx, nz=nz, npmlbot=4, npmltop=4, option=18)
    else:
        p = small_params(nx=nx, ny=ny, nz=nz, npmlbot=4, npmltop=4 if option == 8 else 0, option=option,
                         xlength=200e8, ylength=200e8)
    tab = table_for(p)
    g, o = Solver(p, tab), oracle_mod.Oracle(p, tab)
    if option == 18:
        bg = flux_sheet_background(p, tab)
        g.set_mhd2d_background(*bg)
        o.set_mhd2d(*bg)
        a0, pml0 = _state2d(p, 41)
    else:
        bg = flux_tube_background(p, tab, b_surf=800.0, r_surf_mm=8.0)
        g.set_mhd_background(*bg)
        o.set_mhd(*bg)
        a0, pml0 = (_state8 if option == 8 else _state)(p, 41)
    g.set_state(a0, pml0)
    o.set_state(a0, pml0)
    plane = gaussian_plane(p, sigma_mm=8.0)
    series = oracle_mod.forward_source(p, 200) * 1e3
    g.set_source_series(plane, series)
    o.set_source(1, plane[None].copy(), series)
    g.step(nsteps)
    o.step(nsteps)
    ag, pg = g.state()
    ao, _, po = o.state()
    for f in range(ag.shape[0]):
        if np.abs(ao[f]).max() == 0:
            assert np.abs(ag[f]).max() == 0, f
            continue
        assert rel_l2(ag[f], ao[f]) < TOL64, (f, rel_l2(ag[f], ao[f]))
    for f in range(6):
        if np.abs(po[f]).max() > 0:
            assert rel_l2(pg[f], po[f]) < TOL64, ("pml", f, rel_l2(pg[f], po[f]))


# ---- sensitivity kernels of option 18 (kernels.f90:197-453) --------------------

def _kernel_pair(prec):
    from sparc_gb300.solver import Solver
    p, tab, bg = _case2d(prec)
    pa = p.replace(compute_forward=False, compute_adjoint=True)
    fwd, adj = Solver(p, tab), Solver(pa, tab)
    for s in (fwd, adj):
        s.set_mhd2d_background(*bg)
    a1, pml1 = _state2d(p, 51)
    a2, pml2 = _state2d(p, 52)
    fwd.set_state(a1 * 1e3, pml1)
    adj.set_state(a2 * 1e3, pml2)
    return p, tab, bg, fwd, adj


@pytest.mark.parametrize("nsnap", [1, 2])
def test_mhd2d_kernels_match_oracle(gpu_lib, oracle_mod, nsnap):
    """K_c, K_rho, hessian on the 2-D MHD background (rho0, c^2 varying in x)
    and the B-field kernels (kernel_bx, kernel_bz, kernel_vectorpsi) against
    the oracle on the GPU's own snapshot fields, FP64 <= 1e-10."""
    p, tab, bg, fwd, adj = _kernel_pair("f64")
    o = oracle_mod.Oracle(p, tab)
    o.set_mhd2d(*bg)
    o.kernel_reset()
    adj.kernel_reset()
    graw = tab[:, 4] * o.info()["rsun"] / 1e12
    for k in range(nsnap):
        fwd.step(2)
        adj.step(2)
        fwd.snapshot(k, nsnap)
        adj.kernel_accumulate(fwd, k)
        af, _ = fwd.state()
        acc = np.stack([fwd.field(9), fwd.field(10), fwd.field(11)])
        aa, _ = adj.state()
        o.kernel_accumulate(np.concatenate([af[0:3], acc]), aa[3:6], graw)
        o.kernel_accumulate_b(af[0:3], aa[3:6])
    steps = int(fwd.info()["steps"])
    ref = o.kernel_finish(steps)
    refb = o.kernel_finish_b(steps)
    kc, kr, hs = adj.kernels()
    kbx, kbz, kpsi = adj.kernels_b()
    assert rel_l2(hs, ref[2]) < 1e-12
    assert rel_l2(kc, ref[0]) < TOL64, rel_l2(kc, ref[0])
    assert rel_l2(kr, ref[1]) < TOL64, rel_l2(kr, ref[1])
    for got, want, name in ((kbx, refb[0], "bx"), (kbz, refb[1], "bz"), (kpsi, refb[2], "psi")):
        assert np.abs(want).max() > 0, name
        assert rel_l2(got, want) < TOL64, (name, rel_l2(got, want))


def test_mhd2d_kernels_fp32(gpu_lib):
    """The FP32 path (FP32 fields, FP64 sums) against FP64 on the same inputs."""
    out = []
    for prec in ("f64", "f32"):
        p, tab, bg, fwd, adj = _kernel_pair(prec)
        adj.kernel_reset()
        for k in range(2):
            fwd.step(3)
            adj.step(3)
            fwd.snapshot(k, 2)
            adj.kernel_accumulate(fwd, k)
        out.append(adj.kernels() + adj.kernels_b())
    for q, name in enumerate(("kc", "krho", "hessian", "bx", "bz", "psi")):
        assert rel_l2(out[1][q], out[0][q]) < 1e-3, (name, rel_l2(out[1][q], out[0][q]))


def test_mhd3d_kernels_are_refused(gpu_lib):
    from sparc_gb300.native import SparcError
    from sparc_gb300.solver import Solver
    p, tab, bg = _case()
    s = Solver(p, tab)
    s.set_mhd_background(*bg)
    with pytest.raises(SparcError):
        s.snapshot(0, 1)


@pytest.mark.parametrize("option", [10, 18])
def test_mhd_fp32_paired_z_solve(gpu_lib, oracle_mod, option, monkeypatch):
    """The FP32 chunked z solve with two pencils per lane (paired FP32
    instructions) against the one-pencil kernel, through 16 steps of the MHD
    forms: the same elimination, so the states agree to FP32 rounding."""
    from sparc_gb300.solver import Solver
    out = []
    for scalar in (False, True):
        if scalar:
            monkeypatch.setenv("SPARC_ZCHUNK_SCALAR", "1")
        else:
            monkeypatch.delenv("SPARC_ZCHUNK_SCALAR", raising=False)
        if option == 10:
            p, tab, bg = _case("f32")
            s = Solver(p, tab)
            s.set_mhd_background(*bg)
            a0, pml0 = _state(p, 32)
            s.set_state(a0, pml0)
        else:
            p, tab, bg = _case2d("f32")
            s = Solver(p, tab)
            s.set_mhd2d_background(*bg)
        s.set_source_series(gaussian_plane(p), oracle_mod.forward_source(p, 200) * 1e3)
        s.step(16)
        out.append(s.state()[0])
        s.close()
    assert np.abs(out[1]).max() > 0
    for f in range(out[0].shape[0]):
        assert rel_l2(out[0][f], out[1][f]) < 1e-5, (f, rel_l2(out[0][f], out[1][f]))
