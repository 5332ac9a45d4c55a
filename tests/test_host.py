"""Host-side logic (no GPU): parameters, background, sources, byte model."""
import numpy as np
import pytest

from sparc_gb300 import bytes_model, sources
from sparc_gb300.background import polytrope_table
from sparc_gb300.params import SparcParams, config_quiet_256, r4

PARAMS_I = """
integer nx, ny, nz
parameter (nx = 256, ny = 256, nz = 300)
real*8 xlength, ylength, timestep
parameter (xlength = 400.0 * 10**(8), ylength = xlength, timestep = 2.0)
real*8 cadforcing
parameter( cadforcing = 30.0)
logical, parameter :: DAMP_WAVES = .TRUE.
logical, parameter :: magnetic = .false.
logical, parameter :: FLOWS = .FALSE.
integer npmltop, npmlbot,nzpml
parameter(npmlbot = 10, npmltop = 0, nzpml = (npmlbot + npmltop))
real*8 solartime
parameter(solartime = 2.0)
real*8 obsheight
parameter (obsheight = 20000000.0)
real *8 outputcad
parameter (outputcad = 30.0)
real*8 excitdep
parameter( excitdep = - 50000000.0)
"""


def test_params_i_parsing_and_instruction():
    p = SparcParams.from_params_i(PARAMS_I)
    assert (p.nx, p.ny, p.nz) == (256, 256, 300)
    assert p.xlength == 4.0e10 and p.npmlbot == 10 and p.npmltop == 0
    assert p.excitdep == -5.0e7 and p.damp_waves
    q = p.instruction("adjoint\n3D\n")
    assert q.compute_adjoint and not q.compute_forward and q.option == 4
    q2 = SparcParams.from_params_i(PARAMS_I.replace("ny = 256", "ny = 1")).instruction("spectral\n2D\nT\n")
    assert q2.option == 17 and q2.ny == 1 and q2.compute_forward


def test_params_magnetic_selects_option_10():
    """PARSE_OPTIONS (initialize.f90:778-824): MAGNETIC + DISPL + USE_PML -> 10,
    and 18 with a 2D instruction; MAGNETIC without DISPL -> 8 (its 2-D form,
    12, and FLOWS are not built)."""
    mag = PARAMS_I.replace("magnetic = .false.", "magnetic = .true.")
    assert SparcParams.from_params_i(mag).option == 10
    q = SparcParams.from_params_i(mag).instruction("adjoint\n2D\n")
    assert q.option == 18 and q.ny == 1 and q.compute_adjoint
    with pytest.raises(ValueError):
        SparcParams(option=18, ny=4).validate()
    q8 = SparcParams.from_params_i(mag + "logical, parameter :: DISPL = .false.\n")
    assert q8.option == 8
    with pytest.raises(ValueError):
        q8.instruction("spectral\n2D\n")
    with pytest.raises(ValueError):
        SparcParams.from_params_i(PARAMS_I.replace("FLOWS = .FALSE.", "FLOWS = .TRUE."))
    assert SparcParams.from_params_i(PARAMS_I + "logical, parameter :: DISPL = .false.\n").option == 2


def test_params_validation():
    with pytest.raises(ValueError):
        SparcParams(nx=100).validate()
    with pytest.raises(ValueError):
        SparcParams(option=12).validate()            # the 2-D MHD velocity form is not built
    with pytest.raises(ValueError):
        SparcParams(option=17, ny=4).validate()
    SparcParams(option=8).validate()
    SparcParams(option=10).validate()
    SparcParams().validate()


def test_derived_quantities_match_read_parameters():
    # initialize.f90:978-981 with solartime = 4 h, nupeak = 0.0017 (REAL*4)
    p = config_quiet_256()
    mt = int(np.floor((4 * 3600.0 + 2.0 / r4(0.0017)) / 2.0)) + 2
    assert p.maxtime == 15 * (mt // 15) == 7785
    assert p.forcing_length == 520 and p.steps == 15 and p.freq_filtering == 30


def test_polytrope_table_law():
    t = polytrope_table(300, z_bot_mm=-25.0, z_top_mm=1.2)
    z = (t[:, 0] - 1.0) * 69598946770.0 / 1e8
    assert np.all(np.diff(z) > 0)
    assert z[0] == pytest.approx(-25.0, abs=1e-6) and abs(z[-1] - 1.2) < 0.05
    below = z <= 1e-9
    dc = np.diff(t[below, 1])
    assert np.allclose(dc, dc[0], rtol=1e-9)       # uniform in sound speed below z = 0
    assert np.allclose(t[:, 3], t[:, 2] * t[:, 1] ** 2 / t[:, 5])
    assert np.all(t[:, 2] > 0) and np.all(t[:, 4] == t[0, 4])


def test_adjoint_planes_time_reversal_and_placement():
    p = SparcParams(nx=32, ny=32, nz=48)
    pix = sources.receiver_pixels(p, n=4, radius_mm=50.0)
    res = np.arange(4 * 5, dtype=float).reshape(4, 5)
    pl = sources.adjoint_planes(p, res, pix)
    for r, (iy, ix) in enumerate(pix):
        assert np.array_equal(pl[:, iy, ix], res[r, ::-1])
    assert pl.sum() == res.sum()


def test_master_pixel_plane_peaks_at_xloc():
    p = SparcParams(nx=256, ny=1, nz=300, option=17)
    pl = sources.master_pixel_plane(p, -5.0)
    x = (np.arange(p.nx) / p.nx - 0.5) * r4(p.xlength) * float(np.float32(1e-8))
    assert abs(x[np.argmax(pl[0])] - (-5.0)) <= (x[1] - x[0])


def test_byte_model():
    p = config_quiet_256().replace(precision="f32", nsrc=1)
    f = bytes_model.field_bytes(p)
    assert f == 129 * 256 * 300 * 8
    assert bytes_model.stage_alg_bytes(p, 2) == 18 * f + 6 * bytes_model.pml_field_bytes(p)
    per_pt = bytes_model.alg_bytes_per_point_step(p)
    assert 405 < per_pt < 425


def test_compute_tt_recovers_a_shift():
    from sparc_gb300.pipeline import compute_tt
    dt = 30.0
    t = np.arange(256) * dt
    w = lambda tt: np.cos(2 * np.pi * 3e-3 * (tt - 3000)) * np.exp(-((tt - 3000) / 600.0) ** 2)
    u0 = w(t)
    for shift in (0.0, 12.0, -47.0, 95.0):
        tau = compute_tt(u0, w(t - shift), dt)
        assert abs(tau - shift) < 2.0, (shift, tau)
    assert abs(compute_tt(u0, u0, dt)) < 1e-6


def test_roofline_credits():
    """The per-unit figures of the roofline lines: the quiet form's minimal
    per-stage schedule (163.3 field accesses per point-step) and the flux
    tube's (423), in bytes per grid-point-step."""
    assert abs(bytes_model.reference_schedule_bytes_per_point_step("f32") - 653.333) < 1e-3
    assert abs(bytes_model.reference_schedule_bytes_per_point_step("f64") - 1306.667) < 1e-3
    assert bytes_model.MHD_SCHEDULE_ACCESSES == 423
    assert bytes_model.mhd_schedule_bytes_per_point_step("f32") == 1692
    assert bytes_model.mhd_schedule_bytes_per_point_step("f64") == 3384
