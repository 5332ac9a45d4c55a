"""Size-independent properties at the full sizes of the workloads (256x256x300
and the largest serving grid, 512x512x300), where the oracle is too slow to
compare against directly.  The path is linear in the state and the source,
and the state starts at zero:

* doubling the source doubles every field bit for bit in FP64 (scaling by 2
  commutes with rounding of normal numbers).  In FP32 the far tails of the
  field reach the subnormal range, where results round on a fixed grid; once
  the two runs differ there, later roundings can differ by an ulp, and the
  difference settles at the FP32 rounding level of the field (1e-7 to 1e-6
  of its maximum over hundreds of steps, measured) without growing: the
  FP32 runs are bounded at 1e-5 of each field's maximum, and the 675-step
  kernel workflow at the FP32 tolerances (relative L2 1e-4 for seismograms,
  1e-3 for kernels);
* superposition: the response to s1 + s2 is the sum of the responses, to
  FP64 rounding;
* the FP32 fused step against the FP64 per-stage path: surface seismograms
  within 1e-4 relative L2."""
import numpy as np
import pytest

from cases import rel_l2

pytestmark = pytest.mark.gpu


def _params(prec, nsrc, big=False):
    from sparc_gb300.params import config_quiet_256
    p = config_quiet_256().replace(precision=prec, nsrc=nsrc)
    if big:
        p = p.replace(nx=512, ny=512)
    return p


def _solver(p):
    from sparc_gb300.background import polytrope_table
    from sparc_gb300.solver import Solver
    return Solver(p, polytrope_table(p.nz))


def _series(p, n):
    from sparc_gb300 import sources
    return sources.ricker_series(p, n, delay=20.0)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_doubling_is_exact_256(gpu_lib, prec):
    from sparc_gb300 import sources
    p = _params(prec, 2)
    n = 30
    with _solver(p) as s:
        pl = sources.gaussian_plane(p, sigma_mm=1.0, x0_mm=3.0, y0_mm=-2.0)
        se = _series(p, n + 8)
        s.set_source_series(pl, se, slot=0)
        s.set_source_series(pl, 2.0 * se, slot=1)
        s.record_surface(n // p.steps + 2)
        s.step(n)
        s.sync(check_finite=True)
        a0, m0 = s.state(0)
        a1, m1 = s.state(1)
        r0, r1 = s.records(0), s.records(1)
    assert np.abs(a0).max() > 0 and np.abs(r0).max() > 0
    if prec == "f64":
        assert np.array_equal(a1, 2.0 * a0) and np.array_equal(m1, 2.0 * m0)
        assert np.array_equal(r1, 2.0 * r0)
    else:
        for x1, x0 in ((a1, a0), (m1, m0), (r1, r0)):
            assert np.abs(x1 - 2.0 * x0).max() <= 1e-5 * np.abs(x0).max()


def test_superposition_256_f64(gpu_lib):
    from sparc_gb300 import sources
    p = _params("f64", 3)
    n = 30
    with _solver(p) as s:
        p1 = sources.gaussian_plane(p, sigma_mm=1.0, x0_mm=-10.0, y0_mm=4.0)
        p2 = sources.gaussian_plane(p, sigma_mm=2.0, x0_mm=15.0, y0_mm=-6.0)
        se = _series(p, n + 8)
        s.set_source_series(p1, se, slot=0)
        s.set_source_series(p2, se, slot=1)
        s.set_source_series(p1 + p2, se, slot=2)
        s.step(n)
        a = [s.state(k)[0] for k in range(3)]
    assert rel_l2(a[2], a[0] + a[1]) < 1e-12, rel_l2(a[2], a[0] + a[1])


def test_fp32_seismograms_against_fp64_256(gpu_lib):
    """150 steps (10 outputs) of the 256x256x300 forward solve: the FP32 fused
    step's surface vz against the FP64 per-stage path."""
    from sparc_gb300 import sources
    n = 150
    recs = {}
    for prec in ("f64", "f32"):
        p = _params(prec, 1)
        with _solver(p) as s:
            s.set_source_series(sources.gaussian_plane(p, sigma_mm=1.0), _series(p, n + 8))
            s.record_surface(n // p.steps + 2)
            s.step(n)
            recs[prec] = s.records(0)
    assert recs["f64"].shape == recs["f32"].shape and np.abs(recs["f64"]).max() > 0
    err = rel_l2(recs["f32"][1:], recs["f64"][1:])
    assert err < 1e-4, err


def test_largest_grid_512(gpu_lib):
    """512x512x300 (the largest serving grid), FP32: finite, and doubling the
    source doubles the surface records and a field plane to within FP32
    rounding (1e-5 of their maxima)."""
    from sparc_gb300 import sources
    p = _params("f32", 2, big=True)
    n = 30
    with _solver(p) as s:
        pl = sources.gaussian_plane(p, sigma_mm=1.0)
        se = _series(p, n + 8)
        s.set_source_series(pl, se, slot=0)
        s.set_source_series(pl, 2.0 * se, slot=1)
        s.record_surface(n // p.steps + 2)
        s.step(n)
        s.sync(check_finite=True)
        r0, r1 = s.records(0), s.records(1)
        k = p.nz - 20
        f0, f1 = s.field(5, 0, k), s.field(5, 1, k)
    assert np.abs(r0).max() > 0 and np.isfinite(r0).all()
    assert np.abs(r1 - 2.0 * r0).max() <= 1e-5 * np.abs(r0).max()
    assert np.abs(f1 - 2.0 * f0).max() <= 1e-5 * np.abs(f0).max()


def test_mhd_flux_tube_doubling_256_f64(gpu_lib):
    """Option 10 on the 2 kG flux tube at 256x256x300, FP64: the perturbation
    equations are linear about the fixed background, so doubling the source
    doubles the physical state bit for bit."""
    from sparc_gb300 import sources
    from sparc_gb300.background import flux_tube_background, polytrope_table
    from sparc_gb300.solver import Solver
    pm = _params("f64", 2).replace(option=10, npmltop=0)
    tab = polytrope_table(pm.nz)
    n = 5
    with Solver(pm, tab) as s:
        s.set_mhd_background(*flux_tube_background(pm, tab))
        pl = sources.gaussian_plane(pm, 1.0, 20.0, 0.0)
        se = _series(pm, n + 8)
        s.set_source_series(pl, se, slot=0)
        s.set_source_series(pl, 2.0 * se, slot=1)
        s.step(n)
        s.sync(check_finite=True)
        a0, m0 = s.state(0)
        a1, m1 = s.state(1)
    assert np.abs(a0).max() > 0
    assert np.array_equal(a1, 2.0 * a0)
    # the bottom PML, which the wave has not reached after 5 steps, holds only
    # the compact solves' decaying tails (1e-89 and far below, down into the
    # FP64 subnormal range): doubled to within 1e-12 of their maximum
    assert np.abs(m1 - 2.0 * m0).max() <= 1e-12 * np.abs(m0).max()


def test_kernel_workflow_scaling_256_f32(gpu_lib):
    """The forward x adjoint workflow at 256x256x300, FP32 fields with FP64
    accumulation, 3 min of solar time: a forward source twice as strong with
    zero observations gives twice the seismograms and residuals, so twice the
    adjoint source, and four times K_c, K_rho and the hessian (bilinear in
    the forward and adjoint fields), to within the FP32 tolerances against
    FP64 (relative L2: seismograms 1e-4, kernels 1e-3)."""
    from sparc_gb300 import sources
    from sparc_gb300.background import polytrope_table
    from sparc_gb300.pipeline import KernelPipeline
    p = _params("f32", 2).replace(solartime=0.05)
    pl = KernelPipeline(p, polytrope_table(p.nz), segment=4)
    plane = sources.gaussian_plane(p, 1.0, 5.0, -5.0)
    se = _series(p, p.maxtime + 10)
    pix = sources.receiver_pixels(p, n=8, radius_mm=10.0)
    r = pl.run([plane, 2.0 * plane], se, np.zeros((2, pl.nt, p.ny, p.nx)), pix)
    assert np.abs(r.seismograms[0]).max() > 0 and np.abs(r.kc[0]).max() > 0
    assert rel_l2(r.seismograms[1], 2.0 * r.seismograms[0]) < 1e-4
    for q in ("kc", "krho", "hessian"):
        k = getattr(r, q)
        assert rel_l2(k[1], 4.0 * k[0]) < 1e-3, (q, rel_l2(k[1], 4.0 * k[0]))
