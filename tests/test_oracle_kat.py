"""Known-answer tests of the CPU oracle (no GPU).  They pin the restatement to
facts that follow from the reference's own coefficients and literal kinds."""
import os

import numpy as np
import pytest

from cases import rel_l2, small_params, small_params_2d, table_for

from oracle import oracle as O

F32 = np.float32


@pytest.fixture(scope="module")
def orc():
    O.build()
    p = small_params()
    return O.Oracle(p, table_for(p))


@pytest.mark.parametrize("bc", [0, 1])
def test_dbyd2_matches_dense_numpy_twin(bc):
    rng = np.random.default_rng(5)
    b = rng.standard_normal((40, 7))
    assert rel_l2(O.dbyd2(b, bc), O.dbyd2_numpy(b, bc)) < 1e-13


def test_dbyd2_linear_ramp_carries_real4_alpha():
    # interior rows of a linear ramp: R = d2i*5/3 and the solution is
    # R / (1 + 2*alpha) with alpha the REAL*4 value of 1/3 (dbyd2.f90:152)
    n2 = 200
    b = np.arange(n2, dtype=np.float64)[:, None] * np.ones((1, 3))
    a = O.dbyd2(b, 1)
    d2i = float(n2 - 1)
    alpha = float(F32(1.0) / F32(3.0))
    expect = d2i * (d2i * 7.0 / 9.0 * 2.0 + d2i / 36.0 * 4.0) / d2i / (1.0 + 2.0 * alpha)
    mid = a[60:140, 0]
    assert np.allclose(mid, expect, rtol=1e-14, atol=0)
    assert abs(expect / d2i - 1.0) > 1e-8          # not exact: the REAL*4 alpha shows


def test_dbyd2_sixth_order_interior():
    errs = []
    for n2 in (129, 257):
        xi = np.linspace(0.0, 1.0, n2)
        b = np.sin(16 * np.pi * xi)[:, None]
        a = O.dbyd2(b, 1)[:, 0]
        exact = 16 * np.pi * np.cos(16 * np.pi * xi)
        sl = slice(n2 // 4, 3 * n2 // 4)
        errs.append(np.abs(a[sl] - exact[sl]).max())
    assert errs[1] < errs[0] / 30.0


@pytest.mark.parametrize("n2,tol", [(64, 1e-13), (24, 1e-8)])
def test_dbyd2_periodic_matches_dense(n2, tol):
    # The cyclic branch of MTRIDAG (mtridag.f90:19-64) back-substitutes row
    # n2-1 with betau only, dropping the fill-in alpha*betas(n2-2) of size
    # ~0.382**(n2-3): exact to round-off for n2 = 64, ~1e-9 off for n2 = 24.
    rng = np.random.default_rng(9)
    b = rng.standard_normal((n2, 3))
    a = O.dbyd2(b, 5)
    d2i = float(n2)
    c1, c2 = d2i * 7.0 / 9.0, d2i / 36.0
    rhs = c1 * (np.roll(b, -1, 0) - np.roll(b, 1, 0)) + c2 * (np.roll(b, -2, 0) - np.roll(b, 2, 0))
    al = float(F32(1.0) / F32(3.0))
    M = np.eye(n2) + al * (np.roll(np.eye(n2), 1, 1) + np.roll(np.eye(n2), -1, 1))
    err = rel_l2(a, np.linalg.solve(M, rhs))
    assert err < tol
    if n2 == 24:
        assert err > 1e-13       # the fill-in omission is visible at this size


def test_dbyd2_rejects_bad_bc():
    with pytest.raises(ValueError):
        O.dbyd2(np.zeros((10, 2)), 6)


def test_lddrk_amplification_polynomial(orc):
    # G(z) = 1 + z + 0.5 z^2 + o3 z^3 + o4 z^4 + o5 z^5 with the REAL*4 optimals (step.f90:28-40)
    info = orc.info()
    b = [info[f"beta{i}"] / info["deltat"] for i in range(1, 6)]
    assert b[0] == 0.0
    c2, c3 = b[4], b[4] * b[3]
    c4, c5 = c3 * b[2], c3 * b[2] * b[1]
    assert c2 == 0.5
    assert c3 == pytest.approx(float(F32(0.1665579725791151184)), rel=1e-15)
    assert c4 == pytest.approx(float(F32(0.03950410250586729987)), rel=1e-15)
    assert c5 == pytest.approx(float(F32(0.007810706393337838236)), rel=1e-15)


def test_z_filter_coefficients_preserve_dc_and_kill_nyquist():
    co = [0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125]
    assert co[0] + sum(co[1:]) == 1.0
    assert co[0] + sum(c * (-1) ** i for i, c in enumerate(co[1:], 1)) == 0.0


def test_spectral_ddx_is_exact_and_drops_nyquist(orc):
    p = orc.p
    info = orc.info()
    x = np.arange(p.nx) / p.nx
    k = 3
    v = np.broadcast_to(np.sin(2 * np.pi * k * x), (p.nz, p.ny, p.nx)).copy()
    d = orc.ddx(v)
    # eyekx uses the REAL*4 pi (initialize.f90:205)
    expect = k * 2 * info["pi"] * np.cos(2 * np.pi * k * x) * info["stretchx"]
    assert np.abs(d - expect).max() < 1e-11 * np.abs(expect).max()
    nyq = np.broadcast_to(np.cos(np.pi * np.arange(p.nx)), (p.nz, p.ny, p.nx)).copy()
    assert np.abs(orc.ddx(nyq)).max() < 1e-12


def test_ddx_matches_numpy_fft_twin(orc):
    rng = np.random.default_rng(2)
    v = rng.standard_normal((orc.p.nz, orc.p.ny, orc.p.nx))
    info = orc.info()
    assert rel_l2(orc.ddx(v), O.fft_ddx_numpy(v, info["stretchx"], info["pi"])) < 1e-13
    vt = np.ascontiguousarray(np.swapaxes(v, 1, 2))
    dy = np.swapaxes(O.fft_ddx_numpy(vt, info["stretchy"], info["pi"]), 1, 2)
    assert rel_l2(orc.ddy(v), dy) < 1e-13


def test_damping_rates_formula(orc):
    p = orc.p
    info = orc.info()
    pi, rsun = info["pi"], info["rsun"]
    constx = 2.0 * pi / float(F32(p.xlength)) * rsun
    h = p.nx // 2 + 1
    i = np.arange(h)
    j = np.arange(p.ny)
    jj = np.where(j <= p.ny // 2, j, p.ny - j)
    kay = np.sqrt(constx ** 2 * i[None, :] ** 2 + constx ** 2 * jj[:, None] ** 2)
    rate = rsun / info["dimc"] * float(F32(1e-6)) * 150.0 * (kay / 902.0) ** float(F32(2.2)) / p.nx / p.ny
    assert rel_l2(orc.damping_rates(), rate) < 1e-13


def test_damping_is_a_real_symmetric_multiplier(orc):
    rng = np.random.default_rng(4)
    v = rng.standard_normal((orc.p.nz, orc.p.ny, orc.p.nx))
    r = orc.damp(v, np.zeros_like(v))
    # linear, and the DC mode is untouched (rate 0 at k = 0)
    assert rel_l2(orc.damp(2 * v, np.zeros_like(v)), 2 * r) < 1e-14
    assert abs(r.mean()) < 1e-13 * np.abs(r).max()


def test_forward_source_restatements_agree():
    from sparc_gb300.sources import gabor_series
    p = small_params()
    a = O.forward_source(p, 3000)
    b = gabor_series(p, 3000)
    assert np.allclose(a, b, rtol=1e-14, atol=1e-14 * np.abs(a).max())
    assert np.abs(a).max() > 0


def test_setup_derived_quantities(orc):
    p = orc.p
    info = orc.info()
    assert int(info["steps"]) == p.steps == 15
    assert int(info["freq_filtering"]) == p.freq_filtering == 30
    assert int(info["maxtime"]) == p.maxtime
    assert int(info["forcing_length"]) == p.forcing_length
    assert int(info["num_steps"]) == p.num_steps
    tab = table_for(p)
    z = tab[:, 0]
    assert abs(z[int(info["e_rad"]) - 1] - (1 + p.excitdep / 69598945280.0)) <= np.diff(z).max()
    assert info["rsun"] == float(F32(69598946770.0))
    assert info["pi"] == float(F32(3.14159265358979))


def test_pml_profiles(orc):
    pr = orc.profiles()
    nb, nt, nz = orc.p.npmlbot, orc.p.npmltop, orc.p.nz
    # az = -dampz vanishes outside the PML; g and the gradients are scaled by
    # functiondecay = alpha/(dampz+alpha), which is 0 at k = 1 (physics.f90:265-289)
    assert np.all(pr["az"][nb:nz - nt] == 0.0)
    assert np.all(pr["az"][:nb - 1] < 0)
    assert pr["g"][0] == 0.0 and pr["gradp0_z"][0] == 0.0
    assert pr["g"][nz - 1] == 0.0


def test_oracle_step_is_linear():
    p = small_params(nx=16, ny=16, nz=32, npmlbot=4, npmltop=4)
    tab = table_for(p)
    rng = np.random.default_rng(0)
    a1 = rng.standard_normal((6, p.nz, p.ny, p.nx)) * 1e-3
    a2 = rng.standard_normal((6, p.nz, p.ny, p.nx)) * 1e-3
    out = []
    for a in (a1, a2, a1 + a2):
        o = O.Oracle(p, tab)
        o.set_state(a)
        o.step(3)
        out.append(o.state()[0])
    assert rel_l2(out[2], out[0] + out[1]) < 1e-12


def test_oracle_2d_runs_and_conserves_zero_y_fields():
    p = small_params_2d(nx=32, nz=32, npmlbot=4, npmltop=4)
    o = O.Oracle(p, table_for(p))
    rng = np.random.default_rng(1)
    a = rng.standard_normal((6, p.nz, 1, p.nx)) * 1e-3
    a[1] = 0; a[4] = 0
    o.set_state(a)
    o.step(31)
    s = o.state()[0]
    assert np.all(np.isfinite(s))
    assert np.abs(s[1]).max() == 0 and np.abs(s[4]).max() == 0


GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz")


def test_oracle_reproduces_golden_fixtures():
    from golden.make_golden import compute
    g = np.load(GOLDEN)
    now = compute()
    for k in g.files:
        assert rel_l2(now[k], g[k]) < 1e-12, k


def _mhd_case(nx=16, ny=16, nz=32, b_surf=800.0):
    from cases import small_params, table_for
    from sparc_gb300.background import flux_tube_background
    p = small_params(nx=nx, ny=ny, nz=nz, npmlbot=4, npmltop=0, option=10)
    tab = table_for(p)
    return p, tab, flux_tube_background(p, tab, b_surf=b_surf, r_surf_mm=8.0)


def test_mhd_setup_follows_the_reference_order():
    """READ_IN_FIELD, the field reduction with its REAL*4 top taper, and curl
    B0 without its d/dz parts (physics.f90:116-159), against numpy twins."""
    from oracle import oracle as O
    p, tab, (rho, c, pr, bx, by, bz) = _mhd_case()
    o = O.Oracle(p, tab)
    o.set_mhd(rho, c, pr, bx, by, bz)
    m = o.mhd_profiles()
    info = o.info()
    dimc, dimrho = info["dimc"], info["dimrho"]
    dimb = np.sqrt(4.0 * info["pi"] * dimc ** 2 * dimrho)
    cq = tab[:, 1] / dimc
    red = ((bz / dimb) ** 2 + (bx / dimb) ** 2 + (by / dimb) ** 2) / ((rho / dimrho) * cq[:, None, None] ** 2)
    red = 8.0 / (8.0 + red)
    nz = p.nz
    for k1 in range(nz - 10, nz + 1):
        red[k1 - 1] *= float(np.float32(np.float32(k1 - nz) / np.float32(10.0)) ** np.float32(4.0))
    assert rel_l2(m["boz"], bz / dimb * np.sqrt(red)) < 1e-14
    assert np.abs(m["boz"][-1]).max() == 0.0                        # the taper zeroes the top plane
    assert np.array_equal(m["curlboy"], -o.ddx(m["boz"]))
    assert np.array_equal(m["curlbox"], o.ddy(m["boz"]))
    assert rel_l2(m["curlboz"], o.ddx(m["boy"]) - o.ddy(m["box"])) < 1e-15
    z = tab[:, 0]
    spz = 200.0 / (1.0 + np.exp((float(np.float32(1.002)) - z) / float(np.float32(1e-4)))) + \
        300.0 / (1.0 + np.exp((z - (z[0] + float(np.float32(0.005)))) / float(np.float32(5e-4))))
    assert rel_l2(m["spongexyz"][:, 0, 0], spz) < 1e-14
    assert np.array_equal(m["gradp0_x"], o.ddx(pr / (dimrho * dimc ** 2)))


def test_mhd_runs_and_drives_the_induction_pml():
    from oracle import oracle as O
    p, tab, bg = _mhd_case()
    o = O.Oracle(p, tab)
    o.set_mhd(*bg)
    a = np.zeros((6, p.nz, p.ny, p.nx))
    a[0, 8:12] = 1e-6 * np.random.default_rng(0).standard_normal((4, p.ny, p.nx))
    o.set_state(a)
    o.step(3)
    st, scr, pml = o.state()
    assert np.isfinite(st).all() and np.isfinite(pml).all()
    assert pml.shape[0] == 6
    assert np.abs(pml[2:]).max() > 0          # psi_dzbx, psi_dzby, psi_induction_bx/by are driven


def _mhd2d_case(nx=32, nz=32, b_surf=300.0):
    from cases import small_params_2d, table_for
    from sparc_gb300.background import flux_sheet_background
    p = small_params_2d(nx=nx, nz=nz, npmlbot=4, npmltop=4, option=18)
    tab = table_for(p)
    return p, tab, flux_sheet_background(p, tab, b_surf=b_surf)


def _dbyd1_ibc0_dense(b, n1):
    """DBYD1 (dbyd1.f) with ibc 0 as a dense solve: REAL*4 coefficients,
    rows 1 and n1 of the right side zero, the tridiagonal system with
    diagonal 1, upper (0, 3/4, 1/3 ..., 1/8, 0) and its mirror below."""
    f = np.float32
    d1i = f(n1 - 1)
    c1, c2 = float(d1i * f(7) / f(9)), float(d1i / f(36))
    bc = [float(f(-43) / f(96) * d1i), float(f(-5) / f(6) * d1i), float(f(9) / f(8) * d1i),
          float(f(1) / f(6) * d1i), float(f(-1) / f(96) * d1i)]
    up = np.zeros(n1)
    up[2:n1 - 2] = float(f(1) / f(3))
    up[1] = float(f(3) / f(4))
    up[n1 - 2] = float(f(1) / f(8))
    lo = up[::-1].copy()
    lo[n1 - 1] = 0.0
    M = np.eye(n1) + np.diag(up[:-1], 1) + np.diag(lo[1:], -1)
    r = np.zeros(b.shape)
    r[..., 2:n1 - 2] = c1 * (b[..., 3:n1 - 1] - b[..., 1:n1 - 3]) + c2 * (b[..., 4:] - b[..., :n1 - 4])
    r[..., 1] = sum(bc[i] * b[..., i] for i in range(5))
    r[..., n1 - 2] = -sum(bc[i] * b[..., n1 - 1 - i] for i in range(5))
    return np.linalg.solve(M, r.reshape(-1, n1).T).T.reshape(b.shape)


def test_mhd2d_setup_follows_the_reference_order():
    """mp_Initialize_RHS_2d's magnetic part (physics2d.f90:106-195): B_x =
    -d psi/dz, B_z = DBYD1(psi) stretchx, curl_y B0 = dBx/dz - dBz/dx, the
    PML at both ends, against numpy twins."""
    from oracle import oracle as O
    p, tab, (rho, c, pr, psi) = _mhd2d_case()
    o = O.Oracle(p, tab)
    o.set_mhd2d(rho, c, pr, psi)
    m = o.mhd_profiles()
    info = o.info()
    dimc, dimrho = info["dimc"], info["dimrho"]
    dimb = np.sqrt(4.0 * info["pi"] * dimc ** 2 * dimrho)
    stretchx = info["rsun"] / float(np.float32(p.xlength))
    assert rel_l2(m["box"], -o.ddz(psi, 1) / dimb) < 1e-14
    assert rel_l2(m["boz"], _dbyd1_ibc0_dense(psi, p.nx) * stretchx / dimb) < 1e-12
    assert np.abs(m["boy"]).max() == 0.0 and np.abs(m["curlbox"]).max() == 0.0
    assert rel_l2(m["curlboy"], o.ddz(m["box"], 1) - o.ddx(m["boz"])) < 1e-14
    # B_z a plane below the fade is close to the generator's field (DBYD1
    # spans the box with n-1 intervals, so the scale is n/(n-1) off)
    z_cm = (tab[:, 0] - 1.0) * 69598946770.0
    k0 = int(np.argmin(np.abs(z_cm + 1.0e8)))
    bz_cgs = m["boz"][k0, 0] * dimb
    assert abs(bz_cgs.max() / 300.0 - 1.0) < 0.1, bz_cgs.max()
    # PML: a_z = -dampz in both layers, zero on each layer's inner plane and
    # growing towards the edge
    az = m["az"][:, 0, p.nx // 2]
    assert (az[:3] < 0).all() and (az[-3:] < 0).all() and np.all(az[3:-3] == 0)
    assert az[0] < az[1] < az[2] and az[-1] < az[-2] < az[-3]
    assert np.array_equal(m["gradp0_x"], o.ddx(pr / (dimrho * dimc ** 2)))


def test_mhd2d_without_field_is_the_quiet_2d_form():
    """With psi = 0 every magnetic term vanishes and option 18 steps as
    option 17 does (physics2d.f90:724-943 against :948-1105, same filter
    cadence) once damping is off: option 18 calls DAMP_VELOCITY, option 17
    never does."""
    from oracle import oracle as O
    from cases import random_state
    p, tab, (rho, c, pr, psi) = _mhd2d_case()
    p = p.replace(damp_waves=False)
    p17 = p.replace(option=17)
    o18, o17 = O.Oracle(p, tab), O.Oracle(p17, tab)
    o18.set_mhd2d(tab[:, 2][:, None, None] * np.ones_like(rho), c, tab[:, 3][:, None, None] * np.ones_like(pr),
                  np.zeros_like(psi))
    a, pml = random_state(p17, 5, 1e-6)
    pml6 = np.zeros((6,) + pml.shape[1:])
    pml6[:2] = pml
    pml6[1, 0] = 0.0
    pml[1, 0] = 0.0
    o18.set_state(a, pml6)
    o17.set_state(a, pml)
    o18.step(31)
    o17.step(31)
    s18, _, q18 = o18.state()
    s17, _, q17 = o17.state()
    assert rel_l2(s18, s17) < 1e-12
    assert rel_l2(q18[:2], q17) < 1e-12


def test_mhd2d_runs_and_drives_both_pml_layers():
    from oracle import oracle as O
    p, tab, bg = _mhd2d_case()
    o = O.Oracle(p, tab)
    o.set_mhd2d(*bg)
    a = np.zeros((6, p.nz, 1, p.nx))
    rng = np.random.default_rng(0)
    a[0, 2:6] = 1e-6 * rng.standard_normal((4, 1, p.nx))
    a[2, -6:-2] = 1e-6 * rng.standard_normal((4, 1, p.nx))
    o.set_state(a)
    o.step(3)
    st, scr, pml = o.state()
    assert np.isfinite(st).all() and np.isfinite(pml).all()
    assert pml.shape[0] == 6
    for i in (0, 1, 2, 4):                 # psi_vz, psi_p, psi_dzbx, psi_induction_bx
        assert np.abs(pml[i, :4]).max() > 0 and np.abs(pml[i, 4:]).max() > 0, i
    assert np.abs(pml[3]).max() == 0 and np.abs(pml[5]).max() == 0
    assert np.abs(st[1]).max() == 0 and np.abs(st[4]).max() == 0


def test_mhd8_without_field_keeps_b_at_zero():
    """MP_MHD_PML_3D (pml.f90:80-208) with B0 = 0: the fluxes of v x B0
    vanish, so b and the four magnetic PML auxiliaries stay exactly zero
    while the hydrodynamic fields evolve."""
    from oracle import oracle as O
    from cases import small_params, table_for
    p = small_params(nx=16, ny=16, nz=32, npmlbot=4, npmltop=4, option=8)
    tab = table_for(p)
    o = O.Oracle(p, tab)
    rho = np.broadcast_to(tab[:, 2][:, None, None], o.shape).copy()
    c = np.broadcast_to(tab[:, 1][:, None, None], o.shape).copy()
    pr = np.broadcast_to(tab[:, 3][:, None, None], o.shape).copy()
    z = np.zeros(o.shape)
    o.set_mhd(rho, c, pr, z, z, z)
    a = np.zeros((8,) + o.shape)
    a[1:4] = np.random.default_rng(3).standard_normal((3,) + o.shape) * 1e-6
    o.set_state(a)
    o.step(31)
    st, _, pml = o.state()
    assert np.abs(st[5:]).max() == 0.0
    assert np.abs(pml[2:]).max() == 0.0
    assert np.isfinite(st).all() and np.abs(st[1:4]).max() > 0 and np.abs(pml[:2]).max() > 0


def test_mhd8_drives_induction_and_both_pml_layers():
    from oracle import oracle as O
    p, tab, bg = _mhd_case()
    p = p.replace(option=8, npmltop=4)
    o = O.Oracle(p, tab)
    o.set_mhd(*bg)
    a = np.zeros((8,) + o.shape)
    a[1:4] = np.random.default_rng(4).standard_normal((3,) + o.shape) * 1e-6
    o.set_state(a)
    o.step(5)
    st, _, pml = o.state()
    assert np.isfinite(st).all()
    assert np.abs(st[5:]).max() > 0                       # b from the induction equation
    for i in range(6):
        assert np.abs(pml[i, :4]).max() > 0 and np.abs(pml[i, 4:]).max() > 0, i


def _filter_var_z(v):
    """FILTER_VAR_Z (kernels.f90:845-881) on (nz, ny, nx)."""
    co = [0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125]
    nz = v.shape[0]
    out = v.copy()
    for k in (1, 2, 3, 4):
        out[k] = 0.5 * (v[k + 1] + v[k - 1])
    for k in range(5, nz - 5):
        out[k] = co[0] * v[k] + sum(0.5 * co[i] * (v[k - i] + v[k + i]) for i in range(1, 6))
    for k in (nz - 5, nz - 4, nz - 3, nz - 2):
        out[k] = 0.5 * (v[k + 1] + v[k - 1])
    return out


def test_mhd2d_b_kernels_reduce_to_the_2d_algebra():
    """The MAGNETIC_KERNELS block (kernels.f90:337-453), restated in the oracle
    term by term on 3-vectors, against its 2-D reduction (B0 = (Bx, 0, Bz),
    curl B0 = (0, curlby, 0), d/dy = 0: every cross product has one
    component and each curl two derivatives), built here from the oracle's
    d/dx and d/dz with bc 0 and FILTER_VAR_Z (CURL_KERN's ddzkern)."""
    from oracle import oracle as O
    p, tab, bg = _mhd2d_case()
    o = O.Oracle(p, tab)
    o.set_mhd2d(*bg)
    rng = np.random.default_rng(21)
    sh = (p.nz, 1, p.nx)
    fxx, fxz, avx, avz = (rng.standard_normal(sh) for _ in range(4))
    z0 = np.zeros(sh)
    fxi = np.stack([fxx, z0, fxz])
    av = np.stack([avx, z0, avz])
    o.kernel_reset()
    o.kernel_accumulate_b(fxi, av)
    kb = o.kernel_finish_b(15)
    Dx = o.ddx
    Dz0 = lambda v: _filter_var_z(o.ddz(v, 0))
    m = o.mhd_profiles()
    info = o.info()
    dimb = np.sqrt(4.0 * info["pi"] * info["dimc"] ** 2 * info["dimrho"])
    psi = bg[3]
    kbox = -Dz0(psi) / dimb
    kboz = m["boz"]
    cby = Dz0(kbox) - Dx(kboz)
    ty = kbox * fxz - fxx * kboz
    fbx, fbz = -Dz0(ty), Dx(ty)
    t2y = Dz0(fbx) - Dx(fbz)
    t3y = avx * fbz - fbx * avz
    uy = kbox * avz - avx * kboz
    abx, abz = -Dz0(uy), Dx(uy)
    t4y = Dz0(abx) - Dx(abz)
    sy = Dz0(-avz * cby) - Dx(avx * cby)
    dA = Dx(avx) + _filter_var_z(o.ddz(avz, 1))
    vy = fxx * dA * kboz - kbox * fxz * dA
    kx = -avz * t2y - Dz0(t3y) - fxz * t4y + sy * fxz - fxz * cby * dA - Dz0(vy)
    kz = avx * t2y + Dx(t3y) + fxx * t4y - sy * fxx + fxx * cby * dA + Dx(vy)
    ts = float(np.float32(p.timestep))
    dimen = 1.0 / (info["diml"] * float(np.float32(1e-8)) * float(np.float32(p.xlength))
                   * float(np.float32(1e-8)) * dimb)
    assert rel_l2(kb[0], kx * 15 * ts * dimen) < 1e-11
    assert rel_l2(kb[1], kz * 15 * ts * dimen) < 1e-11
    kpsi = Dz0(kx * 15 * ts * dimen) - Dx(kz * 15 * ts * dimen)
    assert rel_l2(kb[2], kpsi) < 1e-11
    # bilinear in (xi, v_adjoint); zero without a field
    o.kernel_reset()
    o.kernel_accumulate_b(2.0 * fxi, av)
    assert rel_l2(o.kernel_finish_b(15), 2.0 * kb) < 1e-14
    o0 = O.Oracle(p, tab)
    o0.set_mhd2d(bg[0], bg[1], bg[2], np.zeros_like(bg[3]))
    o0.kernel_reset()
    o0.kernel_accumulate_b(fxi, av)
    assert np.abs(o0.kernel_finish_b(15)).max() == 0.0


# ---- adjoint source (ADJOINT_SOURCE_FILT, driver.f90:1262-1686) -------------------

def test_adjsrc_inverse_and_compute_tt():
    from oracle import adjoint_source as A
    m = np.array([[1.0, -0.5, 0.25], [1.0, 0.0, 0.0], [1.0, 0.5, 0.25]])
    assert np.allclose(A.inverse3(m), np.linalg.inv(m), rtol=1e-14, atol=1e-14)
    t = np.arange(81) * 0.5
    w = lambda s: np.cos(2 * np.pi * 0.2 * (t - 20 - s)) * np.exp(-((t - 20 - s) / 4.0) ** 2)
    for s in (0.0, 0.13, -0.31):
        assert abs(A.compute_tt(w(0.0), w(s), 0.5) - s) < 0.02, s
    assert list(A.distmat(6)) == [0.0, 1.0, 2.0, 3.0, -2.0, -1.0]


def test_adjsrc_zero_for_equal_data_and_measures_a_shift():
    from adjsrc_cases import CASE, delayed, ridge_field
    from oracle import adjoint_source as A
    c = CASE
    t = np.arange(c["nt"]) * 0.5
    acc = ridge_field(c["nx"], c["nt"], c["xlength"], c["outputcad"], seed=3)
    adj0, mis0, n0, win, taus0 = A.adjoint_source_filt(acc, acc.copy(), c["xlength"], c["outputcad"], c["x00"], t,
                                                        c["ridges"], c["bands"])
    assert n0 > 20 and mis0 < 1e-20 and max(abs(v) for v in taus0.values()) < 1e-9
    assert np.abs(adj0).max() < 1e-9 * np.abs(acc).max()
    shift = 12.0                                     # s
    adj, mis, n, win2, taus = A.adjoint_source_filt(acc, delayed(acc, shift, c["outputcad"]), c["xlength"],
                                                    c["outputcad"], c["x00"], t, c["ridges"], c["bands"])
    tt = np.array(list(taus.values())) * 60.0       # minutes -> s
    assert n == n0 and win2 == win
    assert np.median(np.abs(tt - shift)) < 1.5, np.median(tt)
    assert mis > 0 and np.abs(adj).max() > 0
    # a line search reuses the windows (windows.0/1) and measures the same
    adj3, mis3, n3, _, _ = A.adjoint_source_filt(acc, delayed(acc, shift, c["outputcad"]), c["xlength"],
                                                 c["outputcad"], c["x00"], t, c["ridges"], c["bands"], windows_in=win)
    assert np.array_equal(adj3, adj) and mis3 == mis and n3 == n


def test_misfit_all_zero_for_equal_data():
    """MISFIT_ALL (driver.f90:1702-2076): three bands x three sets, zero misfit
    when the data equal the synthetic, measurements in every band and set."""
    from adjsrc_cases import CASE, delayed, ridge_field
    from oracle import adjoint_source as A
    c = CASE
    t = np.arange(c["nt"]) * 0.5
    acc = ridge_field(c["nx"], c["nt"], c["xlength"], c["outputcad"], seed=6)
    m0, n0, w0 = A.misfit_all(acc, acc.copy(), c["xlength"], c["outputcad"], c["x00"], t, c["ridges"])
    assert m0.shape == (3, 3) and np.all(n0 > 10) and np.abs(m0).max() < 1e-18
    m1, n1, w1 = A.misfit_all(acc, delayed(acc, 12.0, c["outputcad"]), c["xlength"], c["outputcad"], c["x00"], t,
                              c["ridges"])
    assert np.array_equal(n1, n0) and w1 == w0 and np.all(m1 > 0)


# ---- model update (grad.py:158-301) --------------------------------------------------

def test_model_update_filters_pin():
    """gaussian_z against scipy.ndimage.gaussian_filter1d (mode 'reflect', as
    grad.py calls it); filterz 'smooth' zeroes plane 4 and the top plane (its
    temp array starts at zero); filterx is a circular convolution with the
    unnormalised Gaussian."""
    from oracle import model_update as U
    rng = np.random.default_rng(8)
    a = rng.standard_normal((40, 1, 24))
    gf = pytest.importorskip("scipy.ndimage").gaussian_filter1d
    assert rel_l2(U.gaussian_z(a, 2.0), gf(a, sigma=2.0, axis=0)) < 1e-14
    s = U.filterz_smooth(a)
    assert np.all(s[4] == 0) and np.all(s[-1] == 0) and np.array_equal(s[0], a[0])
    assert np.allclose(s[2], 0.5 * (a[1] + a[3]))
    x = np.fft.fftfreq(24) * 24
    g = np.exp(-x ** 2 / 32.0)
    conv = np.stack([[np.array([np.sum(a[k, 0] * np.roll(g[::-1], i + 1)) for i in range(24)])] for k in range(40)])
    assert rel_l2(U.filterx(a), conv) < 1e-12
    anti = U.antisymmetrize(a)
    assert np.allclose(anti, -anti[..., ::-1])


def test_model_update_directions_and_models():
    from oracle import model_update as U
    rng = np.random.default_rng(9)
    g_c, g_psi = rng.standard_normal((2, 30, 1, 16))
    u_c, u_psi, con = U.update_direction(g_c, g_psi)
    assert con == 0.0 and u_psi is g_psi
    lg, lu_c, lu_psi = rng.standard_normal((3, 30, 1, 16))
    u_c, u_psi, con = U.update_direction(g_c, g_psi, (lg, lu_c, lu_psi))
    want = max(np.sum(g_psi * (g_psi - lg)) / np.sum(lg ** 2), 0.0)
    assert con == pytest.approx(want) and np.allclose(u_psi, g_psi + want * lu_psi)
    m = rng.standard_normal((30, 1, 16))
    tm = U.test_models(m, u_psi)
    assert tm.shape == (5, 30, 1, 16)
    assert np.allclose(tm[2] - m, 3e-7 * np.sqrt(np.mean(m ** 2)) * u_psi / np.abs(u_psi).max())


def test_tubex_restatement_pins():
    """The restatement of code_python/tubex.py: the shipped zeroB run gives
    back the quiet column; the compact z derivative of A reproduces the
    analytic B_x = -dA/dz; the FFT calculus differentiates and integrates
    band-limited fields exactly."""
    from cases import small_params_2d
    from oracle import backgrounds as B
    from oracle.oracle import Oracle
    from sparc_gb300.background import polytrope_table
    nz, nx = 120, 128
    tab = polytrope_table(nz, z_bot_mm=-25.0, z_top_mm=1.2)
    o = Oracle(small_params_2d(nx=nx, nz=nz, xlength=400e8, ylength=400e8), tab)
    r = B.tubex(tab, o, nx=nx)
    assert np.array_equal(r["p"][:, 0, :], np.broadcast_to(tab[:, 3, None], (nz, nx)))
    assert np.array_equal(r["rho"][:, 0, :], np.broadcast_to(tab[:, 2, None], (nz, nx)))
    assert np.abs(r["c"][:, 0, :] / tab[:, 1, None] - 1).max() < 1e-14
    assert not any(np.any(r[m][f]) for m in ("true", "start") for f in ("bx", "bz", "psi"))
    # the starting field's B_x is the numerical -dA/dz; against the analytic one
    a0, dx, dz = 20.0, 10.0, 12.0
    r = B.tubex(tab, o, nx=nx, a0=a0, zero_b=False)
    assert not r["negative"]
    x = np.linspace(-200.0, 200.0, nx, endpoint=False)
    z = (tab[:, 0] - 1.0) * B.RSUN
    fx = -(x / dx) / (1 + (x / dx) ** 4)
    bx_exact = -a0 * (np.exp(z / dz) / dz)[:, None] * fx[None, :]
    # (the table's grid spacing jumps near z = 0: the compact scheme is good to ~1e-4 there)
    assert np.abs(r["start"]["bx"][:, 0, :] - bx_exact).max() < 5e-4 * np.abs(bx_exact).max()
    # the FFT calculus on a band-limited periodic field
    L = 400.0
    f = np.sin(2 * np.pi * 3 * (x[:, None] + 200) / L) + 0.5 + np.cos(2 * np.pi * 5 * x[:, None] / L) * z[None, :]
    df = (2 * np.pi * 3 / L) * np.cos(2 * np.pi * 3 * (x[:, None] + 200) / L) \
        - (2 * np.pi * 5 / L) * np.sin(2 * np.pi * 5 * x[:, None] / L) * z[None, :]
    assert np.abs(B.fft_differentiate(f, L) - df).max() < 1e-12
    assert np.abs(B.fft_integrate(df, L) - (f - f.mean(axis=0))).max() < 1e-12
