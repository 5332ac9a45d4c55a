"""GPU parity: the CUDA path (through the C ABI) against the FP64 CPU oracle on
the same seeded inputs.  Tolerances: FP64 path <= 1e-10 relative L2 per field;
FP32 path <= 1e-4 relative L2 on surface seismograms."""
import os

import numpy as np
import pytest

from cases import (gaussian_plane, random_state, rel_l2, small_params, small_params_2d, table_for)

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-4


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def make_pair(p, oracle_mod, gpu_lib):
    from sparc_gb300.solver import Solver
    tab = table_for(p)
    return Solver(p, tab), oracle_mod.Oracle(p, tab)


def test_setup_matches_oracle(gpu_lib, oracle_mod):
    p = small_params()
    g, o = make_pair(p, oracle_mod, gpu_lib)
    gi, oi = g.info(), o.info()
    for k in ("e_rad", "o_rad", "steps", "freq_filtering", "maxtime", "forcing_length", "num_steps"):
        assert gi[k] == int(oi[k]), k
    for k in ("delta_width", "deltat", "beta2", "beta3", "beta4", "beta5"):
        assert gi[k] == pytest.approx(oi[k], rel=1e-15), k
    zt, _ = g.tables()
    pr = o.profiles()
    # rows: stretch, unstretch, c2rho0, gradp0, rho0, gradrho0, rhoinv, g, az, bz
    np.testing.assert_allclose(zt[0], pr["stretch"], rtol=1e-14)
    np.testing.assert_allclose(zt[3], pr["gradp0_z"], rtol=1e-13, atol=1e-14 * abs(pr["gradp0_z"]).max())
    np.testing.assert_allclose(zt[5], pr["gradrho0_z"], rtol=1e-13, atol=1e-14 * abs(pr["gradrho0_z"]).max())
    np.testing.assert_allclose(zt[7], pr["g"], rtol=1e-14)
    np.testing.assert_allclose(zt[8], pr["az"], rtol=1e-14)
    np.testing.assert_allclose(zt[9], pr["bzpml"], rtol=1e-14)


def test_primitives_match_oracle(gpu_lib, oracle_mod):
    p = small_params()
    g, o = make_pair(p, oracle_mod, gpu_lib)
    rng = np.random.default_rng(7)
    v = rng.standard_normal((p.nz, p.ny, p.nx))
    assert rel_l2(g.ddx(v), o.ddx(v)) < 1e-13
    assert rel_l2(g.ddy(v), o.ddy(v)) < 1e-13
    for bc in (0, 1):
        assert rel_l2(g.ddz(v, bc), o.ddz(v, bc)) < 1e-13, bc
    for bc in (2, 3):
        init = np.zeros_like(v)
        init[0 if bc == 2 else -1] = rng.standard_normal((p.ny, p.nx))
        assert rel_l2(g.ddz(v, bc, init), o.ddz(v, bc, init)) < 1e-13, bc
    r = rng.standard_normal(v.shape)
    assert rel_l2(g.damp(v, r), o.damp(v, r)) < 1e-13


@pytest.mark.parametrize("nsteps", [1, 5, 31])
def test_forward_steps_match_oracle_3d(gpu_lib, oracle_mod, nsteps):
    p = small_params()
    g, o = make_pair(p, oracle_mod, gpu_lib)
    a0, pml0 = random_state(p)
    g.set_state(a0, pml0)
    o.set_state(a0, pml0)
    plane = gaussian_plane(p)
    series = oracle_mod.forward_source(p, 200) * 1e3
    g.set_source_series(plane, series)
    o.set_source(1, plane[None].copy(), series)
    g.step(nsteps)
    o.step(nsteps)
    ag, pg = g.state()
    ao, _, po = o.state()
    for f in range(6):
        assert rel_l2(ag[f], ao[f]) < TOL64, (f, rel_l2(ag[f], ao[f]))
    assert rel_l2(pg, po) < TOL64


def test_forward_steps_match_oracle_2d(gpu_lib, oracle_mod):
    p = small_params_2d()
    g, o = make_pair(p, oracle_mod, gpu_lib)
    a0, pml0 = random_state(p)
    # ddz(p, gradp_z, 2) (physics2d.f90:1029) reuses the previous gradp_z(:,:,1)
    # as its Neumann value; it stays exactly zero in every state the reference
    # can reach, which requires psip(:,:,1) = 0 (a non-zero psip there grows
    # by stretch(1) per call in the reference itself).
    pml0[1, 0] = 0.0
    g.set_state(a0, pml0)
    o.set_state(a0, pml0)
    plane = gaussian_plane(p)
    series = oracle_mod.forward_source(p, 200) * 1e3
    g.set_source_series(plane, series)
    o.set_source(1, plane[None].copy(), series)
    for n in (1, 29, 2):      # crosses the mod(time+1, 30) horizontal filter
        g.step(n)
        o.step(n)
        ag, _ = g.state()
        ao, _, _ = o.state()
        for f in (0, 2, 3, 5):
            assert rel_l2(ag[f], ao[f]) < TOL64, (n, f, rel_l2(ag[f], ao[f]))


def test_adjoint_lagrange_source_matches_oracle(gpu_lib, oracle_mod):
    p = small_params(compute_forward=False, compute_adjoint=True)
    g, o = make_pair(p, oracle_mod, gpu_lib)
    rng = np.random.default_rng(3)
    L = 12
    planes = rng.standard_normal((L, p.ny, p.nx)) * 1e-4
    g.set_source_lagrange(planes)
    o.set_source(2, planes)
    g.step(40)
    o.step(40)
    ag, _ = g.state()
    ao, _, _ = o.state()
    for f in range(6):
        assert rel_l2(ag[f], ao[f]) < TOL64, (f, rel_l2(ag[f], ao[f]))


def test_surface_records_match_oracle(gpu_lib, oracle_mod):
    p = small_params()
    g, o = make_pair(p, oracle_mod, gpu_lib)
    plane = gaussian_plane(p)
    series = oracle_mod.forward_source(p, 400) * 1e3
    g.set_source_series(plane, series)
    o.set_source(1, plane[None].copy(), series)
    g.record_surface(10)
    ref = []
    info = o.info()
    orad = int(info["o_rad"])
    for i in range(46):
        o.step(1)
        if i % 15 == 0:
            ao, _, _ = o.state()
            ref.append(ao[5, orad - 1].copy())
    g.step(46)
    rec = g.records()
    assert rec.shape == (4, p.ny, p.nx)
    for r in range(4):
        assert rel_l2(rec[r], ref[r]) < TOL64 or np.abs(ref[r]).max() == 0


def test_fp32_seismograms_within_tolerance(gpu_lib, oracle_mod):
    from sparc_gb300.solver import Solver
    p64 = small_params()
    p32 = p64.replace(precision="f32")
    tab = table_for(p64)
    g64, g32 = Solver(p64, tab), Solver(p32, tab)
    plane = gaussian_plane(p64)
    series = oracle_mod.forward_source(p64, 1000) * 1e3
    for g in (g64, g32):
        g.set_source_series(plane, series)
        g.record_surface(64)
        g.step(300)
    r64, r32 = g64.records(), g32.records()
    assert r64.shape == r32.shape and r64.shape[0] == 20
    assert np.abs(r64).max() > 0
    assert rel_l2(r32, r64) < TOL32, rel_l2(r32, r64)


def test_batched_sources_equal_single(gpu_lib, oracle_mod):
    from sparc_gb300.solver import Solver
    p = small_params(nsrc=3)
    tab = table_for(p)
    gb = Solver(p, tab)
    series = oracle_mod.forward_source(p, 200) * 1e3
    planes = [gaussian_plane(p, x0_mm=x0) for x0 in (-5.0, 0.0, 7.0)]
    for s, pl in enumerate(planes):
        gb.set_source_series(pl, series * (s + 1), slot=s)
    gb.step(20)
    for s, pl in enumerate(planes):
        g1 = Solver(small_params(), tab)
        g1.set_source_series(pl, series * (s + 1))
        g1.step(20)
        a1, _ = g1.state()
        ab, _ = gb.state(slot=s)
        np.testing.assert_array_equal(ab, a1)


def test_checkpoint_roundtrip_and_corruption(gpu_lib, oracle_mod, tmp_path):
    from sparc_gb300 import native
    from sparc_gb300.solver import Solver
    p = small_params()
    tab = table_for(p)
    g = Solver(p, tab)
    a0, pml0 = random_state(p)
    g.set_state(a0, pml0)
    g.step(3)
    path = str(tmp_path / "ck.bin")
    g.checkpoint(path)
    g.step(4)
    a_ref, _ = g.state()
    g2 = Solver(p, tab)
    g2.restore(path)
    assert g2.time == 3
    g2.step(4)
    a2, _ = g2.state()
    np.testing.assert_array_equal(a2, a_ref)
    raw = bytearray(open(path, "rb").read())
    raw[-5] ^= 0xFF
    bad = str(tmp_path / "bad.bin")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(native.SparcError) as e:
        g2.restore(bad)
    assert e.value.status == native.SPARC_EIO
    open(bad, "wb").write(bytes(raw[:100]))
    with pytest.raises(native.SparcError) as e:
        g2.restore(bad)
    assert e.value.status == native.SPARC_EIO


def test_nan_detection(gpu_lib):
    from sparc_gb300 import native
    from sparc_gb300.solver import Solver
    p = small_params()
    g = Solver(p, table_for(p))
    a, _ = random_state(p)
    a[3, 10, 5, 5] = np.nan
    g.set_state(a)
    with pytest.raises(native.SparcError) as e:
        g.sync(check_finite=True)
    assert e.value.status == native.SPARC_ENAN


def test_kernel_accumulation_matches_oracle(gpu_lib, oracle_mod):
    from sparc_gb300.solver import Solver
    p = small_params()
    tab = table_for(p)
    pa = p.replace(compute_forward=False, compute_adjoint=True)
    fwd, adj = Solver(p, tab), Solver(pa, tab)
    o = oracle_mod.Oracle(p, tab)
    a1, _ = random_state(p, seed=11)
    a2, _ = random_state(p, seed=12)
    fwd.set_state(a1)
    fwd.step(1)                      # scr now holds the stage-5 RHS ('acc')
    adj.set_state(a2)
    adj.step(1)
    fwd.snapshot(0, 1)
    adj.kernel_reset()
    adj.kernel_accumulate(fwd, 0)
    kc, kr, hs = adj.kernels()
    # oracle on the GPU's own physical snapshot fields
    af, _ = fwd.state()
    acc = np.stack([fwd.field(9), fwd.field(10), fwd.field(11)])
    aa, _ = adj.state()
    fwd_f = np.concatenate([af[0:3], acc])
    adj_f = aa[3:6]
    o.kernel_reset()
    graw = tab[:, 4] * o.info()["rsun"] / 1e12
    o.kernel_accumulate(fwd_f, adj_f, graw)
    ref = o.kernel_finish(int(fwd.info()["steps"]))
    assert rel_l2(hs, ref[2]) < 1e-12
    assert rel_l2(kc, ref[0]) < 1e-10
    assert rel_l2(kr, ref[1]) < 1e-10


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_kernel_accumulation_source_groups(gpu_lib, prec):
    """Snapshots and accumulation run over groups of 8 sources: with 10 sources
    (groups 8 + 2, two snapshot slots) every slot's kernels equal those of the
    same source run alone, bitwise."""
    from sparc_gb300.solver import Solver
    p = small_params(nx=16, ny=16, precision=prec)
    tab = table_for(p)
    S = 10
    states = [random_state(p, seed=100 + s) for s in range(2 * S)]

    def run(nsrc, slots):
        pf = p.replace(nsrc=nsrc)
        pa = pf.replace(compute_forward=False, compute_adjoint=True)
        fwd, adj = Solver(pf, tab), Solver(pa, tab)
        for i, s in enumerate(slots):
            fwd.set_state(states[s][0], slot=i)
            adj.set_state(states[S + s][0], slot=i)
        adj.kernel_reset()
        for k in range(2):
            fwd.step(2)
            adj.step(2)
            fwd.snapshot(k, 2)
            adj.kernel_accumulate(fwd, k)
        return [adj.kernels(slot=i) for i in range(nsrc)]

    many = run(S, list(range(S)))
    for s in (0, 7, 8, 9):
        alone = run(1, [s])[0]
        for q in range(3):
            assert np.array_equal(many[s][q], alone[q]), (s, q)


def _velocity_state(p, seed):
    a, pml = random_state(p, seed=seed)
    a[0] = 0.0          # rest density and pressure: the velocity form's natural seed
    a[4] = 0.0
    a[5] = 0.0
    return a, pml


@pytest.mark.parametrize("nsteps,mode", [(1, 1), (5, 1), (31, 1), (31, 2)])
def test_velocity_form_matches_oracle(gpu_lib, oracle_mod, nsteps, mode):
    """Option 2 (MP_QUIET_PML_3D, pml.f90:12-76): rho, v_x, v_y, v_z, p with the
    9-plane source_dep forcing, the PML accounting and the damping."""
    p = small_params(option=2)
    g, o = make_pair(p, oracle_mod, gpu_lib)
    a0, pml0 = _velocity_state(p, 21)
    g.set_state(a0, pml0)
    o.set_state(a0, pml0)
    if mode == 1:
        plane = gaussian_plane(p)
        series = oracle_mod.forward_source(p, 200) * 1e3
        g.set_source_series(plane, series)
        o.set_source(1, plane[None].copy(), series)
    else:
        planes = np.random.default_rng(5).standard_normal((12, p.ny, p.nx)) * 1e-4
        g.set_source_lagrange(planes)
        o.set_source(2, planes, None)
    g.step(nsteps)
    o.step(nsteps)
    ag, pg = g.state()
    ao, _, po = o.state()
    for f in range(5):
        assert rel_l2(ag[f], ao[f]) < TOL64, (f, rel_l2(ag[f], ao[f]))
    assert np.abs(ag[5]).max() == 0
    assert rel_l2(pg, po) < TOL64


def test_velocity_form_fp32_and_records(gpu_lib, oracle_mod):
    """FP32 (per-stage kernels) against FP64, and the surface records of the
    velocity form come from v_z (its fourth field)."""
    from sparc_gb300.solver import Solver
    p64 = small_params(option=2)
    tab = table_for(p64)
    a0, pml0 = _velocity_state(p64, 22)
    plane = gaussian_plane(p64)
    series = oracle_mod.forward_source(p64, 200) * 1e3
    out = []
    for p in (p64, p64.replace(precision="f32")):
        g = Solver(p, tab)
        g.set_state(a0, pml0)
        g.set_source_series(plane, series)
        g.record_surface(4)
        g.step(31)
        a, _ = g.state()
        out.append((a, g.records(), g.info()["o_rad"]))
    (a64, r64, orad), (a32, r32, _) = out
    for f in range(5):
        assert rel_l2(a32[f], a64[f]) < 2e-5, (f, rel_l2(a32[f], a64[f]))
    assert r64.shape[0] >= 3
    assert rel_l2(r64[2], a64[3, orad - 1]) < 1e-14      # record 2 = v_z after the step at time 30
    assert rel_l2(r32[2], r64[2]) < 1e-4


def test_gpu_matches_committed_golden_fixtures(gpu_lib):
    import os
    import sys
    from sparc_gb300.solver import Solver
    sys.path.insert(0, os.path.join(os.path.dirname(__file__)))
    from golden.make_golden import golden_inputs, golden_params, golden_params_2d
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))
    p = golden_params()
    s = Solver(p, table_for(p))
    v = np.random.default_rng(43).standard_normal((p.nz, p.ny, p.nx))
    assert rel_l2(s.ddx(v), g["ddx"]) < 1e-13
    assert rel_l2(s.ddy(v), g["ddy"]) < 1e-13
    assert rel_l2(s.ddz(v, 1), g["ddz_bc1"]) < 1e-13
    assert rel_l2(s.damp(v, np.zeros_like(v)), g["damp"]) < 1e-13
    a, pml, plane, series = golden_inputs(p, 44)
    s.set_state(a, pml)
    s.set_source_series(plane, series)
    s.step(3)
    st, pm = s.state()
    for f in range(6):
        assert rel_l2(st[f], g["step3_a"][f]) < TOL64, f
    assert rel_l2(pm, g["step3_pml"]) < TOL64
    p2 = golden_params_2d()
    s2 = Solver(p2, table_for(p2))
    a, pml, plane, series = golden_inputs(p2, 45)
    s2.set_state(a, pml)
    s2.set_source_series(plane, series)
    s2.step(31)
    st2, _ = s2.state()
    for f in (0, 2, 3, 5):
        assert rel_l2(st2[f], g["step31_2d_a"][f]) < TOL64, f
    from golden.make_golden import golden_params_vel
    pv = golden_params_vel()
    sv = Solver(pv, table_for(pv))
    a, pml, plane, series = golden_inputs(pv, 47)
    sv.set_state(a, pml)
    sv.set_source_series(plane, series)
    sv.step(31)
    stv, pmv = sv.state()
    for f in range(5):
        assert rel_l2(stv[f], g["step31_vel_a"][f]) < TOL64, f
    assert np.abs(stv[5]).max() == 0
    assert rel_l2(pmv, g["step31_vel_pml"]) < TOL64


@pytest.mark.parametrize("two_d,nz", [(False, 48), (True, 48), (False, 161), (False, 196), (True, 300)])
def test_fused_fp32_step_matches_fp64(gpu_lib, oracle_mod, two_d, nz):
    """The fused FP32 step (state on chip, scan-based tridiagonal solves)
    against the FP64 path: FP32 round-off only.  nz 48: one warp per pencil;
    161, 196, 300: two warps, padding rows, and (196) the rows nz-2 and nz-1
    owned by different threads."""
    from sparc_gb300.background import polytrope_table
    from sparc_gb300.solver import Solver
    if two_d:
        p64 = small_params_2d(nz=nz)
    else:
        p64 = small_params(nz=nz) if nz < 100 else small_params(nx=16, ny=16, nz=nz)
    p32 = p64.replace(precision="f32")
    tab = table_for(p64) if nz < 100 else polytrope_table(nz, z_bot_mm=-25.0, z_top_mm=1.2)
    a0, pml0 = random_state(p64)
    pml0[1, 0] = 0.0
    plane = gaussian_plane(p64)
    series = oracle_mod.forward_source(p64, 200) * 1e3
    out = []
    for p, per_stage in ((p64, False), (p32, False), (p32, True)):
        if per_stage:
            os.environ["SPARC_FP32_PER_STAGE"] = "1"
        try:
            g = Solver(p, tab)
        finally:
            os.environ.pop("SPARC_FP32_PER_STAGE", None)
        g.set_state(a0, pml0)
        g.set_source_series(plane, series)
        g.step(37)                     # crosses the horizontal-filter steps
        a, pml = g.state()
        out.append((a, pml, np.stack([g.field(f) for f in range(6, 12)])))
    (a64, pml64, s64), (a32, pml32, s32), (ap, pmlp, sp) = out
    fields = (0, 2, 3, 5) if two_d else range(6)
    # FP32 round-off only: within a fixed bound, or within twice the error of
    # the per-stage FP32 kernels (same arithmetic, no fusion) on this case
    for f in fields:
        ea, es = rel_l2(a32[f], a64[f]), rel_l2(s32[f], s64[f])
        assert ea < max(2e-5, 2 * rel_l2(ap[f], a64[f])), (f, ea)
        assert es < max(2e-4, 2 * rel_l2(sp[f], s64[f])), (f, es)
    ep = rel_l2(pml32, pml64)
    assert ep < max(2e-5, 2 * rel_l2(pmlp, pml64)), ep


def test_fused_fp32_lagrange_source_matches_fp64(gpu_lib):
    from sparc_gb300.solver import Solver
    p64 = small_params(compute_forward=False, compute_adjoint=True)
    tab = table_for(p64)
    planes = np.random.default_rng(3).standard_normal((12, p64.ny, p64.nx)) * 1e-4
    res = []
    for p in (p64, p64.replace(precision="f32", nsrc=2)):
        g = Solver(p, tab)
        for s in range(p.nsrc):
            g.set_source_lagrange(planes * (s + 1), slot=s)
        g.step(40)
        res.append([g.state(slot=s)[0] for s in range(p.nsrc)])
    for f in range(6):
        assert rel_l2(res[1][0][f], res[0][0][f]) < 2e-5, f
        assert rel_l2(res[1][1][f], 2 * res[0][0][f]) < 2e-5, f


@pytest.mark.parametrize("nx,nz,prec", [(64, 32, "f64"), (256, 24, "f64"), (64, 32, "f32")])
def test_register_fft_sizes_round_trip_and_steps(gpu_lib, oracle_mod, nx, nz, prec):
    """The R x R register transforms (horizontal sizes 64 and 256) between
    physical planes and the spectral state: set_state -> get_state returns the
    fields, and three steps with the damping match the oracle."""
    p = small_params(nx=nx, ny=nx, nz=nz, npmlbot=4, npmltop=4, xlength=200e8, ylength=200e8, precision=prec)
    g, o = make_pair(p, oracle_mod, gpu_lib)
    a0, pml0 = random_state(p, seed=9)
    g.set_state(a0, pml0)
    a1, p1 = g.state()
    tol_rt = 1e-14 if prec == "f64" else 1e-6
    assert rel_l2(a1, a0) < tol_rt and rel_l2(p1, pml0) < tol_rt
    o.set_state(a0, pml0)
    plane = gaussian_plane(p, sigma_mm=8.0)
    series = oracle_mod.forward_source(p, 200) * 1e3
    g.set_source_series(plane, series)
    o.set_source(1, plane[None].copy(), series)
    g.step(3)
    o.step(3)
    ag, pg = g.state()
    ao, _, po = o.state()
    tol = TOL64 if prec == "f64" else 1e-4
    for f in range(6):
        assert rel_l2(ag[f], ao[f]) < tol, (f, rel_l2(ag[f], ao[f]))
    assert rel_l2(pg, po) < tol


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
@pytest.mark.parametrize("two_d", [False, True])
def test_fp64_chunked_stage_matches_oracle(gpu_lib, oracle_mod, lanes, two_d):
    """The FP64 stage with each z-pencil on 1, 2, 4 or 8 lanes (chunked
    elimination, carries composed across the lanes) against the oracle over
    31 steps (crossing the horizontal filter), <= 1e-10 per field; the
    chunkings agree with each other to round-off."""
    from sparc_gb300.solver import Solver
    p = small_params_2d() if two_d else small_params()
    tab = table_for(p)
    a0, pml0 = random_state(p)
    pml0[1, 0] = 0.0
    plane = gaussian_plane(p)
    series = oracle_mod.forward_source(p, 200) * 1e3
    os.environ["SPARC_STAGE_LANES"] = str(lanes)
    try:
        g = Solver(p, tab)
    finally:
        os.environ.pop("SPARC_STAGE_LANES", None)
    o = oracle_mod.Oracle(p, tab)
    for s in (g, o):
        s.set_state(a0, pml0)
    g.set_source_series(plane, series)
    o.set_source(1, plane[None].copy(), series)
    g.step(31)
    o.step(31)
    ag, pg = g.state()
    ao, _, po = o.state()
    for f in ((0, 2, 3, 5) if two_d else range(6)):
        assert rel_l2(ag[f], ao[f]) < TOL64, (lanes, f, rel_l2(ag[f], ao[f]))
    assert rel_l2(pg, po) < TOL64
