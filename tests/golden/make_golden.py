"""Generates tests/golden/oracle_golden.npz: outputs of the CPU oracle on small
seeded cases (compact derivative for every boundary code, spectral
derivatives, damping, three 3-D time steps with a forward source, thirty-one
2-D time steps, thirty-one velocity-form steps, five MHD steps on a flux
tube, thirty-one MHD velocity-form steps on a flux tube, thirty-one 2-D MHD
steps on a flux sheet, one kernel accumulation).  Regenerate with
    python tests/golden/make_golden.py
The GPU parity tests compare the CUDA path against these fixtures as well as
against the live oracle."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from cases import small_params, small_params_2d, table_for  # noqa: E402
from oracle import oracle as O  # noqa: E402


def golden_params():
    return small_params(nx=16, ny=16, nz=32, npmlbot=4, npmltop=4)


def golden_params_2d():
    return small_params_2d(nx=32, nz=32, npmlbot=4, npmltop=4)


def golden_params_vel():
    """Velocity form (option 2): fields rho, v_x, v_y, v_z, p."""
    return small_params(nx=16, ny=16, nz=32, npmlbot=4, npmltop=4, option=2)


def golden_params_mhd():
    """MHD displacement form (option 10): bottom PML only, flux-tube background."""
    return small_params(nx=16, ny=16, nz=32, npmlbot=4, npmltop=0, option=10)


def golden_mhd_background(p):
    from sparc_gb300.background import flux_tube_background
    return flux_tube_background(p, table_for(p), b_surf=800.0, r_surf_mm=8.0)


def golden_params_mhd8():
    """MHD velocity form (option 8): PML at both ends, flux-tube background."""
    return small_params(nx=16, ny=16, nz=32, npmlbot=4, npmltop=4, option=8)


def golden_params_mhd2d():
    """2-D MHD displacement form (option 18): PML at both ends, flux sheet."""
    return small_params_2d(nx=32, nz=32, npmlbot=4, npmltop=4, option=18)


def golden_mhd2d_background(p):
    from sparc_gb300.background import flux_sheet_background
    return flux_sheet_background(p, table_for(p), b_surf=300.0, w_mm=10.0)


def golden_inputs(p, seed):
    rng = np.random.default_rng(seed)
    if p.option == 8:
        # rho, v, p, b: a velocity perturbation at rest density, pressure
        # and field; the induction drives b
        a = rng.standard_normal((8, p.nz, p.ny, p.nx)) * 1e-3
        a[0] = 0.0
        a[4:] = 0.0
        pml = rng.standard_normal((6, p.nzpml, p.ny, p.nx)) * 1e-5
        pml[1, 0] = 0.0
        X, Y = np.meshgrid(*(2 * [(np.arange(p.nx) / p.nx - 0.5) * p.xlength / 1e8]))
        plane = np.exp(-(X ** 2 + Y ** 2) / 2.0)
        return a, pml, plane, O.forward_source(p, 200) * 1e3
    a = rng.standard_normal((6, p.nz, p.ny, p.nx)) * 1e-3
    if p.ny == 1:
        a[1] = 0.0
        a[4] = 0.0
    if p.option == 2:
        # five fields in the velocity form; a velocity perturbation at rest
        # density and pressure (a random pressure would be scaled by 1/rho0)
        a[0] = 0.0
        a[4] = 0.0
        a[5] = 0.0
    pml = rng.standard_normal((6 if p.option in (10, 18) else 2, p.nzpml, p.ny, p.nx)) * 1e-5
    pml[1, 0] = 0.0
    if p.option == 18:
        pml[3] = 0.0                   # psi_dzby, psi_induction_by: not in the 2-D form
        pml[5] = 0.0
    x = (np.arange(p.nx) / p.nx - 0.5) * p.xlength / 1e8
    if p.ny == 1:
        plane = np.exp(-x ** 2 / 2.0)[None, :]
    else:
        X, Y = np.meshgrid(x, x)
        plane = np.exp(-(X ** 2 + Y ** 2) / 2.0)
    series = O.forward_source(p, 200) * 1e3
    return a, pml, plane, series


def compute():
    O.build()
    out = {}
    rng = np.random.default_rng(42)
    b = rng.standard_normal((24, 5))
    for bc in (0, 1, 2, 3):
        init = np.zeros_like(b)
        init[0 if bc == 2 else -1] = rng.standard_normal(5) if bc in (2, 3) else 0.0
        out[f"dbyd2_bc{bc}"] = O.dbyd2(b, bc, init)
    p = golden_params()
    tab = table_for(p)
    o = O.Oracle(p, tab)
    v = np.random.default_rng(43).standard_normal((p.nz, p.ny, p.nx))
    out["ddx"] = o.ddx(v)
    out["ddy"] = o.ddy(v)
    out["ddz_bc1"] = o.ddz(v, 1)
    out["damp"] = o.damp(v, np.zeros_like(v))
    a, pml, plane, series = golden_inputs(p, 44)
    o.set_state(a, pml)
    o.set_source(1, plane[None].copy(), series)
    o.step(3)
    st, scr, pm = o.state()
    out["step3_a"] = st
    out["step3_pml"] = pm
    p2 = golden_params_2d()
    o2 = O.Oracle(p2, table_for(p2))
    a, pml, plane, series = golden_inputs(p2, 45)
    o2.set_state(a, pml)
    o2.set_source(1, plane[None].copy(), series)
    o2.step(31)
    out["step31_2d_a"] = o2.state()[0]
    pv = golden_params_vel()
    ov = O.Oracle(pv, table_for(pv))
    a, pml, plane, series = golden_inputs(pv, 47)
    ov.set_state(a, pml)
    ov.set_source(1, plane[None].copy(), series)
    ov.step(31)
    st, _, pm = ov.state()
    out["step31_vel_a"] = st
    out["step31_vel_pml"] = pm
    pm_ = golden_params_mhd()
    om = O.Oracle(pm_, table_for(pm_))
    om.set_mhd(*golden_mhd_background(pm_))
    a, pml, plane, series = golden_inputs(pm_, 48)
    a *= 1e-3                          # a small displacement on the strong-field background
    om.set_state(a, pml)
    om.set_source(1, plane[None].copy(), series)
    om.step(5)
    st, _, pm = om.state()
    out["step5_mhd_a"] = st
    out["step5_mhd_pml"] = pm
    # MHD velocity form: 31 steps cover the horizontal filter at time 30
    p8 = golden_params_mhd8()
    o8 = O.Oracle(p8, table_for(p8))
    o8.set_mhd(*golden_mhd_background(p8))
    a, pml, plane, series = golden_inputs(p8, 50)
    o8.set_state(a * 1e-3, pml)
    o8.set_source(1, plane[None].copy(), series)
    o8.step(31)
    st, _, pm = o8.state()
    out["step31_mhd8_a"] = st
    out["step31_mhd8_pml"] = pm
    # 2-D MHD: 31 steps cover the horizontal filter at mod(time+1, 30) = 0
    p18 = golden_params_mhd2d()
    o18 = O.Oracle(p18, table_for(p18))
    o18.set_mhd2d(*golden_mhd2d_background(p18))
    a, pml, plane, series = golden_inputs(p18, 49)
    o18.set_state(a * 1e-3, pml)
    o18.set_source(1, plane[None].copy(), series)
    o18.step(31)
    st, _, pm = o18.state()
    out["step31_mhd2d_a"] = st
    out["step31_mhd2d_pml"] = pm
    # one kernel accumulation on seeded fields
    rng = np.random.default_rng(46)
    fwd = rng.standard_normal((6, p.nz, p.ny, p.nx))
    adj = rng.standard_normal((3, p.nz, p.ny, p.nx))
    o.kernel_reset()
    graw = tab[:, 4] * o.info()["rsun"] / 1e12
    o.kernel_accumulate(fwd, adj, graw)
    out["kernels"] = o.kernel_finish(15)
    return out


if __name__ == "__main__":
    res = compute()
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **res)
    print({k: v.shape for k, v in res.items()})
