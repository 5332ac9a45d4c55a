"""The magnetohydrostatic flux tube (background.mhs_flux_tube_background) on
the CPU, with the z derivative of the FP64 oracle: a zero field gives back
the table's column exactly, the tube is held (p, rho > 0), its field is
divergence-free and carries the same flux at every height, and the
force-balance residual grad p - F - rho g (the table's own hydrostatic
residual taken out) is small against the Lorentz force."""
import numpy as np
import pytest

from cases import small_params


@pytest.fixture(scope="module")
def case():
    from oracle import oracle as O
    from sparc_gb300.background import polytrope_table
    O.build()
    p = small_params(nx=64, ny=64, nz=96, xlength=100e8, ylength=100e8, npmlbot=8, npmltop=0, option=10)
    tab = polytrope_table(p.nz, z_bot_mm=-25.0, z_top_mm=0.0)
    o = O.Oracle(p.replace(option=4), tab)
    return p, tab, o


def test_zero_field_is_the_quiet_column(case):
    from sparc_gb300.background import mhs_flux_tube_background
    p, tab, o = case
    (rho, c, pres, bx, by, bz), info = mhs_flux_tube_background(p, tab, o.ddz, b0=0.0)
    assert not bx.any() and not by.any() and not bz.any()
    np.testing.assert_array_equal(pres, np.broadcast_to(tab[:, 3][:, None, None], pres.shape))
    np.testing.assert_allclose(rho, np.broadcast_to(tab[:, 2][:, None, None], rho.shape), rtol=1e-14)
    np.testing.assert_allclose(c, np.broadcast_to(tab[:, 1][:, None, None], c.shape), rtol=1e-14)


def test_tube_is_held_and_balanced(case):
    from sparc_gb300.background import _dxdy, mhs_flux_tube_background
    p, tab, o = case
    (rho, c, pres, bx, by, bz), info = mhs_flux_tube_background(p, tab, o.ddz)
    assert info["min_p_ratio"] > 0.5 and info["min_rho_ratio"] > 0.9
    assert 1900.0 < info["b_axis_max_G"] <= 2000.0 + 1e-9
    # balance: horizontal to the discretisation of a 3 Mm tube on 1.6 Mm cells,
    # vertical to round-off (the density is solved for)
    assert info["residual_z_max_rel"] < 1e-10
    assert info["residual_h_max_rel"] < 2e-2 and info["residual_l2_rel"] < 2e-2
    # flux through every plane (B_z integrates to Phi = pi b0 R0^2) and div B
    dA = (p.xlength / p.nx) * (p.ylength / p.ny)
    flux = bz.sum(axis=(1, 2)) * dA
    np.testing.assert_allclose(flux, np.pi * 2000.0 * (3e8) ** 2, rtol=1e-10)
    dx, dy = _dxdy(p.nx, p.ny, p.xlength, p.ylength)
    z = (tab[:, 0] - 1.0) * 69598946770.0
    dzi = o.ddz(np.ascontiguousarray(np.broadcast_to(z[:, None, None], bz.shape)), 1)[:, :1, :1]
    divb = dx(bx) + dy(by) + o.ddz(bz, 1) / dzi
    assert np.abs(divb).max() * 3e8 / 2000.0 < 1e-3
    # far from the tube the column is the table's
    np.testing.assert_allclose(pres[:, 0, 0], tab[:, 3], rtol=1e-12)
    np.testing.assert_allclose(rho[:, 0, 0], tab[:, 2], rtol=1e-12)
    # a tube the column cannot hold is refused
    with pytest.raises(ValueError):
        mhs_flux_tube_background(p, tab, o.ddz, b0=2000.0, z_min_mm=0.0, d_mm=0.5)
