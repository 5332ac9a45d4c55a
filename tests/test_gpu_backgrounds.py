"""The magnetohydrostatic background generator of code_python/tubex.py on
the library (z derivatives from the FP64 GPU primitive) against the numpy
restatement in the oracle, FP64 <= 1e-10 relative L2; the FITS files it
writes under true/ and start/."""
import os

import numpy as np
import pytest

from cases import rel_l2, small_params_2d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("a0,zero_b", [(20.0, False), (100.0, False), (5000.0, True)])
def test_vector_potential_background_matches_oracle(gpu_lib, a0, zero_b):
    from oracle import backgrounds as B
    from oracle.oracle import Oracle
    from sparc_gb300.background import polytrope_table, vector_potential_background
    from sparc_gb300.solver import Solver
    nz, nx = 120, 128
    tab = polytrope_table(nz, z_bot_mm=-25.0, z_top_mm=1.2)
    p = small_params_2d(nx=nx, nz=nz, xlength=400e8, ylength=400e8)
    with Solver(p, tab) as s:
        got = vector_potential_background(s, tab, a0=a0, zero_b=zero_b)
    ref = B.tubex(tab, Oracle(p, tab), nx=nx, a0=a0, zero_b=zero_b)
    for key in ("p", "rho", "c"):
        assert rel_l2(got[key], ref[key]) < 1e-10, (key, rel_l2(got[key], ref[key]))
    for m in ("true", "start"):
        for f in ("bx", "bz", "psi"):
            if zero_b:
                assert not got[m][f].any()
            else:
                assert rel_l2(got[m][f], ref[m][f]) < 1e-10, (m, f, rel_l2(got[m][f], ref[m][f]))


def test_vector_potential_models_files(gpu_lib, tmp_path):
    from sparc_gb300 import io
    from sparc_gb300.background import (polytrope_table, vector_potential_background,
                                        write_vector_potential_models)
    from sparc_gb300.solver import Solver
    nz, nx = 120, 128
    tab = polytrope_table(nz, z_bot_mm=-25.0, z_top_mm=1.2)
    p = small_params_2d(nx=nx, nz=nz, xlength=400e8, ylength=400e8)
    with Solver(p, tab) as s:
        m = vector_potential_background(s, tab, a0=20.0, zero_b=False)
    files = write_vector_potential_models(str(tmp_path), m)
    names = sorted(os.path.relpath(f, tmp_path) for f in files)
    assert names == sorted(["true/B_z2D.fits", "true/B_x2D.fits", "true/true_vectorpsi.fits",
                            "start/model_vectorpsi_ls00.fits", "start/model_c_ls00.fits"]
                           + [f"{d}/{n}2D.fits" for d in ("true", "start") for n in ("pressure", "density",
                                                                                  "soundspeed")])
    bz = io.read_fits(str(tmp_path / "true" / "B_z2D.fits"))
    assert bz.shape == (nz, nx) and np.allclose(bz, m["true"]["bz"][:, 0, :] * np.sqrt(4 * np.pi), rtol=0, atol=0)
    # the 2-D MHD run takes these as its background (psi in G R_sun)
    p18 = small_params_2d(nx=nx, nz=nz, xlength=400e8, ylength=400e8, option=18)
    with Solver(p18, tab) as s18:
        s18.set_mhd2d_background(m["rho"], m["c"], m["p"], io.read_fits(str(tmp_path / "true" / "true_vectorpsi.fits")))


def test_mhs_flux_tube_with_gpu_derivatives_matches_oracle(gpu_lib):
    """The magnetohydrostatic tube built with the library's FP64 z derivative
    equals the same construction with the oracle's, <= 1e-10."""
    from oracle.oracle import Oracle
    from cases import small_params
    from sparc_gb300.background import mhs_flux_tube_background, polytrope_table
    from sparc_gb300.solver import Solver
    p = small_params(nx=64, ny=64, nz=96, xlength=100e8, ylength=100e8, npmlbot=8, npmltop=0, option=10)
    tab = polytrope_table(p.nz, z_bot_mm=-25.0, z_top_mm=0.0)
    with Solver(p, tab) as s:
        got, gi = mhs_flux_tube_background(p, tab, s.ddz)
    ref, ri = mhs_flux_tube_background(p, tab, Oracle(p.replace(option=4), tab).ddz)
    for g, r in zip(got, ref):
        assert rel_l2(g, r) < 1e-10, rel_l2(g, r)
    assert gi["min_p_ratio"] > 0.5 and gi["residual_l2_rel"] < 2e-2
