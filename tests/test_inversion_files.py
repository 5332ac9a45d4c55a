"""Host logic of the model-update file flow (grad.py:150-301): file names,
the kernel sums, the choice of direction and the test_c copies, with the
device calls stood in by the oracle so that it runs without a GPU."""
import os

import numpy as np

from cases import small_params_2d


class OracleSolver:
    """Solver.gradient / Solver.update_models restated by the oracle."""

    def __init__(self, p):
        self.shape = (p.nz, p.ny, p.nx)

    def gradient(self, kc, kpsi, hess, rho_z):
        from oracle import model_update as U
        return U.gradient(kc, kpsi, hess, rho_z)

    def update_models(self, g_c, g_psi, model, last=None, eps=1e-7, nmodels=5):
        from oracle import model_update as U
        u_c, u_psi, con = U.update_direction(g_c, g_psi, last)
        return u_c, u_psi, U.test_models(model, u_psi, eps=eps, n=nmodels), con


def test_model_update_file_flow(tmp_path):
    from sparc_gb300 import inversion, io
    p = small_params_2d(nx=32, nz=24)
    rng = np.random.default_rng(4)
    (tmp_path / "kernel").mkdir()
    for src in (1, 2, 3):
        for name in ("kernel_c", "kernel_vectorpsi", "hessian"):
            io.write_fits(str(tmp_path / "kernel" / f"{name}_{src:02d}.fits"), rng.standard_normal((p.nz, p.nx)))
    kc, kpsi, hess = inversion.sum_kernels(str(tmp_path), 3)
    assert kc.shape == (p.nz, 1, p.nx) and (hess >= 0).all()
    direct = sum(np.abs(io.read_fits(str(tmp_path / "kernel" / f"hessian_{s:02d}.fits"))) for s in (1, 2, 3))
    assert np.allclose(hess[:, 0, :], direct, rtol=0, atol=1e-15)
    (tmp_path / "update").mkdir()
    io.write_fits(str(tmp_path / "update" / "model_vectorpsi_00.fits"), rng.standard_normal((p.nz, 1, p.nx)))
    s = OracleSolver(p)
    rho = np.linspace(1.0, 0.1, p.nz)
    r = inversion.model_update(s, str(tmp_path), 1, 3, rho, conjugate_gradient=True)     # iteration 1: steepest
    assert r.con == 0.0
    got = sorted(os.listdir(tmp_path / "update"))
    want = sorted(["model_vectorpsi_00.fits", "gradient_c_00.fits", "gradient_vectorpsi_00.fits", "update_c_00.fits",
                   "update_vectorpsi_00.fits"] + [f"test_vectorpsi_{i}.fits" for i in range(1, 6)])
    assert got == want
    io.write_fits(str(tmp_path / "update" / "model_vectorpsi_01.fits"), rng.standard_normal((p.nz, 1, p.nx)))
    io.write_fits(str(tmp_path / "update" / "model_c_01.fits"), np.ones((p.nz, 1, p.nx)))
    r2 = inversion.model_update(s, str(tmp_path), 2, 3, rho, conjugate_gradient=True, nmodels=2)
    names = set(os.listdir(tmp_path / "update"))
    assert {"update_psi_01.fits", "update_c_01.fits", "test_c_1.fits", "test_c_2.fits"} <= names
    assert "update_vectorpsi_01.fits" not in names                 # the CG branch's own name (grad.py:230)
    assert r2.test_psi.shape == (2, p.nz, 1, p.nx)


def test_vector_potential_background_host_logic():
    """The library's tubex.py generator with the oracle standing in for the
    GPU z derivative, against the oracle's own restatement (the host logic:
    layout, pinning rows, the FFT calculus, units)."""
    from oracle import backgrounds as B
    from oracle.oracle import Oracle
    from sparc_gb300.background import polytrope_table, vector_potential_background
    nz, nx = 96, 64
    tab = polytrope_table(nz, z_bot_mm=-25.0, z_top_mm=1.2)
    o = Oracle(small_params_2d(nx=nx, nz=nz, xlength=400e8, ylength=400e8), tab)
    o.shape = (nz, 1, nx)
    got = vector_potential_background(o, tab, a0=30.0, zero_b=False)
    ref = B.tubex(tab, o, nx=nx, a0=30.0, zero_b=False)
    for key in ("p", "rho", "c"):
        assert np.allclose(got[key], ref[key], rtol=1e-10, atol=0), key
    for m in ("true", "start"):
        for f in ("bx", "bz", "psi"):
            d = np.abs(got[m][f] - ref[m][f]).max()
            assert d <= 1e-10 * np.abs(ref[m][f]).max(), (m, f, d)


def test_misfit_sums(tmp_path):
    """misfit.py / lsmisfit.py over the files the pipeline writes
    (io.write_misfit lines concatenated per source and per test model)."""
    from sparc_gb300 import inversion, io
    (tmp_path / "update").mkdir()
    (tmp_path / "master.pixels").write_text("-5.0\n3.0\n")
    vals = [1.5, 2.25]
    with open(tmp_path / "update" / "misfit_00", "w") as f:
        for k, v in enumerate(vals):
            tmpf = tmp_path / "m"
            io.write_misfit(str(tmpf), k + 1, 10, v)
            f.write(tmpf.read_text())
    (tmp_path / "update" / "misfit_all_00").write_text("ignored\n")
    assert abs(inversion.total_misfit(str(tmp_path)) - 3.75) < 1e-15
    with open(tmp_path / "update" / "linesearch_00", "w") as f:
        for ls in range(5):
            for k in range(2):
                tmpf = tmp_path / "m"
                io.write_misfit(str(tmpf), k + 1, 10, 0.5 * (ls + 1) + k)
                f.write(tmpf.read_text())
    got = inversion.linesearch_misfits(str(tmp_path))
    assert np.allclose(got, [2 * 0.5 * (ls + 1) + 1 for ls in range(5)])
