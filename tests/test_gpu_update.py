"""The model update of an inversion iteration on the GPU (grad.py:152-301)
against the numpy restatement in the oracle: gradients, steepest-descent and
conjugate-gradient directions and the line-search test models, FP64 <= 1e-11
relative L2."""
import os

import numpy as np
import pytest

from cases import rel_l2, small_params, small_params_2d, table_for

pytestmark = pytest.mark.gpu


def _solver(p):
    from sparc_gb300.solver import Solver
    return Solver(p, table_for(p))


def _fields(p, seed):
    rng = np.random.default_rng(seed)
    shape = (p.nz, p.ny, p.nx)
    kc = rng.standard_normal(shape)
    kpsi = rng.standard_normal(shape)
    hess = np.abs(rng.standard_normal(shape)) * np.linspace(0.01, 1.0, p.nz)[:, None, None]
    rho_z = np.exp(np.linspace(2.0, -3.0, p.nz))
    return kc, kpsi, hess, rho_z


@pytest.mark.parametrize("three_d", [False, True])
def test_gradient_matches_oracle(gpu_lib, three_d):
    from oracle import model_update as U
    p = small_params(nx=32, ny=16, nz=40) if three_d else small_params_2d(nx=64, nz=48)
    s = _solver(p)
    kc, kpsi, hess, rho_z = _fields(p, 7)
    g_c, g_psi = s.gradient(kc, kpsi, hess, rho_z)
    o_c, o_psi = U.gradient(kc, kpsi, hess, rho_z)
    assert rel_l2(g_c, o_c) < 1e-11, rel_l2(g_c, o_c)
    assert rel_l2(g_psi, o_psi) < 1e-11, rel_l2(g_psi, o_psi)
    # grad.py's smooth filter leaves planes 4 and nz-1 at zero and keeps plane 0
    assert not g_c[4].any() and not g_c[-1].any()
    # antisymmetric along x after the z smoothing too
    assert np.abs(g_psi + g_psi[..., ::-1]).max() <= 1e-14 * np.abs(g_psi).max()
    # one gradient alone
    only_c, none_psi = s.gradient(kc, None, hess, rho_z)
    assert none_psi is None and np.array_equal(only_c, g_c)


def test_update_directions_and_test_models(gpu_lib):
    from oracle import model_update as U
    p = small_params_2d(nx=64, nz=48)
    s = _solver(p)
    kc, kpsi, hess, rho_z = _fields(p, 11)
    g_c, g_psi = U.gradient(kc, kpsi, hess, rho_z)
    rng = np.random.default_rng(3)
    model = rng.standard_normal(g_psi.shape) * 1e3
    # steepest descent
    uc, up, tp, con = s.update_models(g_c, g_psi, model)
    assert con == 0.0 and np.array_equal(uc, g_c) and np.array_equal(up, g_psi)
    ref = U.test_models(model, g_psi)
    assert tp.shape == ref.shape and rel_l2(tp, ref) < 1e-14
    # a step large enough that the offsets from the model are resolved
    _, _, tp, _ = s.update_models(g_c, g_psi, model, eps=0.05, nmodels=3)
    ref = U.test_models(model, g_psi, eps=0.05, n=3)
    for i in range(3):
        assert rel_l2(tp[i] - model, ref[i] - model) < 1e-11
    # conjugate gradient from a previous iteration's gradient and update
    lg = g_psi * 0.7 + rng.standard_normal(g_psi.shape) * 0.1 * np.abs(g_psi).max()
    luc = rng.standard_normal(g_c.shape)
    lup = rng.standard_normal(g_psi.shape)
    uc, up, tp, con = s.update_models(g_c, g_psi, model, last=(lg, luc, lup))
    o_c, o_psi, o_con = U.update_direction(g_c, g_psi, (lg, luc, lup))
    assert o_con > 0 and abs(con - o_con) <= 1e-12 * o_con
    assert rel_l2(uc, o_c) < 1e-12 and rel_l2(up, o_psi) < 1e-12
    assert rel_l2(tp, U.test_models(model, o_psi, eps=1e-7, n=5)) < 1e-14
    # a negative coefficient is floored at zero: steepest descent again
    uc, up, tp, con = s.update_models(g_c, g_psi, model, last=(2.0 * g_psi, luc, lup), nmodels=0)
    assert con == 0.0 and np.array_equal(up, g_psi) and tp.shape[0] == 0


def test_model_update_files(gpu_lib, tmp_path):
    """grad.py's file flow: per-source kernels in kernel/, a steepest-descent
    iteration, then a conjugate-gradient one reading the first one's
    gradient and update; values against the oracle, names as grad.py's."""
    from oracle import model_update as U
    from sparc_gb300 import inversion, io
    p = small_params_2d(nx=64, nz=48)
    s = _solver(p)
    rng = np.random.default_rng(21)
    d = tmp_path
    (d / "kernel").mkdir()
    (d / "update").mkdir()
    ks = []
    for src in (1, 2):
        kc, kpsi, hess, _ = _fields(p, 100 + src)
        hess = hess * rng.choice([-1.0, 1.0], size=hess.shape)      # grad.py sums |hessian|
        for name, a in (("kernel_c", kc), ("kernel_vectorpsi", kpsi), ("hessian", hess)):
            io.write_fits(str(d / "kernel" / f"{name}_{src:02d}.fits"), a[:, 0, :])   # 2-D files
        ks.append((kc, kpsi, hess))
    rho_z = np.exp(np.linspace(2.0, -3.0, p.nz))
    model = rng.standard_normal((p.nz, 1, p.nx)) * 1e2
    io.write_fits(str(d / "update" / "model_vectorpsi_01.fits"), model)
    r1 = inversion.model_update(s, str(d), 2, 2, rho_z)
    kc = ks[0][0] + ks[1][0]
    kpsi = ks[0][1] + ks[1][1]
    hs = np.abs(ks[0][2]) + np.abs(ks[1][2])
    o_c, o_psi = U.gradient(kc, kpsi, hs, rho_z)
    assert rel_l2(r1.gradient_c, o_c) < 1e-11 and rel_l2(r1.gradient_psi, o_psi) < 1e-11
    names = sorted(os.path.basename(f) for f in r1.files)
    assert names == sorted(["gradient_c_01.fits", "gradient_vectorpsi_01.fits", "update_c_01.fits",
                            "update_vectorpsi_01.fits"] + [f"test_vectorpsi_{i}.fits" for i in range(1, 6)])
    t3 = io.read_fits(str(d / "update" / "test_vectorpsi_3.fits"))
    assert rel_l2(t3, U.test_models(model, o_psi)[2]) < 1e-14
    # next iteration: new kernels, conjugate gradient against iteration 2's files
    for src in (1, 2):
        for name in ("kernel_c", "kernel_vectorpsi"):
            path = str(d / "kernel" / f"{name}_{src:02d}.fits")
            io.write_fits(path, io.read_fits(path) * 0.5 + rng.standard_normal((p.nz, p.nx)) * 0.2)
    model2 = model + 0.01
    io.write_fits(str(d / "update" / "model_vectorpsi_02.fits"), model2)
    io.write_fits(str(d / "update" / "model_c_02.fits"), model2 * 2.0)
    r2 = inversion.model_update(s, str(d), 3, 2, rho_z, conjugate_gradient=True)
    kc2, kpsi2, hs2 = inversion.sum_kernels(str(d), 2)
    g_c2, g_psi2 = U.gradient(kc2, kpsi2, hs2, rho_z)
    o_uc, o_up, o_con = U.update_direction(g_c2, g_psi2, (r1.gradient_psi, r1.update_c, r1.update_psi))
    assert abs(r2.con - o_con) <= 1e-10 * max(abs(o_con), 1e-30)
    assert rel_l2(r2.update_c, o_uc) < 1e-11 and rel_l2(r2.update_psi, o_up) < 1e-11
    assert os.path.exists(d / "update" / "update_psi_02.fits")            # grad.py:230's name
    assert np.array_equal(io.read_fits(str(d / "update" / "test_c_1.fits")), model2 * 2.0)
