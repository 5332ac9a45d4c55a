"""Model update of an inversion iteration with the reference's files
(grad.py:150-301): read the per-source kernels, form the preconditioned and
smoothed gradients on the GPU, choose the update direction and write the
line-search test models.

Files, all under ``datadir`` and in the (nz, ny, nx) FITS layout grad.py
writes through its ``fitswrite`` (NAXIS1 = nx):
  kernel/kernel_c_XX.fits, kernel/kernel_vectorpsi_XX.fits,
  kernel/hessian_XX.fits                      (read, XX = 01..num_src)
  update/model_vectorpsi_II.fits, update/model_c_II.fits (optional)
  update/gradient_c_II.fits, update/gradient_vectorpsi_II.fits
  update/update_c_II.fits, update/update_vectorpsi_II.fits
  update/test_c_i.fits (when model_c exists), update/test_vectorpsi_i.fits
with II = iterno - 1 (grad.py:111 iterminus).  Like grad.py, the
conjugate-gradient branch writes its vectorpsi update as update_psi_II.fits
(grad.py:230) while it reads the previous one as update_vectorpsi (grad.py:
215); both names are kept so that the files match the reference's.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from . import io
from .solver import Solver


def _two(m: int) -> str:
    return str(int(m)).zfill(2)


def _read(path: str) -> np.ndarray:
    a = io.read_fits(path)
    return a[:, None, :] if a.ndim == 2 else a          # 2-D files: (nz, nx) -> (nz, 1, nx)


@dataclasses.dataclass
class UpdateResult:
    gradient_c: np.ndarray
    gradient_psi: np.ndarray
    update_c: np.ndarray
    update_psi: np.ndarray
    test_psi: np.ndarray        # (nmodels, nz, ny, nx)
    con: float
    files: list


def sum_kernels(datadir: str, num_src: int):
    """grad.py:157-164: sum of kernel_c, sum of kernel_vectorpsi and sum of
    |hessian| over sources 1..num_src."""
    kc = kpsi = hess = None
    for src in range(1, num_src + 1):
        d = os.path.join(datadir, "kernel")
        a = _read(os.path.join(d, f"kernel_c_{_two(src)}.fits"))
        b = _read(os.path.join(d, f"kernel_vectorpsi_{_two(src)}.fits"))
        h = np.abs(_read(os.path.join(d, f"hessian_{_two(src)}.fits")))
        kc = a if kc is None else kc + a
        kpsi = b if kpsi is None else kpsi + b
        hess = h if hess is None else hess + h
    return kc, kpsi, hess


def model_update(solver: Solver, datadir: str, iterno: int, num_src: int, rho_z: np.ndarray,
                 conjugate_gradient: bool = False, eps: float = 1e-7, nmodels: int = 5) -> UpdateResult:
    """grad.py:150-301 with the smoothing, reductions and test models on the
    GPU.  rho_z is the density column of the background (the third column of
    the polytrope file, grad.py:167).  Steepest descent unless
    conjugate_gradient and iterno > 1 (grad.py:133-134, 191, 206)."""
    upd = os.path.join(datadir, "update")
    os.makedirs(upd, exist_ok=True)
    kc, kpsi, hess = sum_kernels(datadir, num_src)
    g_c, g_psi = solver.gradient(kc, kpsi, hess, rho_z)
    files = []

    def put(name, arr):
        path = os.path.join(upd, name)
        io.write_fits(path, arr)
        files.append(path)

    i1, i2 = _two(iterno - 1), _two(iterno - 2)
    put(f"gradient_c_{i1}.fits", g_c)
    put(f"gradient_vectorpsi_{i1}.fits", g_psi)
    model_c_path = os.path.join(upd, f"model_c_{i1}.fits")
    model_c = _read(model_c_path) if os.path.exists(model_c_path) else None
    model_psi = _read(os.path.join(upd, f"model_vectorpsi_{i1}.fits"))
    cg = conjugate_gradient and iterno > 1
    last = None
    if cg:
        last = (_read(os.path.join(upd, f"gradient_vectorpsi_{i2}.fits")),
                _read(os.path.join(upd, f"update_c_{i2}.fits")),
                _read(os.path.join(upd, f"update_vectorpsi_{i2}.fits")))
    u_c, u_psi, test_psi, con = solver.update_models(g_c, g_psi, model_psi, last=last, eps=eps, nmodels=nmodels)
    put(f"update_c_{i1}.fits", u_c)
    put(f"update_psi_{i1}.fits" if cg else f"update_vectorpsi_{i1}.fits", u_psi)
    for i in range(1, nmodels + 1):
        if model_c is not None:
            put(f"test_c_{i}.fits", model_c)          # c is not updated (grad.py:285-293)
        put(f"test_vectorpsi_{i}.fits", test_psi[i - 1])
    return UpdateResult(g_c, g_psi, u_c, u_psi, test_psi, con, files)


def _count_master_pixels(datadir: str) -> int:
    with open(os.path.join(datadir, "master.pixels")) as f:
        return sum(1 for _ in f)


def total_misfit(datadir: str, iterno: int | None = None) -> float:
    """misfit.py: the sum of the third column of update/misfit_II over the
    first nmasterpixels rows (one row per source).  iterno None takes the
    last iteration, as the script does from the count of misfit files."""
    upd = os.path.join(datadir, "update")
    if iterno is None:
        n = len([f for f in os.listdir(upd) if f.startswith("misfit_") and "all" not in f])
        if n == 0:
            raise FileNotFoundError("no misfit files in " + upd)
        iterno = n - 1
    col = np.loadtxt(os.path.join(upd, f"misfit_{_two(iterno)}"), usecols=[2], ndmin=1)
    return float(np.sum(col[:_count_master_pixels(datadir)]))


def linesearch_misfits(datadir: str, iterno: int | None = None, n_linesearches: int = 5) -> list:
    """lsmisfit.py: per test model, the sum of the third column of
    update/linesearch_II over that model's block of nmasterpixels rows."""
    upd = os.path.join(datadir, "update")
    if iterno is None:
        n = len([f for f in os.listdir(upd) if f.startswith("linesearch_") and "all" not in f])
        if n == 0:
            raise FileNotFoundError("no linesearch files in " + upd)
        iterno = n - 1
    col = np.loadtxt(os.path.join(upd, f"linesearch_{_two(iterno)}"), usecols=[2], ndmin=1)
    npix = _count_master_pixels(datadir)
    return [float(np.sum(col[i * npix:(i + 1) * npix])) for i in range(n_linesearches)]
