"""CPU restatement (numpy, FP64) of the model update of grad.py:158-301:
Hessian preconditioning of the summed kernels, the x smoothing (filterx), the
z filters (filterz 'smooth' and 'gaussian'), antisymmetrize, the
steepest-descent and conjugate-gradient directions and the line-search test
models.

Test infrastructure: only the tests import this module, as the checker of
the CUDA path.  grad.py holds arrays as (nx, ny, nz); here they are
(nz, ny, nx), the layout of the library, with the axes mapped accordingly.
"""
from __future__ import annotations

import numpy as np


def filterx(kern: np.ndarray) -> np.ndarray:
    """filterx (grad.py:47-61): the spectrum along x times the rfft of a
    Gaussian of 4 pixels (not normalised)."""
    nx = kern.shape[-1]
    x = np.fft.fftfreq(nx) * nx
    g = np.exp(-x ** 2.0 / (2.0 * 4 ** 2.0))
    filtx = np.fft.rfft(g)
    return np.fft.irfft(np.fft.rfft(kern, axis=-1) * filtx, n=nx, axis=-1).real


def filterz_smooth(arr: np.ndarray) -> np.ndarray:
    """filterz(algo='smooth') (grad.py:63-96): the 11-point filter on planes
    5..nz-6, 3-point averages on planes 1-3 and nz-5..nz-2, and (the temp
    array starts at zero) planes 4 and nz-1 set to zero; plane 0 kept."""
    co = [0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125]
    nz = arr.shape[0]
    temp = np.zeros_like(arr)
    for k in range(5, nz - 5):
        temp[k] = (co[0] * arr[k] + 0.5 * co[1] * (arr[k - 1] + arr[k + 1]) + 0.5 * co[2] * (arr[k - 2] + arr[k + 2])
                   + 0.5 * co[3] * (arr[k - 3] + arr[k + 3]) + 0.5 * co[4] * (arr[k - 4] + arr[k + 4])
                   + 0.5 * co[5] * (arr[k - 5] + arr[k + 5]))
    temp[nz - 5:nz - 1] = 0.5 * (arr[nz - 4:] + arr[nz - 6:nz - 2])
    temp[1:4] = 0.5 * (arr[:3] + arr[2:5])
    out = arr.copy()
    out[1:nz] = temp[1:nz]
    return out


def gaussian_z(arr: np.ndarray, sigma: float) -> np.ndarray:
    """filterz(algo='gaussian') (grad.py:106-107): scipy's gaussian_filter1d
    along z, restated: weights exp(-x^2 / 2 sigma^2) for |x| <= int(4 sigma +
    0.5), normalised to sum 1, with the half-sample symmetric boundary
    ('reflect': d c b a | a b c d | d c b a)."""
    r = int(4.0 * sigma + 0.5)
    x = np.arange(-r, r + 1)
    w = np.exp(-0.5 / (sigma * sigma) * x ** 2)
    w = w / w.sum()
    nz = arr.shape[0]
    idx = np.arange(-r, nz + r)
    period = 2 * nz
    m = np.mod(idx, period)
    src = np.where(m < nz, m, period - 1 - m)
    ext = arr[src]
    out = np.zeros_like(arr)
    for j in range(2 * r + 1):
        out = out + w[j] * ext[j:j + nz]
    return out


def antisymmetrize(arr: np.ndarray) -> np.ndarray:
    """antisymmetrize (grad.py:109): 0.5 (a - a reversed along x)."""
    return 0.5 * (arr - arr[..., ::-1])


def gradient(kc_sum: np.ndarray, kpsi_sum: np.ndarray, hess_sum: np.ndarray, rho_z: np.ndarray):
    """grad.py:159-197: (gradient_c, gradient_vectorpsi) from the kernels
    summed over sources (hess_sum = sum |hessian|), rho_z the density column
    of the background (polytrope column 3)."""
    hess = hess_sum * rho_z[:, None, None]
    hess = hess / hess.max()
    hess = np.where(hess < 5e-3, 5e-3, hess)
    kern = kc_sum / hess
    kern = filterx(kern)
    g_c = filterz_smooth(kern)
    kern = kpsi_sum / hess
    kern = filterx(kern)
    kern = antisymmetrize(kern)
    g_psi = gaussian_z(kern, 2.0)
    return g_c, g_psi


def update_direction(g_c, g_psi, prev=None):
    """grad.py:205-244: steepest descent (prev None), or the conjugate
    gradient with prev = (last gradient_psi, last update_c, last update_psi):
    con = sum g (g - g_last) / sum g_last^2, floored at 0."""
    if prev is None:
        return g_c, g_psi, 0.0
    lg_psi, lu_c, lu_psi = prev
    con = np.sum(g_psi * (g_psi - lg_psi))
    den = np.sum(lg_psi ** 2.0)
    con = con / den
    if con < 0:
        con = 0.0
    return g_c + con * lu_c, g_psi + con * lu_psi, con


def test_models(model_psi: np.ndarray, update_psi: np.ndarray, eps: float = 1e-7, n: int = 5) -> np.ndarray:
    """grad.py:282-301: test_vectorpsi_i = model + eps i rms(model) update /
    max|update|, i = 1..n."""
    u = update_psi / np.abs(update_psi).max()
    scale = np.sqrt(np.sum(model_psi ** 2) / np.prod(model_psi.shape))
    return np.stack([model_psi + eps * i * scale * u for i in range(1, n + 1)])
