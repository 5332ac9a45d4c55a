"""Source terms (host FP64 set-up, DETERMINE_STATUS / FORWARD_SOURCE roles).

* ``gabor_series``   -- FORWARD_SOURCE (driver.f90:1046-1071), the reference's
                        forward wavelet, sampled every time step.
* ``ricker_series``  -- Ricker wavelet used by the benchmark workloads.
* ``master_pixel_plane`` -- the 2-D forward source shape of DETERMINE_STATUS
                        (driver.f90:618-624): Gaussian x sinc around the
                        master-pixel x position.
* ``gaussian_plane`` -- 2-D Gaussian around a point.
* ``adjoint_planes`` -- vr(:,:,1..L) of an adjoint run: time-reversed,
                        windowed residual seismograms placed at receiver pixels,
                        sampled every cadforcing seconds.
"""
from __future__ import annotations

import numpy as np

from .params import SparcParams, r4


def gabor_series(p: SparcParams, nt: int) -> np.ndarray:
    pi = r4(3.14159265358979)
    ts = r4(p.timestep)
    nup, nuw = r4(p.nupeak), r4(p.nuwidth)
    k = np.arange(1, nt + 1)
    tt = (k.astype(np.float32) - np.float32(1.0)).astype(np.float64) * ts
    arg = tt - 0.5 / nup
    f = np.cos(2.0 * pi * nup * tt) * np.exp(-2.0 * (arg * arg) * (nuw * nuw))
    f[np.abs(f) < float(np.float32(0.00001))] = 0.0
    return f * float(np.float32(1.0e-5))


def ricker_series(p: SparcParams, nt: int, f0: float = 3.0e-3, amp: float = 1.0e-5,
                  delay: float | None = None) -> np.ndarray:
    t = np.arange(nt) * p.timestep
    t0 = 1.2 / f0 if delay is None else delay
    a = (np.pi * f0 * (t - t0)) ** 2
    return amp * (1.0 - 2.0 * a) * np.exp(-a)


def gaussian_plane(p: SparcParams, sigma_mm: float = 1.0, x0_mm: float = 0.0, y0_mm: float = 0.0) -> np.ndarray:
    x = (np.arange(p.nx) / p.nx - 0.5) * p.xlength / 1e8 - x0_mm
    if p.ny == 1:
        return np.exp(-x ** 2 / (2 * sigma_mm ** 2))[None, :]
    y = (np.arange(p.ny) / p.ny - 0.5) * p.ylength / 1e8 - y0_mm
    X, Y = np.meshgrid(x, y)
    return np.exp(-(X ** 2 + Y ** 2) / (2 * sigma_mm ** 2))


def master_pixel_plane(p: SparcParams, xloc_mm: float) -> np.ndarray:
    """vr(:,:,1) of DETERMINE_STATUS (driver.f90:618-624), x in Mm."""
    pi = r4(3.14159265358979)
    e8 = float(np.float32(1e-8))
    x = np.arange(p.nx) / p.nx
    dx = (x[1] - x[0]) * r4(p.xlength) * e8
    xdist = (x - 0.5) * r4(p.xlength) * e8 - xloc_mm
    with np.errstate(invalid="ignore", divide="ignore"):
        sincx = np.sin(r4(0.43) * pi * xdist) / (r4(0.43) * pi * xdist)
    sincx[np.argmin(np.abs(xdist))] = 1.0
    row = np.exp(-xdist ** 2 / (400.0 * dx ** 2)) * sincx
    return np.repeat(row[None, :], p.ny, axis=0)


def receiver_pixels(p: SparcParams, n: int = 8, radius_mm: float = 10.0, x0_mm: float = 0.0,
                    y0_mm: float = 0.0):
    """Pixel indices (iy, ix) of n receivers on a ring."""
    ang = 2 * np.pi * np.arange(n) / n
    xs = x0_mm + radius_mm * np.cos(ang)
    ys = y0_mm + radius_mm * np.sin(ang)
    ix = np.round((xs * 1e8 / p.xlength + 0.5) * p.nx).astype(int) % p.nx
    iy = np.round((ys * 1e8 / p.ylength + 0.5) * p.ny).astype(int) % max(p.ny, 1)
    return list(zip(iy.tolist(), ix.tolist()))


def adjoint_planes(p: SparcParams, residual: np.ndarray, pixels, window: np.ndarray | None = None) -> np.ndarray:
    """vr(:,:,1..L) for an adjoint run: residual[r, k] sampled at the output
    cadence (k = 0..L-1), time-reversed, windowed, placed at pixel r."""
    residual = np.asarray(residual, dtype=np.float64)
    R, L = residual.shape
    w = np.ones(L) if window is None else np.asarray(window, dtype=np.float64)
    planes = np.zeros((L, p.ny, p.nx))
    rev = (residual * w)[:, ::-1]
    for r, (iy, ix) in enumerate(pixels):
        planes[:, iy, ix] += rev[r]
    return planes


def hann_window(n: int, lo: int, hi: int) -> np.ndarray:
    w = np.zeros(n)
    hi = min(hi, n)
    if hi > lo:
        w[lo:hi] = np.hanning(hi - lo)
    return w
