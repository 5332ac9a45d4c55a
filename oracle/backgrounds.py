"""CPU restatement (numpy, FP64) of the magnetohydrostatic background
generator code_python/tubex.py:27-141, in the script's own layout: arrays
(nx, nz) with x leading.

Test infrastructure: only the tests import this module, as the checker of
the library's generator.  The z derivative is DBYD2 with ibc = 1 divided by
the same derivative of z (tubex.py:14-17,33-36), taken from the oracle's C++
restatement of the compact scheme (`ddz` of an Oracle context on the same
table: its stretch cancels in the ratio).  The script's fftcalculus module
(differentiate / integrate with a period) is not in the reference; its
operations are restated as the FFT derivative and the FFT antiderivative
with the mean term dropped.
"""
from __future__ import annotations

import numpy as np

RSUN = 695.9894      # tubex.py:9
GRAV = 2.775e4       # tubex.py:44
CONVERT = 1e8        # tubex.py:45


def fft_differentiate(a: np.ndarray, period: float) -> np.ndarray:
    """d/dx along axis 0 (tubex.py:12): multiply the spectrum by i k."""
    n = a.shape[0]
    f = np.fft.fft(a, axis=0)
    k = 2.0 * np.pi * np.fft.fftfreq(n, d=period / n)
    if n % 2 == 0:
        k[n // 2] = 0.0                       # the Nyquist term of a real field has no odd part
    return np.real(np.fft.ifft(f * (1j * k)[:, None], axis=0))


def fft_integrate(a: np.ndarray, period: float) -> np.ndarray:
    """Periodic antiderivative along axis 0 (tubex.py:72): divide the
    spectrum by i k, with the k = 0 (and Nyquist) terms set to zero."""
    n = a.shape[0]
    f = np.fft.fft(a, axis=0)
    k = 2.0 * np.pi * np.fft.fftfreq(n, d=period / n)
    q = np.zeros(n, dtype=complex)
    nz = k != 0
    q[nz] = 1.0 / (1j * k[nz])
    if n % 2 == 0:
        q[n // 2] = 0.0
    return np.real(np.fft.ifft(f * q[:, None], axis=0))


def tubex(table: np.ndarray, oracle, nx: int = 256, lx: float = 400.0, a0: float = 5000.0, decay_x: float = 10.0,
          decay_z: float = 10.0, decay_z_start: float = 12.0, zero_b: bool = True) -> dict:
    """tubex.py:27-141.  `oracle`: an Oracle context of shape (nz, 1, nx) on
    `table`.  Returns the script's arrays transposed to (nz, 1, nx)."""
    z = (table[:, 0] - 1.0) * RSUN
    nz = z.shape[0]
    x = np.linspace(-lx / 2, lx / 2, num=nx, endpoint=False)

    def dbyd2_ratio(arr_xz):                    # dbyd2(arr) / dbyd2(z), both ibc = 1
        zz = np.tile(z[:, None, None], (1, 1, nx))
        num = oracle.ddz(np.ascontiguousarray(arr_xz.T[:, None, :]), 1)
        den = oracle.ddz(zz, 1)
        return (num / den)[:, 0, :].T

    p0, rho0, c2 = table[:, 3], table[:, 2], table[:, 1] ** 2
    fx = -(x / decay_x) / (1 + (x / decay_x) ** 4)
    dfx = -decay_x ** 3 * (decay_x ** 4 - 3 * x ** 4) / (decay_x ** 4 + x ** 4) ** 2
    gz = np.exp(z / decay_z)
    dgz = 1 / decay_z * gz
    bx = -a0 * np.atleast_2d(fx).T * dgz
    bz = a0 * np.atleast_2d(dfx).T * gz
    a_true = a0 * np.atleast_2d(fx).T * gz
    a_start = a0 * np.atleast_2d(fx).T * np.exp(z / decay_z_start)
    bx_start = -dbyd2_ratio(a_start)
    bz_start = fft_differentiate(a_start, lx)
    if zero_b:
        bx = np.zeros_like(bx); bz = np.zeros_like(bz)
        bx_start = np.zeros_like(bx); bz_start = np.zeros_like(bx)
        a_start = np.zeros_like(a_start); a_true = np.zeros_like(a_true)
    force = dbyd2_ratio(bx) - fft_differentiate(bz, lx)
    hz = bx * force
    hx = bz * force
    p = fft_integrate(hx, lx)
    p -= p[0] - p0
    dzp = dbyd2_ratio(p)
    rho = -(hz + dzp) / (GRAV * CONVERT)
    rho -= rho[0] - rho0
    c = np.sqrt(c2 * rho0 / p0 * p / rho)
    t = lambda a: np.ascontiguousarray(a.T[:, None, :])
    s4 = np.sqrt(4 * np.pi)
    return {"true": {"bx": t(bx), "bz": t(bz), "psi": t(a_true * s4 / RSUN)},
            "start": {"bx": t(bx_start), "bz": t(bz_start), "psi": t(a_start * s4 / RSUN)},
            "p": t(p), "rho": t(rho), "c": t(c),
            "negative": bool((p / p0 - 1).min() < -1 or (rho / rho0 - 1).min() < -1)}
