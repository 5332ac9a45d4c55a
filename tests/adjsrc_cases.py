"""Seeded synthetic surface seismograms for the adjoint-source tests: a
random field shaped by the ridge filters in (k, nu), and observed data as the
same field delayed by a known time."""
import numpy as np


def ridge_field(nx, nt, xlength, outputcad, seed=0):
    from oracle import adjoint_source as A
    rng = np.random.default_rng(seed)
    shape = A.fmode_filter(nx, nt, xlength, outputcad) + A.pmode_filter(nx, nt, xlength, outputcad) + 0.05
    spec = shape * (rng.standard_normal((nt, nx)) + 1j * rng.standard_normal((nt, nx)))
    return np.fft.ifft2(spec).real * 1e3


def delayed(field, shift_s, outputcad):
    nt = field.shape[0]
    nu = np.fft.fftfreq(nt, d=outputcad)
    return np.fft.ifft(np.fft.fft(field, axis=0) * np.exp(-2j * np.pi * nu * shift_s)[:, None], axis=0).real


# geometry of the tests: 128 pixels over 200 Mm, 180 outputs every 30 s, the
# source at x = -5 Mm; ridge ranges that keep every window inside the record
CASE = dict(nx=128, nt=180, xlength=200e8, outputcad=30.0, x00=-5.0,
            ridges={0: (10.0, 30.0, 20.0), 1: (15.0, 40.0, 15.0), 2: (15.0, 40.0, 15.0)},
            bands={0: (2.0, 5.0), 1: (2.5, 5.5)})
