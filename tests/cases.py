"""Small seeded cases shared by the CPU and GPU tests (the oracle finishes
them in seconds)."""
import numpy as np

from sparc_gb300.background import polytrope_table
from sparc_gb300.params import SparcParams


def small_params(**kw) -> SparcParams:
    base = dict(nx=32, ny=32, nz=48, xlength=50e8, ylength=50e8, npmlbot=6, npmltop=6,
                excitdep=-1.5e7, obsheight=2e7, solartime=1.0)
    base.update(kw)
    return SparcParams(**base)


def small_params_2d(**kw) -> SparcParams:
    base = dict(nx=64, ny=1, nz=48, xlength=100e8, ylength=100e8, npmlbot=6, npmltop=6,
                option=17, excitdep=-1.5e7, obsheight=2e7, solartime=1.0)
    base.update(kw)
    return SparcParams(**base)


def table_for(p: SparcParams) -> np.ndarray:
    return polytrope_table(p.nz, z_bot_mm=-6.0, z_top_mm=1.0)


def random_state(p: SparcParams, seed: int = 1234, scale: float = 1e-3):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((6, p.nz, p.ny, p.nx)) * scale
    if p.option == 17:
        a[1] = 0.0
        a[4] = 0.0
    pml = rng.standard_normal((2, p.nzpml, p.ny, p.nx)) * scale * 1e-2
    return a, pml


def gaussian_plane(p: SparcParams, sigma_mm: float = 1.0, x0_mm: float = 0.0, y0_mm: float = 0.0):
    x = (np.arange(p.nx) / p.nx - 0.5) * p.xlength / 1e8 - x0_mm
    if p.ny == 1:
        return np.exp(-x ** 2 / (2 * sigma_mm ** 2))[None, :]
    y = (np.arange(p.ny) / p.ny - 0.5) * p.ylength / 1e8 - y0_mm
    X, Y = np.meshgrid(x, y)
    return np.exp(-(X ** 2 + Y ** 2) / (2 * sigma_mm ** 2))


def rel_l2(a, b) -> float:
    d = np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel())
    n = np.linalg.norm(np.asarray(b).ravel())
    return float(d / n) if n > 0 else float(d)


def smooth_state(p: SparcParams, seed: int = 1234, scale: float = 1e-3, nf: int = 6, npv: int = 2):
    """A seeded state with the spectrum of a wave field rather than white
    noise: horizontal wavenumbers weighted by exp(-(k/k0)^2), k0 = n/8, and a
    Gaussian smoothing over 3 levels in z; PML auxiliaries at 1 % of the
    fields.  The reachable-state rules of the 2-D forms are applied (no y
    components, psi_p zero on the bottom plane)."""
    rng = np.random.default_rng(seed)

    def shaped(shape):
        v = rng.standard_normal(shape)
        ax = [a for a in (-1, -2) if shape[a] > 1]
        f = np.fft.fftn(v, axes=ax)
        for a in ax:
            n = shape[a]
            k = np.fft.fftfreq(n) * n
            w = np.exp(-(k / (n / 8.0)) ** 2)
            sh = [1] * len(shape)
            sh[a] = n
            f = f * w.reshape(sh)
        v = np.fft.ifftn(f, axes=ax).real
        from scipy.ndimage import gaussian_filter1d
        v = gaussian_filter1d(v, 3.0, axis=len(shape) - 3, mode="nearest")
        return v / np.abs(v).max()

    a = shaped((nf, p.nz, p.ny, p.nx)) * scale
    pml = shaped((npv, p.nzpml, p.ny, p.nx)) * scale * 1e-2
    if p.ny == 1:
        a[1] = 0.0
        a[4] = 0.0
        pml[1, 0] = 0.0
        if npv == 6:
            pml[3] = 0.0
            pml[5] = 0.0
    return a, pml
