"""Background stratification (FP64 set-up; never on the time-stepping path).

The reference reads a ``polytrope`` table (initialize.f90:728-774): one row per
z-level, columns r/R_sun, c [cm/s], rho [g/cc], p [dyn/cm^2], g [cm/s^2],
Gamma_1.  Its shipped table is an adiabatic Gamma = 5/3 polytrope with constant
gravity on a grid uniform in sound speed (dz proportional to c).

``polytrope_table`` generates tables of the same law for any nz and depth range.
Above the photosphere the adiabatic profile would reach T = 0 within a few
hundred km, so the generator continues it as an isothermal layer (constant c,
exponential rho and p) on the uniform spacing of the top polytropic cell; the
box can then reach +1.2 Mm.
"""
from __future__ import annotations

import numpy as np

RSUN_CM = 69598946770.0      # initialize.f90:38 (value as written)
G_SURF = 2.775841e4          # constant gravity of the shipped table
R_GAS = 8.314462618e7        # erg / (mol K)


def polytrope_table(nz: int, z_bot_mm: float = -25.0, z_top_mm: float = 1.2,
                    t_surf: float = 5800.0, gamma: float = 5.0 / 3.0, mu: float = 1.0,
                    rho_surf: float = 2.78e-7, g: float = G_SURF) -> np.ndarray:
    """(nz, 6) table, bottom row first, in the reference's column order."""
    gm1 = gamma - 1.0
    c2_0 = gamma * R_GAS * t_surf / mu            # c^2 at z = 0
    zs = c2_0 / (gm1 * g)                          # polytrope surface height (cm)
    zb = z_bot_mm * 1e8
    zt = z_top_mm * 1e8
    c0 = np.sqrt(c2_0)
    cb = np.sqrt(gm1 * g * (zs - zb))

    def z_of_c(c):
        return zs - c * c / (gm1 * g)

    # choose the split (rows below z=0 uniform in c, rows above uniform in z)
    best = None
    for n_above in range(0, nz // 2):
        n_below = nz - n_above
        dc = (cb - c0) / (n_below - 1)
        dz0 = z_of_c(c0) - z_of_c(c0 + dc)
        top = n_above * dz0
        err = abs(top - zt)
        if best is None or err < best[0]:
            best = (err, n_below, n_above, dc, dz0)
    _, n_below, n_above, dc, dz0 = best
    c_below = cb - dc * np.arange(n_below)           # bottom -> z = 0
    z_below = z_of_c(c_below)
    z_above = dz0 * np.arange(1, n_above + 1)
    z = np.concatenate([z_below, z_above])
    c = np.concatenate([c_below, np.full(n_above, c0)])
    # density: adiabatic rho ~ (zs - z)^(1/(gamma-1)) below, isothermal above
    m = 1.0 / gm1
    rho = np.empty(nz)
    rho[:n_below] = rho_surf * ((zs - z_below) / zs) ** m
    h = c2_0 / (gamma * g)
    rho[n_below:] = rho_surf * np.exp(-z_above / h)
    p = rho * c * c / gamma
    table = np.empty((nz, 6))
    table[:, 0] = 1.0 + z / RSUN_CM
    table[:, 1] = c
    table[:, 2] = rho
    table[:, 3] = p
    table[:, 4] = g
    table[:, 5] = gamma
    return table


def read_polytrope(path: str, nz: int) -> np.ndarray:
    """Read a reference-format background file; like solar_data it needs
    exactly nz rows (initialize.f90:742-744)."""
    t = np.loadtxt(path, dtype=np.float64)
    if t.ndim != 2 or t.shape[1] != 6 or t.shape[0] < nz:
        raise ValueError(f"{path}: need {nz} rows of 6 columns")
    return np.ascontiguousarray(t[:nz])


def write_polytrope(path: str, table: np.ndarray) -> None:
    with open(path, "w") as f:
        for row in table:
            f.write("%.6f %.6e %.6e %.6e %.6e %12.6f\n" % tuple(row))
