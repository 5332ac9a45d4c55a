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


def flux_tube_background(p, table: np.ndarray, b_surf: float = 2000.0, r_surf_mm: float = 3.0,
                         x0_mm: float = 0.0, y0_mm: float = 0.0, b_max_ratio: float = 4.0,
                         p_floor: float = 0.2):
    """Axisymmetric self-similar magnetic flux tube on the quiet column, as the
    3-D cgs arrays the reference reads for a magnetic run (rho, c, p, B_x,
    B_y, B_z; READ_IN_FIELD, all_modules.f90:486-513), each (nz, ny, nx).

    Field from an azimuthal vector potential in FP64,
        A_phi(r, z) = (Phi / 2 pi r) (1 - exp(-r^2 / R(z)^2)),  Phi = pi b_surf R0^2,
    so B = curl(A_phi e_phi) is divergence-free with a Gaussian profile
    B_z = B_axis(z) exp(-r^2/R^2), B_axis R^2 = b_surf R0^2 (flux
    conservation, self-similar), B_r = r B_z R'(z) / R.  The axis strength
    follows p_quiet(z)^(1/4) relative to z = 0 (a tube that narrows with
    depth), bounded to [b_surf / b_max_ratio, b_surf * b_max_ratio].
    Balance: horizontal pressure balance of a thin tube, p = p_quiet - B^2 / 8pi,
    floored at p_floor * p_quiet (the evacuated core), and rho scaled with p
    at the quiet temperature (c unchanged).  This is a synthetic test
    background in approximate magnetohydrostatic balance, not the reference's
    own tube model (whose generator needs modules absent from it).
    """
    nx, ny, nz = p.nx, p.ny, p.nz
    z_cm = (table[:, 0] - 1.0) * RSUN_CM
    c_q, rho_q, p_q = table[:, 1], table[:, 2], table[:, 3]
    k0 = int(np.argmin(np.abs(z_cm)))
    b_axis = b_surf * (p_q / p_q[k0]) ** 0.25
    b_axis = np.clip(b_axis, b_surf / b_max_ratio, b_surf * b_max_ratio)
    r0 = r_surf_mm * 1e8
    R = r0 * np.sqrt(b_surf / b_axis)                       # flux conservation
    dRdz = np.gradient(R, z_cm)
    x = (np.arange(nx) / nx - 0.5) * p.xlength - x0_mm * 1e8
    y = (np.arange(ny) / ny - 0.5) * p.ylength - y0_mm * 1e8
    X, Y = np.meshgrid(x, y)                               # (ny, nx)
    r2 = X ** 2 + Y ** 2
    bz = np.empty((nz, ny, nx)); bx = np.empty_like(bz); by = np.empty_like(bz)
    for k in range(nz):
        g = np.exp(-r2 / R[k] ** 2)
        bz[k] = b_axis[k] * g
        br_over_r = b_axis[k] * g * dRdz[k] / R[k]            # B_r / r
        bx[k] = br_over_r * X
        by[k] = br_over_r * Y
    b2 = bx ** 2 + by ** 2 + bz ** 2
    pq = p_q[:, None, None]
    pres = np.maximum(pq - b2 / (8.0 * np.pi), p_floor * pq)
    rho = rho_q[:, None, None] * pres / pq
    c = np.broadcast_to(c_q[:, None, None], (nz, ny, nx)).copy()
    return rho, c, pres, bx, by, bz


def flux_sheet_background(p, table: np.ndarray, b_surf: float = 300.0, w_mm: float = 10.0,
                          z_fade_mm: float = 0.0, fade_mm: float = 0.2, x0_mm: float = 0.0,
                          p_floor: float = 0.2):
    """2-D (ny = 1) magnetic flux sheet on the quiet column, as the cgs arrays
    the reference reads for the 2-D MHD run (density, sound speed, pressure
    and the vector potential psi of model_vectorpsi, physics2d.f90:106-146),
    each (nz, 1, nx).

    The reference forms B_x = -d psi/dz and B_z = d psi/dx * stretchx with x
    and z in solar radii, so psi is in G R_sun.  Here
        psi(x, z) = (sqrt(pi)/2) b(z) W erf((x - x0) / W),
        b(z) = b_surf / (1 + exp((z - z_fade) / fade)),
    a sheet of constant half-width W (a few pixels: DBYD1 rings on a sheet
    narrower than the grid): B_z = b(z) exp(-(x-x0)^2/W^2), and a
    horizontal B_x = -(sqrt(pi)/2) W b'(z) erf(.) only in the fade layer.
    The field fades out of the low-density atmosphere: a sheet that spread
    with height there (flux conservation over ~140 km pressure scale heights)
    carries a strong horizontal field in which this linear system grows
    exponentially (the reference notes the form fails at very small
    densities).  Pressure p = p_quiet - B^2/8pi floored at p_floor * p_quiet,
    density scaled with p, c unchanged: a synthetic test background in
    approximate horizontal pressure balance.
    """
    from math import erf
    nx, nz = p.nx, p.nz
    z_r = table[:, 0]
    z_cm = (z_r - 1.0) * RSUN_CM
    c_q, rho_q, p_q = table[:, 1], table[:, 2], table[:, 3]
    W = w_mm * 1e8 / RSUN_CM
    prof = 1.0 / (1.0 + np.exp((z_cm - z_fade_mm * 1e8) / (fade_mm * 1e8)))
    dprof = np.gradient(prof, z_r)
    x = ((np.arange(nx) / nx - 0.5) * p.xlength - x0_mm * 1e8) / RSUN_CM
    E = np.vectorize(erf)(x / W)
    amp = 0.5 * np.sqrt(np.pi) * b_surf * W
    psi = (amp * prof)[:, None, None] * E[None, None, :]
    bz = (b_surf * prof)[:, None, None] * np.exp(-(x / W) ** 2)[None, None, :]
    bx = -(amp * dprof)[:, None, None] * E[None, None, :]
    pq = p_q[:, None, None]
    pres = np.maximum(pq - (bx ** 2 + bz ** 2) / (8.0 * np.pi), p_floor * pq)
    rho = rho_q[:, None, None] * pres / pq
    c = np.broadcast_to(c_q[:, None, None], (nz, 1, nx)).copy()
    return rho, c, pres, psi
