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


def _dxdy(nx: int, ny: int, lx: float, ly: float):
    """Spectral d/dx and d/dy (cm) of real (nz, ny, nx) fields; the Nyquist
    multipliers are 0, as the reference's c2r gives them."""
    kx = 2.0 * np.pi * np.fft.rfftfreq(nx, d=lx / nx)
    if nx % 2 == 0:
        kx[-1] = 0.0
    ky = 2.0 * np.pi * np.fft.fftfreq(ny, d=ly / ny)
    if ny % 2 == 0:
        ky[ny // 2] = 0.0

    def dx(f):
        return np.fft.irfft(np.fft.rfft(f, axis=2) * (1j * kx)[None, None, :], n=nx, axis=2)

    def dy(f):
        return np.fft.ifft(np.fft.fft(f, axis=1) * (1j * ky)[None, :, None], axis=1).real

    return dx, dy


def mhs_flux_tube_background(p, table: np.ndarray, ddz, b0: float = 2000.0, r0_mm: float = 3.0,
                             z_min_mm: float = -8.0, d_mm: float = 8.0, x0_mm: float = 0.0, y0_mm: float = 0.0):
    """Axisymmetric magnetic flux tube in magnetohydrostatic balance on the
    quiet column (the 3-D form of code_python/tubex.py:46-90), as the cgs
    arrays a magnetic run reads (rho, c, p, B_x, B_y, B_z; READ_IN_FIELD,
    all_modules.f90:486-513), each (nz, ny, nx), FP64.

    Field: B = curl(A_phi e_phi) with
        A_phi(r, z) = (Phi / 2 pi r) (1 - exp(-r^2 / R(z)^2)),  Phi = pi b0 R0^2,
    i.e. B_z = (Phi / pi R^2) exp(-r^2/R^2), B_r = r B_z R'(z) / R, taken
    analytically: divergence-free, flux Phi at every height.  The radius
    R(z) = R0 sqrt(1 + ((z - z_min) / D)^2) is narrowest (R0, axis field b0)
    at z_min and widens smoothly above and below (R R'' <= R0^2 / D^2), so
    the tube's curvature forces stay a fraction of its pressure deficit.
    Balance: with the Lorentz force F = (curl B) x B / 4 pi formed by the
    solver's own operators (spectral d/dx, d/dy; d/dz the compact scheme
    with ibc 1, ddz(f, 1) / ddz(z, 1) as tubex.py:14-17 forms it),
      * p solves the horizontal balance grad_h p = F_h in the least-squares
        sense on each plane (div_h grad_h p = div_h F_h, FFT), pinned to the
        table's p at the box corner, far from the tube (tubex.py:71-73);
      * rho = (F_z - dp/dz) / g balances the vertical force, pinned the same
        way to the table's rho (tubex.py:84-86): far from the tube the column
        is the table's, whose own hydrostatic residual is kept as it is;
      * c^2 = c_q^2 rho_q / p_q * p / rho (tubex.py:98).
    ddz(f, bc): the FP64 compact z derivative of an (nz, ny, nx) array of
    this grid (Solver.ddz of any context on this table).

    Returns ((rho, c, p, bx, by, bz), info).  info holds the force-balance
    residual R = grad p - F - rho g (g pointing down) relative to the largest
    Lorentz force, with the table's own hydrostatic residual Q(z) taken out
    of R_z, and the smallest p / p_q and rho / rho_q.  A tube the column
    cannot hold (p or rho <= 0 anywhere) raises ValueError.
    """
    nx, ny, nz = p.nx, p.ny, p.nz
    z = (table[:, 0] - 1.0) * RSUN_CM
    c_q, rho_q, p_q, g_q = table[:, 1], table[:, 2], table[:, 3], table[:, 4]
    dz_idx = ddz(np.ascontiguousarray(np.broadcast_to(z[:, None, None], (nz, ny, nx))), 1)[:, :1, :1]

    def dz(f):
        return ddz(np.ascontiguousarray(f), 1) / dz_idx

    dx, dy = _dxdy(nx, ny, p.xlength, p.ylength)
    r0, zm, dd = r0_mm * 1e8, z_min_mm * 1e8, d_mm * 1e8
    u = (z - zm) / dd
    R = r0 * np.sqrt(1.0 + u * u)
    dR = r0 * u / (dd * np.sqrt(1.0 + u * u))
    phi = np.pi * b0 * r0 * r0
    x = (np.arange(nx) / nx - 0.5) * p.xlength - x0_mm * 1e8
    y = (np.arange(ny) / ny - 0.5) * p.ylength - y0_mm * 1e8
    X, Y = np.meshgrid(x, y)
    E = np.exp(-(X * X + Y * Y)[None] / (R * R)[:, None, None])
    bz = (phi / (np.pi * R * R))[:, None, None] * E
    br_r = (phi * dR / (np.pi * R ** 3))[:, None, None] * E         # B_r / r
    bx = br_r * X[None]
    by = br_r * Y[None]
    del E, br_r
    jx = dy(bz) - dz(by)
    jy = dz(bx) - dx(bz)
    jz = dx(by) - dy(bx)
    f4 = 4.0 * np.pi
    fx = (jy * bz - jz * by) / f4
    fy = (jz * bx - jx * bz) / f4
    fz = (jx * by - jy * bx) / f4
    del jx, jy, jz
    # horizontal balance: div_h grad_h p = div_h F_h per plane (FFT over y, x)
    kx = 2.0 * np.pi * np.fft.fftfreq(nx, d=p.xlength / nx)
    ky = 2.0 * np.pi * np.fft.fftfreq(ny, d=p.ylength / ny)
    k2 = kx[None, :] ** 2 + ky[:, None] ** 2
    k2[0, 0] = 1.0
    div = np.fft.fft2(fx) * (1j * kx)[None, None, :] + np.fft.fft2(fy) * (1j * ky)[None, :, None]
    ptil = np.fft.ifft2(-div / k2[None]).real
    del div
    pres = p_q[:, None, None] + (ptil - ptil[:, :1, :1])
    del ptil
    dzp = dz(pres)
    rho = (fz - dzp) / g_q[:, None, None]
    rho = rho - (rho[:, :1, :1] - rho_q[:, None, None])
    if pres.min() <= 0.0 or rho.min() <= 0.0:
        raise ValueError(f"the column cannot hold this tube: min p/p_q = {(pres / p_q[:, None, None]).min():.3g}, "
                         f"min rho/rho_q = {(rho / rho_q[:, None, None]).min():.3g}")
    c = np.sqrt((c_q ** 2 * rho_q / p_q)[:, None, None] * pres / rho)
    # residual of grad p = F + rho g, the table's own hydrostatic residual
    # (the same in the quiet column) taken out of the z component
    q = dz(np.broadcast_to(p_q[:, None, None], (nz, ny, nx)))[:, :1, :1] + (rho_q * g_q)[:, None, None]
    rx = dx(pres) - fx
    ry = dy(pres) - fy
    rz = dzp - fz + rho * g_q[:, None, None] - q
    fmag = np.sqrt(fx * fx + fy * fy + fz * fz)
    fmax = float(fmag.max())
    info = {
        "lorentz_max_dyn_cm3": fmax,
        "residual_h_max_rel": float(max(np.abs(rx).max(), np.abs(ry).max()) / fmax) if fmax > 0 else 0.0,
        "residual_z_max_rel": float(np.abs(rz).max() / fmax) if fmax > 0 else 0.0,
        "residual_l2_rel": float(np.sqrt(np.sum(rx * rx + ry * ry + rz * rz)) / np.sqrt(np.sum(fmag * fmag)))
        if fmax > 0 else 0.0,
        "table_hydrostatic_residual_rel": float(np.abs(q).max() / np.abs(rho_q * g_q).max()),
        "min_p_ratio": float((pres / p_q[:, None, None]).min()),
        "min_rho_ratio": float((rho / rho_q[:, None, None]).min()),
        "b_axis_max_G": float(np.abs(bz).max()),
        "b_axis_top_G": float(bz[-1].max()),
        "beta_axis_top": float(8.0 * np.pi * pres[-1].min() / max(bz[-1].max() ** 2, 1e-300)),
        "radius_top_mm": float(R[-1] / 1e8),
    }
    return (rho, c, pres, bx, by, bz), info


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


# ---- magnetohydrostatic sheet from a vector potential (code_python/tubex.py) ----

TUBEX_RSUN_MM = 695.9894      # tubex.py:9 (its own value of R_sun in Mm)
TUBEX_GRAV = 2.775e4          # tubex.py:44
TUBEX_CONVERT = 1e8           # tubex.py:45 (Mm -> cm)


def _x_derivative(a: np.ndarray, period: float) -> np.ndarray:
    """d/dx along the last axis by the FFT (period `period`); the Nyquist
    term of an even length drops out, as it does in a real inverse FFT."""
    n = a.shape[-1]
    k = 2.0 * np.pi * np.fft.rfftfreq(n, d=period / n)
    return np.fft.irfft(np.fft.rfft(a, axis=-1) * (1j * k), n=n, axis=-1)


def _x_integral(a: np.ndarray, period: float) -> np.ndarray:
    """The periodic antiderivative along the last axis by the FFT: the mean
    (k = 0) term has no periodic integral and is dropped, as is Nyquist."""
    n = a.shape[-1]
    k = 2.0 * np.pi * np.fft.rfftfreq(n, d=period / n)
    f = np.fft.rfft(a, axis=-1)
    inv = np.zeros_like(k)
    inv[1:] = 1.0 / k[1:]
    return np.fft.irfft(f * (-1j * inv), n=n, axis=-1)


def vector_potential_background(solver, table: np.ndarray, lx_mm: float = 400.0, a0: float = 5000.0,
                                decay_x: float = 10.0, decay_z: float = 10.0, decay_z_start: float = 12.0,
                                zero_b: bool = True) -> dict:
    """The 2-D magnetohydrostatic backgrounds of code_python/tubex.py:27-141
    (true and starting models of an inversion for the vector potential).

    A(x, z) = a0 f(x) exp(z / decay), f = -(x/dx) / (1 + (x/dx)^4), with
    x = -lx/2 .. lx/2 (nx points, no endpoint) and z = (r/R_sun - 1) R_sun in
    Mm from the background table.  True field: the analytic B_x = -dA/dz,
    B_z = dA/dx (tubex.py:53-54); starting field from the numerical
    derivatives of A_start (decay_z_start).  With the true field's Lorentz
    force F = dB_x/dz - dB_z/dx, the pressure is the periodic x-integral of
    B_z F, pinned to the table's p at x index 0, and the density balances
    dp/dz + B_x F against gravity, pinned the same way (tubex.py:69-90);
    c^2 = c_q^2 rho_q / p_q * p / rho.  zero_b (tubex.py:10, on in the
    reference) zeroes both fields and potentials, leaving the quiet column.

    The z derivatives are the compact scheme with ibc = 1 divided by the
    same derivative of z (tubex.py:14-17,33-36), here from the library's FP64
    ddz on the GPU (solver: a context of shape (nz, 1, nx) on this table); x
    derivatives and the x integral are FFT ones (the fftcalculus module the
    script imports is not in the reference).  Returns (nz, 1, nx) arrays:
    bx, bz, psi (A sqrt(4 pi) / R_sun, the model_vectorpsi unit) for 'true'
    and 'start', and p, rho, c shared by both models.
    """
    nz = table.shape[0]
    nz_s, ny_s, nx = solver.shape
    if nz_s != nz or ny_s != 1:
        raise ValueError(f"solver must be (nz={nz}, 1, nx), got {solver.shape}")
    x = np.linspace(-lx_mm / 2.0, lx_mm / 2.0, num=nx, endpoint=False)
    z = (table[:, 0] - 1.0) * TUBEX_RSUN_MM
    p_q, rho_q, c2_q = table[:, 3], table[:, 2], table[:, 1] ** 2

    def grid(col_z, row_x):                     # (nz, 1, nx) outer product
        return (np.asarray(col_z)[:, None] * np.asarray(row_x)[None, :])[:, None, :]

    dz_idx = solver.ddz(np.broadcast_to(z[:, None, None], (nz, 1, nx)), 1)

    def derivz(a):
        return solver.ddz(a, 1) / dz_idx

    fx = -(x / decay_x) / (1.0 + (x / decay_x) ** 4)
    dfx = -decay_x ** 3 * (decay_x ** 4 - 3.0 * x ** 4) / (decay_x ** 4 + x ** 4) ** 2
    gz = np.exp(z / decay_z)
    bx = -a0 * grid(gz / decay_z, fx)
    bz = a0 * grid(gz, dfx)
    a_true = a0 * grid(gz, fx)
    a_start = a0 * grid(np.exp(z / decay_z_start), fx)
    bx_start = -derivz(a_start)
    bz_start = _x_derivative(a_start, lx_mm)
    if zero_b:
        bx = np.zeros_like(bx); bz = np.zeros_like(bz)
        bx_start = np.zeros_like(bx); bz_start = np.zeros_like(bx)
        a_start = np.zeros_like(a_start); a_true = np.zeros_like(a_true)
    force = derivz(bx) - _x_derivative(bz, lx_mm)
    hz = bx * force
    hx = bz * force
    pres = _x_integral(hx, lx_mm)
    pres = pres - (pres[:, :, :1] - p_q[:, None, None])
    dzp = derivz(pres)
    if (pres / p_q[:, None, None] - 1.0).min() < -1.0:
        raise ValueError("negative pressure")
    rho = -(hz + dzp) / (TUBEX_GRAV * TUBEX_CONVERT)
    rho = rho - (rho[:, :, :1] - rho_q[:, None, None])
    if (rho / rho_q[:, None, None] - 1.0).min() < -1.0:
        raise ValueError("negative density")
    c = np.sqrt((c2_q * rho_q / p_q)[:, None, None] * pres / rho)
    s4 = np.sqrt(4.0 * np.pi)
    return {"true": {"bx": bx, "bz": bz, "psi": a_true * s4 / TUBEX_RSUN_MM},
            "start": {"bx": bx_start, "bz": bz_start, "psi": a_start * s4 / TUBEX_RSUN_MM},
            "p": pres, "rho": rho, "c": c, "x_mm": x, "z_mm": z}


def write_vector_potential_models(modeldir: str, models: dict) -> list:
    """The FITS files tubex.py:143-160 writes, (nz, nx) arrays under
    modeldir/true and modeldir/start: B_z2D, B_x2D (times sqrt(4 pi)),
    true_vectorpsi, model_vectorpsi_ls00, pressure2D, density2D,
    soundspeed2D and model_c_ls00."""
    import os
    from . import io
    s4 = np.sqrt(4.0 * np.pi)
    t, st = os.path.join(modeldir, "true"), os.path.join(modeldir, "start")
    os.makedirs(t, exist_ok=True)
    os.makedirs(st, exist_ok=True)
    out = []

    def put(path, a):
        io.write_fits(path, np.asarray(a)[:, 0, :])
        out.append(path)

    put(os.path.join(t, "B_z2D.fits"), models["true"]["bz"] * s4)
    put(os.path.join(t, "B_x2D.fits"), models["true"]["bx"] * s4)
    put(os.path.join(t, "true_vectorpsi.fits"), models["true"]["psi"])
    put(os.path.join(st, "model_vectorpsi_ls00.fits"), models["start"]["psi"])
    for d in (t, st):
        put(os.path.join(d, "pressure2D.fits"), models["p"])
        put(os.path.join(d, "density2D.fits"), models["rho"])
        put(os.path.join(d, "soundspeed2D.fits"), models["c"])
    put(os.path.join(st, "model_c_ls00.fits"), models["c"])
    return out


def config3_background(p, table: np.ndarray, ddz):
    """The flux-tube configuration's background: the magnetohydrostatic
    tube of mhs_flux_tube_background with its defaults (2 kG and 3 Mm at
    z = -8 Mm, widening over D = 8 Mm; about 1 kG and 4.2 Mm at the
    surface), on the box centre.  Returns ((rho, c, p, bx, by, bz), info)."""
    return mhs_flux_tube_background(p, table, ddz)
