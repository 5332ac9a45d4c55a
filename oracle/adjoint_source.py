"""CPU restatement (numpy, FP64) of the adjoint source of a 2-D run,
ADJOINT_SOURCE_FILT (driver.f90:1262-1686), with the ridge filters
FMODE_FILTER / PMODE_FILTER (driver.f90:1074-1119, 1173-1222), FREQ_FILTER
(:1225-1237), COMPUTE_TT (:921-960) with its 3x3 `inverse` (:964-1042) and
distmat (initialize.f90:1124-1141).

Test infrastructure: only the tests import this module, as the checker of
the CUDA path.  The FFTW calls of the reference are numpy FFTs here:
dfftw_plan_dft_3d(nx, 1, nt) forward is fftn (unnormalised, sign -1), and its
backward plan is ifftn times nx*nt (FFTW's unnormalised inverse).

Arrays are (nt, nx) in C order, the memory layout of the reference's
(nx, 1, nt) Fortran arrays.  Literal constants keep the reference's kinds:
REAL*4 literals (0.4, 1.1, 2.056565, ...) enter as their float32 values.
"""
from __future__ import annotations

import numpy as np


def r4(v: float) -> float:
    return float(np.float32(v))


PI = r4(3.14159265358979)            # initialize.f90:38


def distmat(n: int) -> np.ndarray:
    """distmat(n, 1, f) (initialize.f90:1124-1141): signed index distance
    min(i-1, n-i+1), negative in the upper half."""
    i = np.arange(1, n + 1)
    i2 = np.minimum(i - 1, n - i + 1).astype(np.float64)
    sig = np.where((i - 1) > (n - i + 1), -1.0, 1.0)
    return np.sqrt(i2 ** 2) * sig


def _kw(nx: int, nt: int, xlength: float, outputcad: float):
    k = np.abs(distmat(nx)) * 2.0 * PI / (xlength * r4(1e-8) * nx / (nx - 1.0))
    w = np.abs(distmat(nt)) * 2.0 * PI / (nt * outputcad)
    return k, w


def fmode_filter(nx, nt, xlength, outputcad) -> np.ndarray:
    """FMODE_FILTER (driver.f90:1074-1119), (nt, nx)."""
    poly = (1.0, 3.0, r4(-0.6))
    const, df, f_low = r4(2.056565), 0.5, r4(1.1)
    k, w = _kw(nx, nt, xlength, outputcad)
    f0 = const * k ** 0.5
    f1 = poly[0] + poly[1] * k + poly[2] * k ** 2.0
    f = w / (2.0 * PI) * 1e3
    out = np.zeros((nt, nx))
    delta = f1 - f0
    for j in range(nt):
        d = f[j] - f0
        m = (d < delta) & (d > 0)
        out[j, m] = 0.5 * (1.0 + np.cos(PI * (2.0 * d[m] / delta[m] - 1)))
    for j in range(nt):
        if f[j] < f_low + df:
            out[j] = out[j] * 0.5 * (1.0 + np.cos(PI * (f[j] - (f_low + df)) / df))
        if f[j] < f_low:
            out[j] = 0.0
    return out


def pmode_filter(nx, nt, xlength, outputcad) -> np.ndarray:
    """PMODE_FILTER (driver.f90:1173-1222), (nt, nx)."""
    poly = (r4(1.1), r4(5.2), r4(-1.3))
    const, df, f_low = r4(3.96), 0.5, r4(1.6)
    k, w = _kw(nx, nt, xlength, outputcad)
    f0 = const * np.abs(k) ** 0.5
    f1 = poly[0] + poly[1] * k + poly[2] * k ** 2.0
    f = w / (2.0 * PI) * 1e3
    out = np.zeros((nt, nx))
    delta = f1 - f0
    for j in range(nt):
        d = f[j] - f0
        m = (d < delta) & (d > 0)
        out[j, m] = 0.5 * (1.0 + np.cos(PI * (2.0 * d[m] / delta[m] - 1)))
    for j in range(nt):
        if f[j] < f_low:
            out[j] = 0.0
        if f[j] < f_low + df:
            out[j] = out[j] * 0.5 * (1.0 + np.cos(PI * (f[j] - (f_low + df)) / df))
    return out


def freq_filter(f1: float, f2: float, nt: int, outputcad: float) -> np.ndarray:
    """FREQ_FILTER (driver.f90:1225-1237): band pass between f1 and f2 (mHz)."""
    w = np.abs(distmat(nt)) * 1e3 / (nt * outputcad)
    wid = r4(0.4) * (w[1] - w[0])
    return 1.0 / (1.0 + np.exp((f1 - w) / wid)) - 1.0 / (1.0 + np.exp((f2 - w) / wid))


def inverse3(a: np.ndarray) -> np.ndarray:
    """`inverse` (driver.f90:964-1042): Doolittle LU without pivoting, then
    one forward and back substitution per column of the identity."""
    a = np.array(a, dtype=np.float64)
    n = a.shape[0]
    L = np.zeros((n, n))
    U = np.zeros((n, n))
    for k in range(n - 1):
        for i in range(k + 1, n):
            coeff = a[i, k] / a[k, k]
            L[i, k] = coeff
            for j in range(k + 1, n):
                a[i, j] = a[i, j] - coeff * a[k, j]
    for i in range(n):
        L[i, i] = 1.0
    for j in range(n):
        for i in range(j + 1):
            U[i, j] = a[i, j]
    c = np.zeros((n, n))
    b = np.zeros(n)
    for k in range(n):
        b[k] = 1.0
        d = np.zeros(n)
        d[0] = b[0]
        for i in range(1, n):
            d[i] = b[i]
            for j in range(i):
                d[i] = d[i] - L[i, j] * d[j]
        x = np.zeros(n)
        x[n - 1] = d[n - 1] / U[n - 1, n - 1]
        for i in range(n - 2, -1, -1):
            x[i] = d[i]
            for j in range(n - 1, i, -1):
                x[i] = x[i] - U[i, j] * x[j]
            x[i] = x[i] / U[i, i]
        c[:, k] = x
        b[k] = 0.0
    return c


def compute_tt(u0: np.ndarray, u: np.ndarray, dt: float) -> float:
    """COMPUTE_TT (driver.f90:921-960): cross-correlation over lags
    -nt+1..nt-1, parabola through the maximum and its neighbours."""
    nt = len(u0)
    cc = np.zeros(2 * nt - 1)
    t = np.zeros(2 * nt - 1)
    for i in range(-nt + 1, 1):
        t[i + nt - 1] = i * dt
        l1 = -i + 1
        cc[i + nt - 1] = np.sum(u0[l1 - 1:nt] * u[0:nt - l1 + 1]) * dt
    for i in range(1, nt):
        t[i + nt - 1] = i * dt
        l2 = nt - i
        cc[i + nt - 1] = np.sum(u0[0:l2] * u[i:nt]) * dt
    loc = int(np.argmax(cc))                    # 0-based position of maxloc(cc)
    if loc < 1 or loc > 2 * nt - 3:
        raise ValueError("cross-correlation peak at the end of the lag range")
    times = t[loc - 1:loc + 2]
    mat = np.stack([np.ones(3), times, times ** 2.0], axis=1)
    inv = inverse3(mat)
    p1 = inv[1, 0] * cc[loc - 1] + inv[1, 1] * cc[loc] + inv[1, 2] * cc[loc + 1]
    p2 = inv[2, 0] * cc[loc - 1] + inv[2, 1] * cc[loc] + inv[2, 2] * cc[loc + 1]
    return float(-p1 * 0.5 / p2)


def adjoint_source_filt(acc: np.ndarray, dat: np.ndarray, xlength: float, outputcad: float, x00: float,
                        t: np.ndarray, ridges: dict, bands: dict, windows_in: dict | None = None):
    """ADJOINT_SOURCE_FILT (driver.f90:1262-1686) of a 2-D run.

    acc, dat: synthetic and observed surface v_z, (nt, nx); x00: master
    pixel (Mm); t: output times in minutes, ascending (the reversed timeline,
    driver.f90:1310-1315); ridges: {0: f mode, 1: p1 ridge, 2: band-passed
    phase-speed set} -> (mindist, maxdist, window) of params.0..2 (absent key
    = no file); bands: {0, 1} -> (left, right) corners (mHz) of
    filter.params.0/1; windows_in: {0, 1} -> {x index: (lef, rig)} read in a
    line search (windows.0/1), else None.

    Returns (adj (nt, nx), misfit_tot = 0.5 sum tau^2, nmeasurements,
    windows {0, 1} -> {x index: (lef, rig)}, taus {(pord, x index): tau}).
    """
    nt, nx = acc.shape
    linesearch = windows_in is not None
    x = np.arange(nx) / nx
    kk = distmat(nx)
    eyekh = 1j * kk * 2.0 * PI
    distances = np.abs((x - 0.5) * xlength * r4(1e-8) - x00)
    dt = t[1] - t[0]
    freqnu = distmat(nt) / (nt * dt * 60.0)
    N = nx * nt
    spec = np.fft.fftn(acc.astype(np.complex128))
    specd = np.fft.fftn(dat.astype(np.complex128))
    fmode = fmode_filter(nx, nt, xlength, outputcad)
    pmode = pmode_filter(nx, nt, xlength, outputcad)
    filt = np.ones(nt)
    if 0 in bands:
        filt = freq_filter(bands[0][0], bands[0][1], nt, outputcad)
    fmode = fmode * filt[:, None]
    if 1 in bands:
        filt = freq_filter(bands[1][0], bands[1][1], nt, outputcad)
    pmode = pmode * filt[:, None]
    adj = np.zeros((nt, nx))
    misfit = 0.0
    nmeas = 0
    windows = {0: {}, 1: {}}
    taus = {}
    vel = (0.75, 1.00)

    def measure(pord, i, filt2, lef, rig, a_, d_, c_):
        nonlocal misfit, nmeas
        leng = rig - lef + 1
        tau = compute_tt(a_[lef - 1:rig, i].real, d_[lef - 1:rig, i].real, dt)
        taus[(pord, i)] = tau
        win = np.zeros(nt)
        win[lef - 1:rig] = 1.0
        ccdotone = np.fft.fft(c_[:, i] * win)
        filtemp = filt2 * ccdotone[:, None] * np.exp(-eyekh * x[i])[None, :]
        filtex = np.fft.ifftn(filtemp) * N
        misfit += tau ** 2.0
        nmeas += 1
        con = -tau / (np.sum(c_[lef - 1:rig, i] * c_[lef - 1:rig, i]) * dt)
        adj[::-1, :] += (filtex * con).real
        return leng

    def filtered(filt2):
        a_ = np.fft.ifftn(spec * filt2) * N
        d_ = np.fft.ifftn(specd * filt2) * N
        c_ = np.fft.ifftn(spec * filt2 * (1j * freqnu * (2.0 * PI))[:, None]) * N
        return a_, d_, c_

    for pord in (0, 1):
        if pord not in ridges:
            continue
        mindist, maxdist, window = ridges[pord]
        halftime = int(np.floor(window / (2.0 * dt) + 0.5))       # nint
        filt2 = fmode if pord == 0 else pmode
        a_, d_, c_ = filtered(filt2)
        for i in range(nx):
            if not (distances[i] > mindist and distances[i] < maxdist):
                continue
            if not linesearch:
                timest = int(np.floor(distances[i] / vel[pord] * 1.0 / dt))
                timefin = timest + 40
                seg = np.abs(a_[timest - 1:timefin, i].real)
                loc = int(np.argmax(seg)) + timest
                lef, rig = loc - halftime, loc + halftime
                windows[pord][i] = (lef, rig)
            else:
                lef, rig = windows_in[pord][i]
            measure(pord, i, filt2, lef, rig, a_, d_, c_)
    # phase-speed set: the high-p filter is the last band pass alone
    pcoef = (r4(13.4090), r4(0.3421), r4(-0.0005), 0.0, 0.0)
    if 2 in ridges:
        mindist, maxdist, window = ridges[2]
        halftime = int(np.floor(window / (2.0 * dt) + 0.5))
        filt2 = np.ones((nt, nx)) * filt[:, None]
        a_, d_, c_ = filtered(filt2)
        for i in range(nx):
            if not (distances[i] > mindist and distances[i] < maxdist):
                continue
            d = distances[i]
            if d < 250.0:
                v = (pcoef[0] - t[0] + pcoef[1] * d + pcoef[2] * d ** 2.0 + pcoef[3] * d ** 3.0
                     + pcoef[4] * d ** 4.0) / dt
                timesmax = int(np.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1) + 1
                loc = int(np.argmax(a_[timesmax - 7:timesmax + 6, i].real)) + timesmax - 6
            else:
                loc = int(np.argmax(a_[:, i].real)) + 1
            lef, rig = loc - halftime, loc + halftime
            measure(2, i, filt2, lef, rig, a_, d_, c_)
    adj = adj * nt / 60.0
    return adj, 0.5 * misfit, nmeas, windows, taus


MISFIT_BANDS = ((2.0, 3.5), (3.5, 4.5), (4.5, 6.0))    # driver.f90:1812-1824 (mHz)


def misfit_all(acc: np.ndarray, dat: np.ndarray, xlength: float, outputcad: float, x00: float, t: np.ndarray,
               ridges: dict, windows_in: dict | None = None):
    """MISFIT_ALL (driver.f90:1702-2076) of a 2-D run: for each of three
    frequency bands the f, p1 and band-passed sets of ADJOINT_SOURCE_FILT,
    with its own ridge speeds (1.01, 1.465 Mm/min) and arrival polynomial,
    measure tau per pixel; no adjoint source.

    Returns (misfit[band][set] = 0.5 sum tau^2, nmeas[band][set], windows
    {(band, set): {pixel: (lef, rig)}} of sets 0 and 1); windows_in, keyed
    the same way, are read in a line search (windows.all.N)."""
    nt, nx = acc.shape
    linesearch = windows_in is not None
    x = np.arange(nx) / nx
    distances = np.abs((x - 0.5) * xlength * r4(1e-8) - x00)
    dt = t[1] - t[0]
    N = nx * nt
    spec = np.fft.fftn(acc.astype(np.complex128))
    specd = np.fft.fftn(dat.astype(np.complex128))
    vel = (1.01, 1.465)
    pcoef = (r4(22.5000), r4(0.235317), r4(0.00134167), r4(-1.32222e-05), r4(3.00000e-08))
    mis = np.zeros((3, 3))
    nmeas = np.zeros((3, 3), dtype=int)
    windows = {}
    for b, (lc, rc) in enumerate(MISFIT_BANDS):
        filt = freq_filter(lc, rc, nt, outputcad)
        sets = {0: fmode_filter(nx, nt, xlength, outputcad) * filt[:, None],
                1: pmode_filter(nx, nt, xlength, outputcad) * filt[:, None],
                2: np.ones((nt, nx)) * filt[:, None]}
        for pord in (0, 1, 2):
            if pord not in ridges:
                continue
            mindist, maxdist, window = ridges[pord]
            halftime = int(np.floor(window / (2.0 * dt) + 0.5))
            a_ = np.fft.ifftn(spec * sets[pord]) * N
            d_ = np.fft.ifftn(specd * sets[pord]) * N
            if pord < 2:
                windows[(b, pord)] = {}
            for i in range(nx):
                if not (distances[i] > mindist and distances[i] < maxdist):
                    continue
                if pord < 2 and linesearch:
                    lef, rig = windows_in[(b, pord)][i]
                elif pord < 2:
                    timest = int(np.floor(distances[i] / vel[pord] * 1.0 / dt))
                    timefin = timest + 40
                    loc = int(np.argmax(np.abs(a_[timest - 1:timefin, i].real))) + timest
                    lef, rig = loc - halftime, loc + halftime
                else:
                    d = distances[i]
                    if d < 250.0:
                        v = (pcoef[0] - t[0] + pcoef[1] * d + pcoef[2] * d ** 2.0 + pcoef[3] * d ** 3.0
                             + pcoef[4] * d ** 4.0) / dt
                        timesmax = int(np.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1) + 1
                        loc = int(np.argmax(a_[timesmax - 7:timesmax + 6, i].real)) + timesmax - 6
                    else:
                        loc = int(np.argmax(a_[:, i].real)) + 1
                    lef, rig = loc - halftime, loc + halftime
                if pord < 2:
                    windows[(b, pord)][i] = (lef, rig)
                tau = compute_tt(a_[lef - 1:rig, i].real, d_[lef - 1:rig, i].real, dt)
                mis[b, pord] = mis[b, pord] + tau ** 2.0
                nmeas[b, pord] += 1
    return mis * 0.5, nmeas, windows
