"""CPU FP64 oracle of the SPARC time-stepping path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU baseline
and ``--impl reference`` arm) may import this module, and only as the checker
or the timed CPU baseline.  The product library never loads it.

Parity status: UNPINNED -- the reference (jishnub/sparc) ships no tests or
golden vectors and cannot be built here (no Fortran compiler, MPI, FFTW or
CFITSIO).  ``sparc_oracle.cpp`` restates the Fortran line for line; this module
adds ctypes bindings and small numpy twins used to cross-check the C++.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libsparc_oracle.so")
_SRC = os.path.join(_HERE, "sparc_oracle.cpp")
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile the oracle shared library (g++, OpenMP, no FMA contraction so the
    x86 and Arm builds round identically)."""
    with _lock:
        if (not force and os.path.exists(_SO)
                and os.path.getmtime(_SO) >= os.path.getmtime(_SRC)):
            return _SO
        os.makedirs(_BUILD, exist_ok=True)
        tmp = _SO + f".tmp{os.getpid()}"
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", _SRC, "-o", tmp]
        subprocess.run(cmd, check=True)
        os.replace(tmp, _SO)
        return _SO


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("npmlbot", ctypes.c_int), ("npmltop", ctypes.c_int),
        ("option", ctypes.c_int),
        ("compute_forward", ctypes.c_int), ("compute_adjoint", ctypes.c_int),
        ("damp_waves", ctypes.c_int), ("src_k", ctypes.c_int), ("reserved", ctypes.c_int),
        ("xlength", ctypes.c_double), ("ylength", ctypes.c_double), ("timestep", ctypes.c_double),
        ("excitdep", ctypes.c_double), ("obsheight", ctypes.c_double),
        ("cadforcing", ctypes.c_double), ("outputcad", ctypes.c_double),
        ("nupeak", ctypes.c_double), ("nuwidth", ctypes.c_double),
        ("solartime", ctypes.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        so = build()
        L = ctypes.CDLL(so)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        L.oracle_create.restype = P
        L.oracle_create.argtypes = [ctypes.POINTER(OracleParams), D]
        L.oracle_destroy.argtypes = [P]
        for name, args in {
            "oracle_info": [P, D], "oracle_profiles": [P, D], "oracle_damping_rates": [P, D],
            "oracle_set_source": [P, ctypes.c_int, D, ctypes.c_int, D, ctypes.c_int],
            "oracle_set_state": [P, D, D], "oracle_get_state": [P, D, D, D],
            "oracle_step": [P, ctypes.c_int], "oracle_set_time": [P, ctypes.c_int],
            "oracle_ddx": [P, D, D], "oracle_ddy": [P, D, D],
            "oracle_ddz": [P, D, D, ctypes.c_int], "oracle_damp": [P, D, D],
            "oracle_kernel_reset": [P], "oracle_kernel_accumulate": [P, D, D, D],
            "oracle_kernel_finish": [P, D, ctypes.c_int],
            "oracle_kernel_accumulate_b": [P, D, D], "oracle_kernel_finish_b": [P, D, ctypes.c_int],
            "oracle_plane_r2c": [P, D, D],
            "oracle_set_mhd": [P, D, D, D, D, D, D], "oracle_mhd_profiles": [P, D],
            "oracle_set_mhd2d": [P, D, D, D, D],
        }.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        L.oracle_dbyd2.argtypes = [D, D, ctypes.c_long, ctypes.c_int, ctypes.c_int]
        L.oracle_dbyd2.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_threads.restype = ctypes.c_int
        L.oracle_forward_source.argtypes = [ctypes.POINTER(OracleParams), ctypes.c_int, D]
        L.oracle_forward_source.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(int(n))


def params_struct(p) -> OracleParams:
    """Build the C struct from a ``sparc_gb300.params.SparcParams``."""
    return OracleParams(
        nx=p.nx, ny=p.ny, nz=p.nz, npmlbot=p.npmlbot, npmltop=p.npmltop,
        option=p.option, compute_forward=int(p.compute_forward),
        compute_adjoint=int(p.compute_adjoint), damp_waves=int(p.damp_waves),
        src_k=int(p.src_k), reserved=0,
        xlength=p.xlength, ylength=p.ylength, timestep=p.timestep,
        excitdep=p.excitdep, obsheight=p.obsheight, cadforcing=p.cadforcing,
        outputcad=p.outputcad, nupeak=p.nupeak, nuwidth=p.nuwidth, solartime=p.solartime)


def dbyd2(b: np.ndarray, ibc: int, a_init: np.ndarray | None = None) -> np.ndarray:
    """C++ DBYD2 on an array shaped (N2, N1) in C order (= Fortran B(N1,N2))."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    n2 = b.shape[0]
    n1 = int(np.prod(b.shape[1:])) if b.ndim > 1 else 1
    a = np.zeros_like(b) if a_init is None else np.ascontiguousarray(a_init, dtype=np.float64).copy()
    rc = lib().oracle_dbyd2(_dp(a), _dp(b), n1, n2, int(ibc))
    if rc != 0:
        raise ValueError(f"dbyd2: ibc out of range ({ibc})")
    return a


def forward_source(p, nt: int) -> np.ndarray:
    out = np.zeros(nt)
    lib().oracle_forward_source(ctypes.byref(params_struct(p)), nt, _dp(out))
    return out


class Oracle:
    """One reference-equivalent solve on the CPU (FP64)."""

    def __init__(self, p, table: np.ndarray):
        self.p = p
        table = np.ascontiguousarray(table, dtype=np.float64)
        assert table.shape == (p.nz, 6)
        self._ps = params_struct(p)
        self.h = lib().oracle_create(ctypes.byref(self._ps), _dp(table))
        if not self.h:
            raise RuntimeError("oracle_create failed")
        self.shape = (p.nz, p.ny, p.nx)
        self.nf = 8 if p.option == 8 else 6          # fields of the state (dimfive, at least 6)

    def close(self):
        if self.h:
            lib().oracle_destroy(self.h)
            self.h = None

    __del__ = close

    def info(self) -> dict:
        out = np.zeros(64)
        n = lib().oracle_info(self.h, _dp(out))
        keys = ["e_rad", "o_rad", "delta_width", "deltat", "steps", "freq_filtering",
                "maxtime", "forcing_length", "cadforcing_step", "num_steps",
                "beta1", "beta2", "beta3", "beta4", "beta5", "stretchx", "stretchy",
                "pi", "rsun", "dimc", "dimrho", "diml"]
        return dict(zip(keys, out[:n].tolist()))

    def profiles(self) -> dict:
        nz = self.p.nz
        out = np.zeros(9 * nz)
        lib().oracle_profiles(self.h, _dp(out))
        names = ["stretch", "unstretch", "g", "gradp0_z", "gradrho0_z", "az", "bzpml", "rho0", "c2"]
        return {k: out[i * nz:(i + 1) * nz].copy() for i, k in enumerate(names)}

    def damping_rates(self) -> np.ndarray:
        h = self.p.nx // 2 + 1
        out = np.zeros(h * self.p.ny)
        lib().oracle_damping_rates(self.h, _dp(out))
        return out.reshape(self.p.ny, h)

    def set_source(self, mode: int, planes: np.ndarray, series: np.ndarray | None = None):
        planes = np.ascontiguousarray(planes, dtype=np.float64)
        L = planes.shape[0] if planes.ndim == 3 else 1
        if series is None:
            lib().oracle_set_source(self.h, mode, _dp(planes), L, None, 0)
        else:
            series = np.ascontiguousarray(series, dtype=np.float64)
            lib().oracle_set_source(self.h, mode, _dp(planes), L, _dp(series), len(series))

    def set_state(self, a: np.ndarray, pml: np.ndarray | None = None):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != self.nf * int(np.prod(self.shape)):
            raise ValueError(f"state must hold {self.nf} x {self.shape}")
        if pml is not None:
            pml = np.ascontiguousarray(pml, dtype=np.float64)
            if pml.size != self.npv * self.p.nzpml * self.p.ny * self.p.nx:
                raise ValueError(f"PML state must be ({self.npv}, {self.p.nzpml}, {self.p.ny}, {self.p.nx})")
        lib().oracle_set_state(self.h, _dp(a), _dp(pml) if pml is not None else None)

    @property
    def npv(self) -> int:
        """PML auxiliary fields: 6 for the MHD forms (options 8, 10, 18), else 2."""
        return 6 if self.p.option in (8, 10, 18) else 2

    def set_mhd(self, rho, c, p, bx, by, bz):
        """3-D cgs background of options 8 and 10 (as READ_IN_FIELD reads it), (nz, ny, nx)."""
        arrs = [np.ascontiguousarray(v, dtype=np.float64).reshape(self.shape) for v in (rho, c, p, bx, by, bz)]
        if lib().oracle_set_mhd(self.h, *[_dp(v) for v in arrs]) != 0:
            raise RuntimeError("oracle_set_mhd needs option 8 or 10")

    def set_mhd2d(self, rho, c, p, psi):
        """2-D MHD background of option 18, (nz, nx) cgs: density, sound speed,
        pressure and the vector potential psi (G R_sun) whose curl is B."""
        arrs = [np.ascontiguousarray(v, dtype=np.float64).reshape(self.shape) for v in (p, rho, c, psi)]
        if lib().oracle_set_mhd2d(self.h, *[_dp(v) for v in arrs]) != 0:
            raise RuntimeError("oracle_set_mhd2d needs option 18")

    def mhd_profiles(self) -> dict:
        out = np.zeros((15,) + self.shape)
        if lib().oracle_mhd_profiles(self.h, _dp(out)) != 0:
            raise RuntimeError("no MHD background")
        names = ["box", "boy", "boz", "curlbox", "curlboy", "curlboz", "gradrho0_x", "gradrho0_y",
                 "gradp0_x", "gradp0_y", "gradrho0_z", "gradp0_z", "az", "bzpml", "spongexyz"]
        return dict(zip(names, out))

    def state(self):
        p = self.p
        a = np.zeros((self.nf,) + self.shape)
        scr = np.zeros((self.nf,) + self.shape)
        pml = np.zeros((self.npv, max(p.npmlbot + p.npmltop, 1), p.ny, p.nx))
        lib().oracle_get_state(self.h, _dp(a), _dp(pml), _dp(scr))
        return a, scr, pml

    def step(self, n: int = 1) -> int:
        return lib().oracle_step(self.h, int(n))

    def set_time(self, t: int):
        lib().oracle_set_time(self.h, int(t))

    def ddx(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64); d = np.zeros_like(v)
        lib().oracle_ddx(self.h, _dp(v), _dp(d)); return d

    def ddy(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64); d = np.zeros_like(v)
        lib().oracle_ddy(self.h, _dp(v), _dp(d)); return d

    def ddz(self, v, bc, d_init=None):
        v = np.ascontiguousarray(v, dtype=np.float64)
        d = np.zeros_like(v) if d_init is None else np.ascontiguousarray(d_init, dtype=np.float64).copy()
        lib().oracle_ddz(self.h, _dp(v), _dp(d), int(bc)); return d

    def damp(self, v, rhs):
        v = np.ascontiguousarray(v, dtype=np.float64)
        r = np.ascontiguousarray(rhs, dtype=np.float64).copy()
        lib().oracle_damp(self.h, _dp(v), _dp(r)); return r

    def kernel_reset(self):
        lib().oracle_kernel_reset(self.h)

    def kernel_accumulate(self, fwd: np.ndarray, adj: np.ndarray, grav_raw: np.ndarray):
        fwd = np.ascontiguousarray(fwd, dtype=np.float64)
        adj = np.ascontiguousarray(adj, dtype=np.float64)
        grav_raw = np.ascontiguousarray(grav_raw, dtype=np.float64)
        lib().oracle_kernel_accumulate(self.h, _dp(fwd), _dp(adj), _dp(grav_raw))

    def kernel_finish(self, stepskern: int) -> np.ndarray:
        out = np.zeros((3,) + self.shape)
        lib().oracle_kernel_finish(self.h, _dp(out), int(stepskern))
        return out

    def kernel_accumulate_b(self, fxi: np.ndarray, av: np.ndarray):
        """One pass of the B-field kernel (kernels.f90:337-453) of the 2-D MHD
        form: forward displacement and adjoint velocity, each (3, nz, ny, nx)."""
        fxi = np.ascontiguousarray(fxi, dtype=np.float64)
        av = np.ascontiguousarray(av, dtype=np.float64)
        if lib().oracle_kernel_accumulate_b(self.h, _dp(fxi), _dp(av)) != 0:
            raise RuntimeError("B-field kernels need the 2-D MHD background (option 18)")

    def kernel_finish_b(self, stepskern: int) -> np.ndarray:
        """(kernel_bx, kernel_bz, kernel_vectorpsi), kernels.f90:498-514."""
        out = np.zeros((3,) + self.shape)
        if lib().oracle_kernel_finish_b(self.h, _dp(out), int(stepskern)) != 0:
            raise RuntimeError("no B-field kernel accumulation")
        return out


# ---------------------------------------------------------------------------
# numpy twins (cross-checks of the C++ restatement)
# ---------------------------------------------------------------------------
def R4(x):
    return float(np.float32(x))


def dbyd2_numpy(b: np.ndarray, ibc: int) -> np.ndarray:
    """numpy restatement of DBYD2 (dbyd2.f90:88-201) for ibc in {0, 1}; b is
    (N2, N1).  Solves the tridiagonal system densely (independent of the
    Thomas recurrence of mtridag.f90)."""
    b = np.asarray(b, dtype=np.float64)
    n2 = b.shape[0]
    d2i = float(n2 - 1)
    a = np.zeros_like(b)
    c1, c2 = d2i * 7.0 / 9.0, d2i / 36.0
    a[2:n2 - 2] = c1 * (b[3:n2 - 1] - b[1:n2 - 3]) + c2 * (b[4:n2] - b[0:n2 - 4])
    f32 = np.float32
    C1 = -float(f32(43.0) / f32(96.0)) * d2i
    C2 = -float(f32(5.0) / f32(6.0)) * d2i
    C3 = float(f32(9.0) / f32(8.0)) * d2i
    C4 = float(f32(1.0) / f32(6.0)) * d2i
    C5 = -float(f32(1.0) / f32(96.0)) * d2i
    a[1] = C1 * b[0] + C2 * b[1] + C3 * b[2] + C4 * b[3] + C5 * b[4]
    a[n2 - 2] = -(C1 * b[n2 - 1] + C2 * b[n2 - 2] + C3 * b[n2 - 3] + C4 * b[n2 - 4] + C5 * b[n2 - 5])
    F1 = -float(f32(10.0) / f32(3.0)) * d2i
    F2, F3 = -3.0 * d2i, 6.0 * d2i
    F4 = float(f32(1.0) / f32(3.0)) * d2i
    if ibc == 0:
        a[0] = 0.0
        a[n2 - 1] = 0.0
    else:
        a[0] = F1 * b[0] + F2 * b[1] + F3 * b[2] + F4 * b[3]
        a[n2 - 1] = -(F1 * b[n2 - 1] + F2 * b[n2 - 2] + F3 * b[n2 - 3] + F4 * b[n2 - 4])
    alpha = float(f32(1.0) / f32(3.0))
    alpha2, gamma2, alpha1, beta1 = 0.75, 0.125, 6.0, 3.0
    const = 1.0 / (alpha2 - beta1 * gamma2)
    up1 = (alpha1 * alpha2 - beta1) * const
    if ibc % 2:
        a[0] = (alpha2 * a[0] - beta1 * a[1]) * const
        a[n2 - 1] = (alpha2 * a[n2 - 1] - beta1 * a[n2 - 2]) * const
    uppr = np.zeros(n2)
    uppr[2:n2 - 2] = alpha
    uppr[0] = up1 if ibc % 2 else 0.0
    uppr[1] = alpha2
    uppr[n2 - 2] = gamma2
    lowr = uppr[::-1].copy()
    lowr[n2 - 1] = up1 if ibc in (1, 2) else 0.0
    M = np.eye(n2)
    for j in range(n2 - 1):
        M[j, j + 1] = uppr[j]
    for j in range(1, n2):
        M[j, j - 1] = lowr[j]
    return np.linalg.solve(M, a.reshape(n2, -1)).reshape(b.shape)


def fft_ddx_numpy(v: np.ndarray, stretchx: float, pi_r4: float) -> np.ndarray:
    """numpy twin of ddx (derivatives.f90:28-58) on the last axis: FFTW r2c x
    eyekx, c2r (Nyquist dropped), times stretchx."""
    nx = v.shape[-1]
    spec = np.fft.rfft(v, axis=-1)
    k = np.arange(nx // 2 + 1, dtype=np.float64)
    eyek = 1j * k * (1.0 / nx) * 2.0 * pi_r4
    spec = spec * eyek * nx
    spec[..., 0] = spec[..., 0].real
    if nx % 2 == 0:
        spec[..., -1] = spec[..., -1].real
    return np.fft.irfft(spec, n=nx, axis=-1) * stretchx
