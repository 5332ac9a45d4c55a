"""Host-side mirror of the reference's time-stepping interface.

``Solver`` owns one library context (one or many sources on the source axis)
and exposes the operations the reference performs inside its executable:
Initialize_all + solar_data + mp_Initialize_RHS + Initialize_step
(constructor), DETERMINE_STATUS source set-up (``set_source_*``), the
TIMESTEPPING loop body (``step``), the vz_cc.bin stream (``record_surface`` /
``records``), WRITE_OUT_PARTIAL_STATE fields (``field``), checkpoints, and the
sensitivity-kernel accumulation of kernels.f90.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .params import SparcParams

_D = ctypes.POINTER(ctypes.c_double)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _dpn(a):
    return None if a is None else a.ctypes.data_as(_D)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class Solver:
    """One GPU solve (or a batch of ``p.nsrc`` solves sharing one background)."""

    XI_X, XI_Y, XI_Z, V_X, V_Y, V_Z = range(6)

    def __init__(self, p: SparcParams, table: np.ndarray):
        p.validate()
        self.p = p
        self.L = native.load()
        self._cp = native.c_params(p)
        h = ctypes.c_void_p()
        rc = self.L.sparc_gpu_create(ctypes.byref(self._cp), ctypes.byref(h))
        if rc != 0:
            raise native.SparcError(rc, self.L.sparc_gpu_errstr(rc).decode())
        self.h = h
        self.shape = (p.nz, p.ny, p.nx)
        self.set_background(table)

    # ---- plumbing ----
    def _ck(self, rc: int):
        if rc != 0:
            msg = self.L.sparc_gpu_last_error(self.h).decode() if self.h else ""
            raise native.SparcError(rc, f"{self.L.sparc_gpu_errstr(rc).decode()}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.sparc_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- set-up ----
    def set_background(self, table: np.ndarray):
        t = _f64(table)
        if t.shape != (self.p.nz, 6):
            raise ValueError(f"background table must be ({self.p.nz}, 6)")
        cols = [_f64(t[:, i]) for i in range(6)]
        self._ck(self.L.sparc_gpu_set_background(self.h, *[_dp(c) for c in cols]))

    def info(self) -> dict:
        out = np.zeros(16)
        self._ck(self.L.sparc_gpu_info(self.h, _dp(out), None, None))
        keys = ["e_rad", "o_rad", "delta_width", "deltat", "steps", "freq_filtering", "maxtime",
                "forcing_length", "cadforcing_step", "num_steps", "beta1", "beta2", "beta3", "beta4", "beta5"]
        d = dict(zip(keys, out[:15].tolist()))
        for k in ("e_rad", "o_rad", "steps", "freq_filtering", "maxtime", "forcing_length",
                  "cadforcing_step", "num_steps"):
            d[k] = int(d[k])
        return d

    def tables(self):
        zt = np.zeros(native.ZTAB_ROWS * self.p.nz)
        m = self.p.ny * (self.p.nx // 2 + 1)
        pt = np.zeros(native.PTAB_ROWS * m)
        self._ck(self.L.sparc_gpu_info(self.h, None, _dp(zt), _dp(pt)))
        return zt.reshape(native.ZTAB_ROWS, self.p.nz), pt.reshape(native.PTAB_ROWS, m)

    def set_source_series(self, plane: np.ndarray, series: np.ndarray, slot: int = 0):
        """forcing(x, y, t_n) = plane(x, y) * series[n], injected at the source plane."""
        pl = _f64(plane).reshape(1, self.p.ny, self.p.nx)
        se = _f64(series)
        self._ck(self.L.sparc_gpu_set_source(self.h, slot, native.SRC_SERIES, _dp(pl), 1, _dp(se), len(se)))

    def set_source_lagrange(self, planes: np.ndarray, slot: int = 0):
        """vr(:,:,1..L) sampled every cadforcing seconds (LAGRANGE_INTERP)."""
        pl = _f64(planes).reshape(-1, self.p.ny, self.p.nx)
        self._ck(self.L.sparc_gpu_set_source(self.h, slot, native.SRC_LAGRANGE, _dp(pl), pl.shape[0], None, 0))

    def clear_source(self, slot: int = 0):
        self._ck(self.L.sparc_gpu_set_source(self.h, slot, native.SRC_NONE, None, 0, None, 0))

    # ---- stepping ----
    def step(self, n: int = 1):
        self._ck(self.L.sparc_gpu_step(self.h, int(n)))

    def autotune(self, steps: int = 1) -> dict:
        """Time each launch variant that gives identical results over real
        steps (4*steps of them) and keep the fastest; returns the choice."""
        choice = ctypes.c_int(0)
        ms = ctypes.c_float(0.0)
        self._ck(self.L.sparc_gpu_autotune(self.h, int(steps), ctypes.byref(choice), ctypes.byref(ms)))
        key = "modes_per_cta" if (self.p.precision == "f32" and self.p.nz <= 320) else "threads_per_cta"
        return {key: choice.value, "ms_per_step": ms.value}

    def stage(self, rk: int):
        """Launch only RK stage rk (1..5) of the current step (timing hook)."""
        self._ck(self.L.sparc_gpu_stage(self.h, int(rk)))

    @property
    def time(self) -> int:
        t = ctypes.c_int()
        self._ck(self.L.sparc_gpu_get_time(self.h, ctypes.byref(t)))
        return t.value

    @time.setter
    def time(self, t: int):
        self._ck(self.L.sparc_gpu_set_time(self.h, int(t)))

    def sync(self, check_finite: bool = False):
        self._ck(self.L.sparc_gpu_sync(self.h, int(check_finite)))

    @property
    def stream_ptr(self) -> int:
        return self.L.sparc_gpu_stream(self.h) or 0

    @property
    def launches(self) -> int:
        return int(self.L.sparc_gpu_launch_count(self.h))

    @property
    def device_bytes(self) -> int:
        return int(self.L.sparc_gpu_device_bytes(self.h))

    # ---- state ----
    def field(self, f: int, slot: int = 0, k: int = 0) -> np.ndarray:
        shape = (self.p.ny, self.p.nx) if k > 0 else self.shape
        out = np.zeros(shape)
        self._ck(self.L.sparc_gpu_get_field(self.h, slot, f, k, _dp(out)))
        return out

    @property
    def npv(self) -> int:
        """PML auxiliary fields: six for the MHD forms (options 8, 10, 18), else two."""
        return 6 if self.p.option in (8, 10, 18) else 2

    @property
    def nf(self) -> int:
        """Fields of the state: eight in the MHD velocity form (option 8:
        rho, v_x, v_y, v_z, p, b_x, b_y, b_z), else six."""
        return 8 if self.p.option == 8 else 6

    def set_mhd_background(self, rho, c, p, bx, by, bz):
        """3-D cgs background of options 8 and 10 (density, sound speed,
        pressure, B_x, B_y, B_z), each (nz, ny, nx); set_background's quiet
        column is the one the source planes are searched on."""
        arrs = [_f64(np.asarray(v, dtype=np.float64).reshape(self.shape)) for v in (rho, c, p, bx, by, bz)]
        self._ck(self.L.sparc_gpu_set_mhd_background(self.h, *[_dp(v) for v in arrs]))

    def set_mhd2d_background(self, rho, c, p, psi):
        """2-D cgs background of option 18 (density, sound speed, pressure and
        the vector potential psi), each (nz, 1, nx) or (nz, nx)."""
        arrs = [_f64(np.asarray(v, dtype=np.float64).reshape(self.shape)) for v in (rho, c, p, psi)]
        self._ck(self.L.sparc_gpu_set_mhd2d_background(self.h, *[_dp(v) for v in arrs]))

    def state(self, slot: int = 0):
        a = np.zeros((self.nf,) + self.shape)
        pml = np.zeros((self.npv, self.p.nzpml, self.p.ny, self.p.nx))
        self._ck(self.L.sparc_gpu_get_state(self.h, slot, _dp(a), _dp(pml)))
        return a, pml

    def set_state(self, a: np.ndarray, pml: np.ndarray | None = None, slot: int = 0):
        a = _f64(a)
        if a.shape != (self.nf,) + self.shape:
            raise ValueError(f"state must be ({self.nf}, nz, ny, nx)")
        pp = None
        if pml is not None:
            pml = _f64(pml)
            if pml.shape != (self.npv, self.p.nzpml, self.p.ny, self.p.nx):
                raise ValueError(f"PML state must be ({self.npv}, {self.p.nzpml}, {self.p.ny}, {self.p.nx})")
            pp = _dp(pml)
        self._ck(self.L.sparc_gpu_set_state(self.h, slot, _dp(a), pp))

    def record_surface(self, max_records: int, enable: bool = True):
        self._ck(self.L.sparc_gpu_record_surface(self.h, int(enable), int(max_records)))

    def records(self, slot: int = 0) -> np.ndarray:
        n = ctypes.c_int()
        self._ck(self.L.sparc_gpu_get_records(self.h, slot, None, ctypes.byref(n)))
        out = np.zeros((n.value, self.p.ny, self.p.nx))
        if n.value:
            self._ck(self.L.sparc_gpu_get_records(self.h, slot, _dp(out), ctypes.byref(n)))
        return out

    def checkpoint(self, path: str):
        self._ck(self.L.sparc_gpu_checkpoint(self.h, path.encode()))

    def restore(self, path: str):
        self._ck(self.L.sparc_gpu_restore(self.h, path.encode()))

    # ---- continuous batching ----
    def slot_reset(self, slot: int):
        self._ck(self.L.sparc_gpu_slot_reset(self.h, int(slot)))

    def slot_time(self, slot: int) -> int:
        t = ctypes.c_int()
        self._ck(self.L.sparc_gpu_slot_time(self.h, int(slot), ctypes.byref(t)))
        return t.value

    def set_active(self, n: int):
        self._ck(self.L.sparc_gpu_set_active(self.h, int(n)))

    def set_stream_priority(self, level: int):
        """Scheduling priority of this context's stream(s): 0 is the default,
        higher levels are more urgent (clamped to the device's range)."""
        self._ck(self.L.sparc_gpu_set_stream_priority(self.h, int(level)))

    def busy(self) -> bool:
        """True while work queued on this context's stream has not finished
        (non-blocking)."""
        b = ctypes.c_int(0)
        self._ck(self.L.sparc_gpu_query(self.h, ctypes.byref(b)))
        return bool(b.value)

    def set_rhs_output(self, on: bool):
        """Whether each step call's last step leaves its right-hand side in
        scr (default True; the forward snapshot needs it, an adjoint context
        of the kernel workflow does not)."""
        self._ck(self.L.sparc_gpu_set_rhs_output(self.h, int(bool(on))))

    def save_device(self, idx: int, capacity: int):
        self._ck(self.L.sparc_gpu_save_device(self.h, int(idx), int(capacity)))

    def load_device(self, idx: int):
        self._ck(self.L.sparc_gpu_load_device(self.h, int(idx)))

    # ---- primitives ----
    def ddx(self, v):
        v = _f64(v); d = np.zeros_like(v)
        self._ck(self.L.sparc_gpu_ddx(self.h, _dp(v), _dp(d))); return d

    def ddy(self, v):
        v = _f64(v); d = np.zeros_like(v)
        self._ck(self.L.sparc_gpu_ddy(self.h, _dp(v), _dp(d))); return d

    def ddz(self, v, bc: int, d_init=None):
        v = _f64(v)
        d = np.zeros_like(v) if d_init is None else _f64(d_init).copy()
        self._ck(self.L.sparc_gpu_ddz(self.h, _dp(v), _dp(d), int(bc))); return d

    def damp(self, v, rhs):
        v = _f64(v); r = _f64(rhs).copy()
        self._ck(self.L.sparc_gpu_damp(self.h, _dp(v), _dp(r))); return r

    # ---- sensitivity kernels ----
    def snapshot(self, snap: int, nsnap: int):
        self._ck(self.L.sparc_gpu_snapshot(self.h, int(snap), int(nsnap)))

    def kernel_reset(self):
        self._ck(self.L.sparc_gpu_kernel_reset(self.h))

    def kernel_accumulate(self, fwd: "Solver", snap: int):
        self._ck(self.L.sparc_gpu_kernel_accumulate(fwd.h, int(snap), self.h))

    def kernels(self, slot: int = 0, sum_slots: bool = False):
        kc = np.zeros(self.shape); kr = np.zeros(self.shape); hs = np.zeros(self.shape)
        self._ck(self.L.sparc_gpu_kernels(self.h, slot, int(sum_slots), _dp(kc), _dp(kr), _dp(hs)))
        return kc, kr, hs

    def adjoint_source(self, data, x00: float, t1_min: float, dt_min: float, ridges: dict, bands: dict,
                       windows: dict | None = None, slot: int = 0, nt: int | None = None, synth=None):
        """ADJOINT_SOURCE_FILT (driver.f90:1262-1686) of a 2-D run on the GPU,
        from this context's surface records of `slot` (the synthetic) and the
        observed data (nt, nx).  ridges: {0, 1, 2} -> (mindist, maxdist,
        window) of params.0..2; bands: {0, 1} -> (left, right) mHz of
        filter.params.0/1; windows: {0, 1} -> {pixel: (lef, rig)} of a line
        search, else None; synth: a synthetic (nt, nx) from the host instead
        of the records.  Returns (adj (nt, nx), misfit, nmeas, windows)."""
        data = _f64(np.asarray(data, dtype=np.float64))
        nt = data.shape[0] if nt is None else int(nt)
        nx = self.p.nx
        if data.shape != (nt, nx):
            raise ValueError(f"data must be ({nt}, {nx})")
        ap = native.CAdjSrcParams()
        ap.x00, ap.t1_min, ap.dt_min = float(x00), float(t1_min), float(dt_min)
        for m in range(3):
            ap.have_ridge[m] = int(m in ridges)
            for q, v in enumerate(ridges.get(m, (0.0, 0.0, 0.0))):
                ap.ridge[m][q] = float(v)
        for m in range(2):
            ap.have_band[m] = int(m in bands)
            for q, v in enumerate(bands.get(m, (0.0, 0.0))):
                ap.band[m][q] = float(v)
        ap.linesearch = int(windows is not None)
        win = np.zeros((2, nx, 2), dtype=np.int32)
        if windows is not None:
            for m in (0, 1):
                for i, (lef, rig) in windows.get(m, {}).items():
                    win[m, i] = (lef, rig)
        adj = np.zeros((nt, nx))
        mis = ctypes.c_double()
        nm = ctypes.c_int()
        wp = win.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        if synth is None:
            self._ck(self.L.sparc_gpu_adjoint_source(self.h, slot, _dp(data), nt, ctypes.byref(ap), wp, _dp(adj),
                                                     ctypes.byref(mis), ctypes.byref(nm)))
        else:
            synth = _f64(np.asarray(synth, dtype=np.float64))
            if synth.shape != (nt, nx):
                raise ValueError(f"synthetic must be ({nt}, {nx})")
            self._ck(self.L.sparc_gpu_adjoint_source_host(self.h, _dp(synth), _dp(data), nt, ctypes.byref(ap), wp,
                                                          _dp(adj), ctypes.byref(mis), ctypes.byref(nm)))
        wout = {m: {i: (int(win[m, i, 0]), int(win[m, i, 1])) for i in range(nx) if win[m, i, 0] > 0}
                for m in (0, 1)}
        return adj, mis.value, nm.value, wout

    def misfit_all(self, data, x00: float, t1_min: float, dt_min: float, ridges: dict,
                   windows: dict | None = None, slot: int = 0, nt: int | None = None, synth=None):
        """MISFIT_ALL (driver.f90:1702-2076) of a 2-D run on the GPU.  Returns
        (misfit (3 bands, 3 sets) = 0.5 sum tau^2, nmeas (3, 3), windows
        {(band, set): {pixel: (lef, rig)}}); windows given -> line search."""
        data = _f64(np.asarray(data, dtype=np.float64))
        nt = data.shape[0] if nt is None else int(nt)
        nx = self.p.nx
        ap = native.CAdjSrcParams()
        ap.x00, ap.t1_min, ap.dt_min = float(x00), float(t1_min), float(dt_min)
        for m in range(3):
            ap.have_ridge[m] = int(m in ridges)
            for q, v in enumerate(ridges.get(m, (0.0, 0.0, 0.0))):
                ap.ridge[m][q] = float(v)
        ap.linesearch = int(windows is not None)
        win = np.zeros((3, 2, nx, 2), dtype=np.int32)
        if windows is not None:
            for (b, m), d in windows.items():
                for i, (lef, rig) in d.items():
                    win[b, m, i] = (lef, rig)
        mis = np.zeros((3, 3))
        nm = np.zeros((3, 3), dtype=np.int32)
        sp = None
        if synth is not None:
            synth = _f64(np.asarray(synth, dtype=np.float64))
            sp = _dp(synth)
        self._ck(self.L.sparc_gpu_misfit_all(self.h, slot, sp, _dp(data), nt, ctypes.byref(ap),
                                             win.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(mis),
                                             nm.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        wout = {(b, m): {i: (int(win[b, m, i, 0]), int(win[b, m, i, 1])) for i in range(nx) if win[b, m, i, 0] > 0}
                for b in range(3) for m in (0, 1) if m in ridges}
        return mis, nm.astype(int), wout

    def gradient(self, kc_sum, kpsi_sum, hess_sum, rho_z):
        """grad.py:152-186 on the GPU: (gradient_c, gradient_vectorpsi) from the
        kernels summed over sources, the summed |hessian| and the density
        column rho_z of the background.  A kernel sum given as None skips its
        gradient (returned as None)."""
        hs = _f64(hess_sum)
        rz = _f64(rho_z)
        if hs.shape != self.shape or rz.shape != (self.p.nz,):
            raise ValueError(f"hess_sum must be {self.shape} and rho_z ({self.p.nz},)")
        kc = None if kc_sum is None else _f64(kc_sum)
        kp = None if kpsi_sum is None else _f64(kpsi_sum)
        for a in (kc, kp):
            if a is not None and a.shape != self.shape:
                raise ValueError(f"kernel sums must be {self.shape}")
        gc = None if kc is None else np.zeros(self.shape)
        gp = None if kp is None else np.zeros(self.shape)
        self._ck(self.L.sparc_gpu_gradient(self.h, _dpn(kc), _dpn(kp), _dp(hs), _dp(rz), _dpn(gc), _dpn(gp)))
        return gc, gp

    def update_models(self, grad_c, grad_psi, model_psi, last=None, eps: float = 1e-7, nmodels: int = 5):
        """grad.py:188-301 on the GPU: the update direction (steepest descent,
        or conjugate gradient with last = (last gradient_vectorpsi, last
        update_c, last update_vectorpsi)) and the line-search test models.
        Returns (update_c or None, update_psi, test_psi (nmodels, ...), con)."""
        gp = _f64(grad_psi)
        gc = None if grad_c is None else _f64(grad_c)
        mp = _f64(model_psi)
        arrs = [gp, mp] + ([] if gc is None else [gc])
        lg = lc = lp = None
        if last is not None:
            lg, lc, lp = (None if a is None else _f64(a) for a in last)
            arrs += [a for a in (lg, lc, lp) if a is not None]
        for a in arrs:
            if a.shape != self.shape:
                raise ValueError(f"fields must be {self.shape}")
        uc = None if gc is None else np.zeros(self.shape)
        up = np.zeros(self.shape)
        tp = np.zeros((int(nmodels),) + self.shape)
        con = ctypes.c_double(0.0)
        self._ck(self.L.sparc_gpu_update_models(self.h, _dpn(gc), _dp(gp), _dpn(lg), _dpn(lc), _dpn(lp), _dp(mp),
                                                float(eps), int(nmodels), _dpn(uc), _dp(up),
                                                _dp(tp) if nmodels > 0 else None,
                                                ctypes.cast(ctypes.pointer(con), _D)))
        return uc, up, tp, con.value

    def kernels_into(self, dev_ptr: int, slot: int = 0, sum_slots: bool = False):
        """Final kernels (K_c, K_rho, hessian; 3 x (nz, ny, nx) doubles) into
        the device buffer at dev_ptr, enqueued on this context's stream (the
        caller orders its own reads after that stream)."""
        self._ck(self.L.sparc_gpu_kernels_device(self.h, slot, int(sum_slots), ctypes.c_void_p(int(dev_ptr))))

    def kernels_b(self, slot: int = 0, sum_slots: bool = False):
        """Option 18: (kernel_bx, kernel_bz, kernel_vectorpsi) of the adjoint context."""
        kx = np.zeros(self.shape); kz = np.zeros(self.shape); kp = np.zeros(self.shape)
        self._ck(self.L.sparc_gpu_kernels_b(self.h, slot, int(sum_slots), _dp(kx), _dp(kz), _dp(kp)))
        return kx, kz, kp
