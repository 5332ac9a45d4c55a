"""Benchmark: grid-point-steps/s of the SPARC time step at 256x256x300.

Workload (synthetic inputs, seeded): quiet-Sun polytrope box 256x256x300,
200 Mm periodic, PML 10 top + 10 bottom, dt = 2 s.  One bench *step* = one
time step of the forward solve AND one time step of the adjoint solve for
every source on the source axis, with the sensitivity-kernel snapshot /
accumulation (FP64 accumulators) at the 30 s output cadence, as in a
forward x adjoint kernel run.  Point-steps per bench step = 2 * nsrc * N.

  value       batched FP32 fields (FP64 set-up and kernel accumulation),
              nsrc sources in one launch per kernel, inputs resident in HBM
  fp64_plain  the plain single-source FP64 solve, same workload
  e2e         batched FP32 through the public API with host buffers: source
              upload (H2D), the steps, seismogram + summed-kernel read-back (D2H)
  roofline    the dominant kernel (the fused FP32 step, batched) against the
              measured HBM copy bandwidth
  cpu_baseline  the FP64 CPU oracle (a restatement of the reference) on a
              bounded sample (rank 0, N = 1)

--impl reference times the CPU oracle on the same configuration with all host
threads (the reference itself is Fortran/MPI/FFTW and cannot be built here).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpoint-steps/s at 256^2x300, batched FP32 vs plain FP64; p50/p99 solve latency"
UNIT = "Mpoint-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nsrc", type=int, default=32)
    ap.add_argument("--nplanes", type=int, default=64, help="adjoint source samples per source")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--small", action="store_true", help="128x128x150 smoke-size workload")
    ap.add_argument("--skip-mhd", action="store_true", help="skip the flux-tube (option 10) line")
    ap.add_argument("--mhd-only", action="store_true",
                    help="only the flux-tube line (--steps timed, --warmup untimed), for profiling")
    ap.add_argument("--mhd-prec", default="f64,f32", help="precisions of the flux-tube line")
    ap.add_argument("--mhd-grid", default="", help="NXxNYxNZ of the flux-tube line (default: the bench grid)")
    ap.add_argument("--serve-requests", type=int, default=32, help="requests of the serving stream (0: skip)")
    ap.add_argument("--serve-compress", type=float, default=120.0, help="request-length compression")
    ap.add_argument("--full-length", default="", choices=["", "config4", "config3", "serving"],
                    help="one full-length workload instead of the bench line (see full_length_*)")
    ap.add_argument("--fl-hours", type=float, default=0.0,
                    help="solar hours of the full-length run (0: the configuration's own; a short check otherwise)")
    return ap.parse_args()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x: float) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(small: bool):
    from sparc_gb300.background import polytrope_table
    from sparc_gb300.params import config_quiet_128, config_quiet_256
    p = config_quiet_128() if small else config_quiet_256()
    return p, polytrope_table(p.nz)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during a timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"sparc_bench_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def source_inputs(p, nplanes, gi, seed=0):
    """Seeded inputs of global source gi: forward source plane (a Gaussian at
    a random surface position) and adjoint residuals at the receivers."""
    from sparc_gb300 import sources
    rng = np.random.default_rng([seed, gi])
    x0, y0 = rng.uniform(-60, 60, size=2)
    pix = sources.receiver_pixels(p)
    res = rng.standard_normal((len(pix), nplanes)) * 1e-6
    return sources.gaussian_plane(p, 1.0, x0, y0), sources.adjoint_planes(p, res, pix)


def make_pair(p, tab, nplanes, src_ids, seed=0):
    """Forward and adjoint solvers with the seeded sources src_ids (global
    indices, one per slot)."""
    from sparc_gb300 import sources
    from sparc_gb300.solver import Solver
    pa = p.replace(compute_forward=False, compute_adjoint=True)
    fwd, adj = Solver(p, tab), Solver(pa, tab)
    adj.set_rhs_output(False)          # the adjoint side of the kernel snapshot reads no scr
    series = sources.ricker_series(p, 20000)
    for s, gi in enumerate(src_ids):
        plane, adjp = source_inputs(p, nplanes, gi, seed)
        fwd.set_source_series(plane, series, slot=s)
        adj.set_source_lagrange(adjp, slot=s)
    return fwd, adj


def run_steps(fwd, adj, nsteps, cad, nsnap_ring=2):
    """nsteps bench steps: forward and adjoint advance in chunks that end on
    the output cadence, where the forward snapshot is stored and the adjoint
    accumulates the kernels against it."""
    done = 0
    while done < nsteps:
        t = fwd.time
        n = min(cad - (t % cad), nsteps - done)
        fwd.step(n)
        adj.step(n)
        done += n
        if fwd.time % cad == 0:
            slot = (fwd.time // cad) % nsnap_ring
            fwd.snapshot(slot, nsnap_ring)
            adj.kernel_accumulate(fwd, slot)


def timed_region(fwd, adj, steps, cad):
    """Device time of `steps` bench steps across both contexts' streams."""
    import torch
    sf = torch.cuda.ExternalStream(fwd.stream_ptr)
    sa = torch.cuda.ExternalStream(adj.stream_ptr)
    torch.cuda.synchronize()
    fwd.sync(); adj.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ea = torch.cuda.Event()
    e0.record(sf)
    sa.wait_event(e0)
    l0 = fwd.launches + adj.launches
    run_steps(fwd, adj, steps, cad)
    ea.record(sa)
    sf.wait_event(ea)
    e1.record(sf)
    e1.synchronize()
    torch.cuda.synchronize()
    launches = fwd.launches + adj.launches - l0
    return e0.elapsed_time(e1), launches


def step_kernel_time(solver, n=15, reps=2):
    """Average duration of one time-step launch (the fused FP32 step kernel is
    the only kernel of a step), CUDA events on the launching stream."""
    import torch
    s = torch.cuda.ExternalStream(solver.stream_ptr)
    solver.sync()
    ts = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        solver.step(n)
        e1.record(s)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) / n)
    return float(np.min(ts))


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def issue_roofline(winst, launch_ms, clocks, sm_count):
    """Issue-side roofline of the fused step: warp instructions per launch
    (ncu, scaled by nsrc) over the launch time, against one warp instruction
    per cycle on each of the 4 schedulers of every SM at the sampled SM clock."""
    if not winst:
        return None
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not mhz:
        return None
    peak = sm_count * 4 * mhz * 1e6
    ach = winst / (launch_ms * 1e-3)
    return {"warp_inst_per_launch": winst, "achieved_ginst_s": ach / 1e9, "peak_ginst_s": peak / 1e9,
            "frac": ach / peak, "sm_mhz": mhz, "sms": sm_count,
            "source": "smsp__inst_executed.sum of one ncu capture of a single-source launch at this grid, "
                      "times nsrc"}


def serving_section(precision: str, n: int, compress: float, rate: float = 4.0, seed: int = 0,
                    max_wall: float = 240.0):
    """Config-5 stream: Poisson arrivals (rate/s) of 1-4 h forward or
    forward+adjoint requests on 128^2x150 / 256^2x300 / 512^2x300 (60/30/10 %),
    request lengths divided by `compress`.  Latency = finish - arrival (wall)."""
    from sparc_gb300.serving import Engine, latency_stats, poisson_stream
    import torch
    reqs = poisson_stream(n, rate=rate, seed=seed, compress=compress)
    budget = 0.85 * torch.cuda.mem_get_info()[0]          # HBM free at the start, with a margin
    eng = Engine(precision=precision, hbm_budget=budget,
                 slots={(128, 128, 150): 8, (256, 256, 300): 4, (512, 512, 300): 2},
                 max_steps=max(r.nsteps for r in reqs))
    tw = time.perf_counter()
    npools = eng.warm()                  # contexts set up before the stream, as at server start
    warm_s = time.perf_counter() - tw
    t0 = time.perf_counter()
    try:
        done = eng.run(reqs, max_wall=max_wall)
    finally:
        eng.close()
    wall = time.perf_counter() - t0
    pts = sum(r.grid[0] * r.grid[1] * r.grid[2] * r.nsteps * (2 if r.kind == "fwd+adj" else 1) for r in done)
    st = latency_stats(done)
    st.update({"precision": precision, "Mpoint_steps_per_s": pts / wall / 1e6, "wall_s": wall,
               "compress": compress, "rate_per_s": rate, "hbm_budget_gb": budget / 1e9,
               "warm_pools": npools, "warm_s": warm_s,
               "flux_tube_requests": sum(r.background == "tube" for r in done)})
    return st


def config1_full():
    """The 1-h configuration at full length: plain FP64 forward of the
    128x128x150 quiet-Sun box, one source, time = 0..maxtime (1801 steps of
    2 s), the surface vz of every output (30 s) recorded on the device and
    read back at the end; device time with CUDA events."""
    import torch
    from sparc_gb300 import sources
    from sparc_gb300.background import polytrope_table
    from sparc_gb300.params import config_quiet_128
    from sparc_gb300.solver import Solver
    p = config_quiet_128().replace(precision="f64", nsrc=1)
    s = Solver(p, polytrope_table(p.nz))
    s.set_source_series(sources.gaussian_plane(p), sources.ricker_series(p, p.maxtime + 8))
    nrec = p.maxtime // p.steps + 1
    s.record_surface(nrec)
    st = torch.cuda.ExternalStream(s.stream_ptr)
    s.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(st)
    s.step(p.maxtime + 1)
    e1.record(st)
    rec = s.records()
    wall = time.perf_counter() - t0
    ms = e0.elapsed_time(e1)
    s.close()
    n = p.maxtime + 1
    return {"grid": [p.nx, p.ny, p.nz], "steps": n, "dtype": "f64", "records": int(rec.shape[0]),
            "device_s": ms * 1e-3, "wall_s": wall, "value": p.points * n / (ms * 1e-3) / 1e6, "unit": UNIT,
            "finite": bool(np.isfinite(rec).all())}


def small_step_latency(n=60):
    """Per-step device time of a 128x128x150 single-source FP32 forward solve
    (the 1-h configuration's grid), steps replayed from captured graphs vs
    launched one by one: where launch overhead is visible."""
    import torch
    from sparc_gb300 import sources
    from sparc_gb300.background import polytrope_table
    from sparc_gb300.params import config_quiet_128
    from sparc_gb300.solver import Solver
    p = config_quiet_128().replace(precision="f32", nsrc=1)
    tab = polytrope_table(p.nz)
    out = {}
    for mode in ("graphs", "direct"):
        if mode == "direct":
            os.environ["SPARC_NO_GRAPHS"] = "1"
        try:
            s = Solver(p, tab)
        finally:
            os.environ.pop("SPARC_NO_GRAPHS", None)
        s.set_source_series(sources.gaussian_plane(p), sources.ricker_series(p, 4000))
        s.record_surface(n // p.steps + 2)
        st = torch.cuda.ExternalStream(s.stream_ptr)
        s.step(p.steps)
        s.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(n // p.steps):
            s.step(p.steps)
        e1.record(st)
        e1.synchronize()
        out[mode + "_us_per_step"] = e0.elapsed_time(e1) * 1e3 / (n // p.steps * p.steps)
        s.close()
    out["grid"] = [p.nx, p.ny, p.nz]
    return out


def accuracy_section(solartime_h: float = 0.1, nsrc: int = 2):
    """Errors of the FP32 path against FP64 on the same inputs, as the bench
    states them for its results: the forward x adjoint kernel workflow on
    the 128x128x150 quiet-Sun box (sources 10 Mm apart, 8 receivers on a
    5 Mm ring, zero observations), FP32 fields with FP64 accumulation
    against the FP64 path (itself within 1e-10 of the CPU oracle).  Reports
    the relative L2 of the surface seismograms and of each kernel, and the
    largest travel-time shift (COMPUTE_TT) over the receivers the wave has
    reached (rms at least 1 % of the strongest)."""
    from sparc_gb300 import sources
    from sparc_gb300.background import polytrope_table
    from sparc_gb300.params import config_quiet_128
    from sparc_gb300.pipeline import KernelPipeline, compute_tt
    p = config_quiet_128().replace(solartime=solartime_h, nsrc=nsrc)
    tab = polytrope_table(p.nz)
    planes = [sources.gaussian_plane(p, 1.0, x0, 0.0) for x0 in (-5.0, 5.0)][:nsrc]
    series = sources.ricker_series(p, p.maxtime + 10)
    pix = sources.receiver_pixels(p, n=8, radius_mm=5.0)
    res = {}
    t0 = time.perf_counter()
    for prec in ("f64", "f32"):
        pl = KernelPipeline(p.replace(precision=prec), tab, segment=8)
        res[prec] = pl.run(planes, series, np.zeros((nsrc, pl.nt, p.ny, p.nx)), pix)
    a, b = res["f64"], res["f32"]

    def rel(x, y):
        return float(np.linalg.norm((x - y).ravel()) / max(np.linalg.norm(y.ravel()), 1e-300))

    dt = p.timestep * p.steps
    shifts = []
    for s in range(nsrc):
        rms = np.sqrt(np.mean(a.seismograms[s] ** 2, axis=0))
        for r in range(len(pix)):
            if rms[r] >= 1e-2 * rms.max():
                shifts.append(abs(compute_tt(a.seismograms[s, :, r], b.seismograms[s, :, r], dt)))
    return {"workload": f"kernel workflow, {p.nx}x{p.ny}x{p.nz}, {nsrc} sources, {p.maxtime + 1} steps "
                        f"({solartime_h} h), FP32 against FP64",
            "seismogram_rel_l2": rel(b.seismograms, a.seismograms),
            "kernel_rel_l2": {q: rel(getattr(b, q), getattr(a, q)) for q in ("kc", "krho", "hessian")},
            "max_tt_shift_s": float(max(shifts)) if shifts else None, "receivers_timed": len(shifts),
            "tolerances": {"seismogram_rel_l2": 1e-4, "tt_shift_s": 0.05},
            "wall_s": time.perf_counter() - t0}


def _hbm_peak() -> float:
    """Measured HBM copy bandwidth (GB/s) of MEASURED_PEAKS.json, else the fallback."""
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        return float(json.load(open(pk)).get("hbm_gbs", 6800.0))
    return 6800.0


def mhd_section(steps=5, warmup=2, precs=("f64", "f32"), grid=None, acc_steps=150):
    """The flux-tube configuration: linearised MHD (option 10) at 256x256x300
    on the magnetohydrostatic flux tube (2 kG and 3 Mm at its narrowest,
    box top at the surface), one source 20 Mm from the axis.  Per precision:
    device time per forward step (CUDA events on the context's stream, after
    `warmup` steps), then the run continued to acc_steps steps with surface
    records every output; FP32 is stated against FP64 on those records (the
    seismograms) and on the final state."""
    import torch
    from sparc_gb300 import bytes_model, sources
    from sparc_gb300.background import config3_background, polytrope_table
    from sparc_gb300.params import config_flux_tube_256
    from sparc_gb300.solver import Solver
    pm, tab = config_flux_tube_256()
    if grid:
        pm = pm.replace(nx=grid[0], ny=grid[1], nz=grid[2])
        tab = polytrope_table(grid[2], z_bot_mm=-25.0, z_top_mm=0.0)
    pm = pm.replace(nsrc=1)
    out = {"grid": [pm.nx, pm.ny, pm.nz]}
    bg = None
    res = {}
    for prec in precs:
        s = Solver(pm.replace(precision=prec), tab)
        if bg is None:
            t0 = time.perf_counter()
            bg, info = config3_background(pm, tab, s.ddz)     # FP64 set-up, the context's FP64 d/dz
            info["setup_s"] = time.perf_counter() - t0
            out["background"] = {"what": "magnetohydrostatic flux tube from an azimuthal vector potential, "
                                         "2 kG and 3 Mm at z = -8 Mm, widening over 8 Mm; box -25..0 Mm",
                                 **info}
        s.set_mhd_background(*bg)
        # an 8 mHz Ricker (peak at 150 s) so that the accuracy run's records hold the wave
        s.set_source_series(sources.gaussian_plane(pm, 1.0, 20.0, 0.0), sources.ricker_series(pm, 4000, f0=8.0e-3))
        s.record_surface(acc_steps // pm.steps + 2)
        s.step(warmup)
        s.sync()
        st = torch.cuda.ExternalStream(s.stream_ptr)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        s.step(steps)
        e1.record(st)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        bps = bytes_model.mhd_schedule_bytes_per_point_step(prec)
        gbs = bps * pm.points / (ms * 1e-3) / 1e9
        out[prec] = {"ms_per_step": ms, "value": pm.points / (ms * 1e-3) / 1e6, "unit": UNIT,
                     "alg_bytes_per_point_step": bps, "hbm_achieved_gbs": gbs,
                     "hbm_frac": gbs / _hbm_peak()}
        if acc_steps > warmup + steps:
            s.step(acc_steps - warmup - steps)
            s.sync(check_finite=True)
            res[prec] = (s.records(), s.state()[0])
        s.close()
    if "f64" in res and "f32" in res:
        (r64, a64), (r32, a32) = res["f64"], res["f32"]

        def rel(x, y):
            return float(np.linalg.norm((x - y).ravel()) / max(np.linalg.norm(y.ravel()), 1e-300))

        out["accuracy"] = {"steps": acc_steps, "records": int(r64.shape[0]),
                           "seismogram_rel_l2": rel(r32, r64),
                           "state_rel_l2": [rel(a32[f], a64[f]) for f in range(6)],
                           "what": "FP32 against FP64 on the same inputs: surface v_z records every output "
                                   "and the six fields after acc_steps steps"}
    return out


def _rel(x, y) -> float:
    return float(np.linalg.norm((np.asarray(x) - np.asarray(y)).ravel()) / max(np.linalg.norm(np.asarray(y).ravel()),
                                                                                1e-300))


def _tt_shifts(a, b, dt):
    """Travel-time shifts (COMPUTE_TT) of seismograms b against a, (nrec,
    nreceivers), on the receivers the wave has reached (rms >= 1 % of the
    strongest)."""
    from sparc_gb300.pipeline import compute_tt
    rms = np.sqrt(np.mean(a ** 2, axis=0))
    return [abs(compute_tt(a[:, r], b[:, r], dt)) for r in range(a.shape[1]) if rms[r] >= 1e-2 * rms.max()]


def full_length_config4(batch=8, segment=24, compare=2, hours=0.0):
    """The 32-source forward x adjoint kernel workflow at full length: 256^2 x
    300 quiet Sun, 4 h of solar time (the pipeline's forward run, adjoint run
    and forward recomputation from device checkpoints), FP32 fields with FP64
    accumulation, in batches of `batch` sources (the checkpoints and snapshot
    store of 32 sources at once would exceed HBM).  The first `compare`
    sources are run again through the FP64 pipeline one by one: their kernels
    and seismograms are stated against FP64."""
    from sparc_gb300 import sources
    from sparc_gb300.pipeline import KernelPipeline
    p0, tab = workload(False)
    if hours > 0:
        p0 = p0.replace(solartime=hours)
    S = 32
    series = sources.ricker_series(p0, p0.maxtime + 10)
    pix = sources.receiver_pixels(p0)
    planes = [source_inputs(p0, 64, gi, seed=4)[0] for gi in range(S)]
    ksum = None
    keep = {}
    t0 = time.perf_counter()
    batches = []
    for b0 in range(0, S, batch):
        tb = time.perf_counter()
        pl = KernelPipeline(p0.replace(precision="f32", nsrc=batch), tab, segment=segment)
        res = pl.run(planes[b0:b0 + batch], series, np.zeros((batch, pl.nt, p0.ny, p0.nx)), pix)
        k = np.stack([res.kc.sum(0), res.krho.sum(0), res.hessian.sum(0)])
        ksum = k if ksum is None else ksum + k
        for i in range(b0, min(b0 + batch, compare)):
            keep[i] = (res.kc[i - b0], res.krho[i - b0], res.hessian[i - b0], res.seismograms[i - b0])
        batches.append(time.perf_counter() - tb)
        log(f"config4: sources {b0}..{b0 + batch - 1} in {batches[-1]:.1f} s")
        del res, pl
    wall32 = time.perf_counter() - t0
    steps = p0.maxtime + 1
    out = {"workload": f"forward x adjoint kernel workflow, {p0.nx}x{p0.ny}x{p0.nz}, {S} sources, "
                       f"{p0.solartime} h ({steps} steps per run; forward, adjoint and recomputed forward)",
           "precision": "f32 fields, f64 set-up and accumulation", "batch": batch, "segment": segment,
           "wall_s": wall32, "batch_wall_s": batches,
           "point_steps": 3 * steps * p0.points * S,
           "Mpoint_steps_per_s": 3 * steps * p0.points * S / wall32 / 1e6,
           "kernel_sum_finite": bool(np.isfinite(ksum).all()), "kernel_sum_max_abs": float(np.abs(ksum).max())}
    cmp = []
    dt = p0.timestep * p0.steps
    for i in range(compare):
        tb = time.perf_counter()
        pl = KernelPipeline(p0.replace(precision="f64", nsrc=1), tab, segment=segment)
        r64 = pl.run([planes[i]], series, np.zeros((1, pl.nt, p0.ny, p0.nx)), pix)
        kc, kr, hs, seis = keep[i]
        sh = _tt_shifts(r64.seismograms[0], seis, dt)
        cmp.append({"source": i, "fp64_wall_s": time.perf_counter() - tb,
                    "seismogram_rel_l2": _rel(seis, r64.seismograms[0]),
                    "kernel_rel_l2": {"kc": _rel(kc, r64.kc[0]), "krho": _rel(kr, r64.krho[0]),
                                      "hessian": _rel(hs, r64.hessian[0])},
                    "max_tt_shift_s": float(max(sh)) if sh else None, "receivers_timed": len(sh)})
        del pl, r64
    out["fp32_against_fp64"] = cmp
    return out


def full_length_config3(hours_fp64=1.0, hours=4.0):
    """The flux-tube configuration at full length: option 10 on the
    magnetohydrostatic tube, 256^2 x 300, one source 20 Mm from the axis,
    4 h of solar time forward in FP32, and the first `hours_fp64` hours in FP64
    (130 ms per FP64 step makes the whole 4 h a 17-minute run); the FP32
    seismograms (8 receivers on a 10 Mm ring around the source) are stated
    against FP64 over that window."""
    import torch
    from sparc_gb300 import sources
    from sparc_gb300.background import config3_background
    from sparc_gb300.params import config_flux_tube_256
    from sparc_gb300.solver import Solver
    pm, tab = config_flux_tube_256()
    pm = pm.replace(nsrc=1, solartime=hours)
    hours_fp64 = min(hours_fp64, hours)
    pix = sources.receiver_pixels(pm, n=8, radius_mm=10.0, x0_mm=20.0)
    plane = sources.gaussian_plane(pm, 1.0, 20.0, 0.0)
    series = sources.ricker_series(pm, pm.maxtime + 10)
    out = {"grid": [pm.nx, pm.ny, pm.nz], "background": "magnetohydrostatic flux tube (config3_background)"}
    bg = None
    seis = {}
    for prec, hours in (("f32", pm.solartime), ("f64", hours_fp64)):
        p = pm.replace(precision=prec, solartime=hours)
        s = Solver(p, tab)
        if bg is None:
            bg, info = config3_background(p, tab, s.ddz)
            out["background_residual_l2_rel"] = info["residual_l2_rel"]
        s.set_mhd_background(*bg)
        s.set_source_series(plane, series)
        n = p.maxtime + 1
        s.record_surface(n // p.steps + 2)
        st = torch.cuda.ExternalStream(s.stream_ptr)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(st)
        s.step(n)
        e1.record(st)
        rec = s.records()
        wall = time.perf_counter() - t0
        ms = e0.elapsed_time(e1)
        s.sync(check_finite=True)
        seis[prec] = np.stack([rec[:, iy, ix] for (iy, ix) in pix], axis=1)
        out[prec] = {"hours": hours, "steps": n, "device_s": ms * 1e-3, "wall_s": wall,
                     "Mpoint_steps_per_s": p.points * n / (ms * 1e-3) / 1e6, "records": int(rec.shape[0])}
        s.close()
    k = seis["f64"].shape[0]
    sh = _tt_shifts(seis["f64"], seis["f32"][:k], pm.timestep * pm.steps)
    out["fp32_against_fp64"] = {"window_records": k, "seismogram_rel_l2": _rel(seis["f32"][:k], seis["f64"]),
                                "max_tt_shift_s": float(max(sh)) if sh else None, "receivers_timed": len(sh)}
    return out


def cpu_baseline(p, tab, steps=1):
    from oracle import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    o = oracle.Oracle(p.replace(precision="f64", nsrc=1), tab)
    from sparc_gb300 import sources
    o.set_source(1, sources.gaussian_plane(p)[None].copy(), sources.ricker_series(p, 100))
    o.step(1)                       # warm-up (first-touch of the arrays)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": p.points * steps / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} forward time step(s) of {p.nx}x{p.ny}x{p.nz} FP64 on the CPU oracle "
                      f"(one source), {dt:.1f} s"}


def _production_worker(bar, q, steps):
    """One single-threaded FP64 oracle solve of the 128x128x150 grid (run in a
    spawned process; the reference's production model is one solve per core)."""
    from oracle import oracle
    from sparc_gb300 import sources
    p, tab = workload(True)
    oracle.set_threads(1)
    o = oracle.Oracle(p.replace(precision="f64", nsrc=1), tab)
    o.set_source(1, sources.gaussian_plane(p)[None].copy(), sources.ricker_series(p, 100))
    o.step(1)                       # warm-up
    bar.wait(timeout=600)
    t0 = time.monotonic()
    o.step(steps)
    t1 = time.monotonic()
    o.close()
    q.put((t0, t1, p.points))


def cpu_production(n: int | None = None, steps: int = 1):
    """The reference's production model on the host: n concurrent
    single-threaded solves (one source each, one per core), started together;
    aggregate point-steps over the span from the first start to the last end."""
    import multiprocessing as mp
    n = n or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    bar, q = ctx.Barrier(n), ctx.Queue()
    procs = [ctx.Process(target=_production_worker, args=(bar, q, steps)) for _ in range(n)]
    for pr in procs:
        pr.start()
    res = [q.get(timeout=900) for _ in range(n)]
    for pr in procs:
        pr.join(timeout=60)
    span = max(r[1] for r in res) - min(r[0] for r in res)
    pts = sum(r[2] for r in res) * steps
    return {"value": pts / span / 1e6, "unit": UNIT, "cores": n, "kind": "port",
            "sample": f"{n} concurrent single-threaded FP64 oracle solves of 128x128x150 (one source each), "
                      f"{steps} timed step(s) each after one warm-up, {span:.1f} s span"}


def arm_config(p0, cad, S, nplanes, ws=1):
    """The workload both arms name (the reference arm times a bounded sample of it)."""
    return {"workload": f"quiet-Sun {p0.nx}x{p0.ny}x{p0.nz} forward+adjoint time step with "
                        f"sensitivity-kernel accumulation every {cad} steps, {S} sources batched per GPU",
            "grid": [p0.nx, p0.ny, p0.nz], "nsrc": S, "point_steps_per_step": 2 * p0.points * S,
            "sources_global": S * ws, "sharding": "sources round-robin over the ranks; kernels summed by one "
                                                  "FP64 all-reduce in device memory",
            "l2": "inputs larger than L2 (state of each context > 30 GB)",
            "adjoint_source_samples": nplanes}


def run_reference(args):
    """The reference arm: the CPU oracle (the reference's algorithm restated in
    C++ FP64; the Fortran/MPI/FFTW reference cannot be built here) on the
    arm's workload, with every host thread.  A bench step of that workload is
    a forward and an adjoint time step of every source plus, every cad steps,
    one kernel accumulation per source.  The sample times K forward steps of
    one source and one kernel accumulation; the bench step's time is
    extrapolated from them (an adjoint step costs what a forward step does,
    and the sources are independent), and value = point-steps of a bench step
    / that time."""
    ws, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return 0
    p, tab = workload(args.small)
    from oracle import oracle
    from sparc_gb300 import sources
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    K = max(1, min(args.steps, 3))
    W = max(0, min(args.warmup, 1))
    S = args.nsrc
    pp = p.replace(precision="f64", nsrc=1)
    o = oracle.Oracle(pp, tab)
    o.set_source(1, sources.gaussian_plane(p)[None].copy(), sources.ricker_series(p, 100))
    o.step(W)
    t0 = time.perf_counter()
    o.step(K)
    t_step = (time.perf_counter() - t0) / K
    # one kernel accumulation (kernels.f90:276-311) on the oracle's state
    a, scr, _ = o.state()
    fsnap = np.concatenate([a[0:3], scr[3:6]])
    asnap = np.ascontiguousarray(a[3:6])
    graw = tab[:, 4] * o.info()["rsun"] / 1e12
    o.kernel_reset()
    t0 = time.perf_counter()
    o.kernel_accumulate(fsnap, asnap, graw)
    t_acc = time.perf_counter() - t0
    o.close()
    cad = p.steps
    t_bench = 2 * S * t_step + S * t_acc / cad
    pts = 2 * p.points * S
    v = pts / t_bench / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1 if ws <= 1 else ws,
        "steps": K, "warmup": W, "ms_per_step": t_bench * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": arm_config(p, cad, S, args.nplanes),
        "ms_per_step_what": (f"one bench step of the workload ({2 * S} source time steps and {S}/{cad} kernel "
                             "accumulations), extrapolated from the sample"),
        "sample": {"forward_step_ms": t_step * 1e3, "kernel_accumulation_ms": t_acc * 1e3,
                   "point_steps_per_forward_step": p.points},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{K} forward steps of one source of {p.nx}x{p.ny}x{p.nz} (FP64) after "
                                   f"{W} warm-up and one kernel accumulation, on {threads} threads, "
                                   f"extrapolated to a bench step ({2 * S} source steps, {S}/{cad} "
                                   "accumulations); the reference Fortran/MPI/FFTW cannot be built here, so "
                                   "the CPU oracle (its line-for-line FP64 restatement) stands in"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    try:
        line["cpu_baseline"]["production"] = cpu_production()
    except Exception as e:
        line["cpu_baseline"]["production"] = {"value": None, "sample": f"failed: {e}"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    ws, rank, local = dist_init()
    import torch
    torch.cuda.set_device(local)
    from sparc_gb300 import build as b
    b.build()
    from sparc_gb300 import bytes_model
    from sparc_gb300 import dist as sd
    p0, tab = workload(args.small)
    if args.full_length:
        h = args.fl_hours
        fn = {"config4": lambda: full_length_config4(hours=h),
              "config3": lambda: full_length_config3(hours=h) if h > 0 else full_length_config3(),
              "serving": lambda: serving_section("f32", args.serve_requests,
                                                 min(args.serve_compress, 4.0) if h <= 0 else args.serve_compress,
                                                 max_wall=1800.0)}[args.full_length]
        print(json.dumps({"full_length": args.full_length, "result": fn()}), flush=True)
        return 0
    if args.mhd_only:
        grid = tuple(int(v) for v in args.mhd_grid.lower().split("x")) if args.mhd_grid else None
        print(json.dumps({"mhd": mhd_section(steps=max(1, args.steps), warmup=max(1, args.warmup),
                                             precs=tuple(args.mhd_prec.split(",")), grid=grid, acc_steps=0)}),
              flush=True)
        return 0
    K, W = max(1, args.steps), max(3, args.warmup)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    N = p0.points
    out = {}

    # ---- plain FP64, one source ----
    log("plain FP64")
    if not args.skip_fp64:
        p64 = p0.replace(precision="f64", nsrc=1)
        fwd, adj = make_pair(p64, tab, args.nplanes, sd.shard_sources(ws, rank, ws), seed=1)
        cad = fwd.info()["steps"]
        tuning64 = {"forward": fwd.autotune(1), "adjoint": adj.autotune(1)}
        run_steps(fwd, adj, W, cad)
        barrier(ws)
        ms, _ = timed_region(fwd, adj, K, cad)
        ms = allmax(ws, ms)
        b64 = bytes_model.reference_schedule_bytes_per_point_step("f64")
        out["fp64_plain"] = {"value": 2 * N * K * ws / (ms * 1e-3) / 1e6, "unit": UNIT,
                             "ms_per_step": ms / K, "nsrc": 1, "dtype": "f64", "tuning": tuning64,
                             "hbm_achieved_gbs": b64 * 2 * N / (ms / K * 1e-3) / 1e9,
                             "hbm_frac": b64 * 2 * N / (ms / K * 1e-3) / 1e9 / hbm_peak}
        fwd.close(); adj.close()
        del fwd, adj

    # ---- batched FP32 ----
    log("batched FP32")
    # the global source list (nsrc per rank) split round-robin over the ranks
    S = args.nsrc
    mine = sd.shard_sources(S * ws, rank, ws)
    p32 = p0.replace(precision="f32", nsrc=S)
    fwd, adj = make_pair(p32, tab, args.nplanes, mine, seed=2)
    cad = fwd.info()["steps"]
    # launch variants with identical results, picked by timing real steps
    # (part of the warm-up: 4 steps per context)
    tuning = {"forward": fwd.autotune(1), "adjoint": adj.autotune(1)}
    run_steps(fwd, adj, W, cad)
    barrier(ws)
    with ClockSampler(local) as clk:
        ms, launches = timed_region(fwd, adj, K, cad)
        # dominant kernel: the fused FP32 step, timed on its own stream
        st_ms = step_kernel_time(fwd)
    ms = allmax(ws, ms)
    value = 2 * N * S * K * ws / (ms * 1e-3) / 1e6
    # roofline of the dominant kernel (the fused FP32 step): its own
    # compulsory bytes per launch (12 field accesses, the PML planes and the
    # source plane of every source) over its average launch time
    own = bytes_model.fused_step_alg_bytes(p32)
    achieved = own / (st_ms * 1e-3) / 1e9
    traffic = bytes_model.fused_traffic_per_launch(p32)
    winst = bytes_model.fused_warp_inst_per_launch(p32)
    # the per-stage schedule's credit (653.3 B per grid-point-step), kept
    # apart: it counts bytes this kernel does not move
    bpps = bytes_model.reference_schedule_bytes_per_point_step("f32")
    clocks = clk.summary()
    # per-step latency distribution of the batched solve
    import torch
    lat = []
    for _ in range(min(K, 10)):
        t0 = time.perf_counter()
        run_steps(fwd, adj, 1, cad)
        fwd.sync(); adj.sync()
        lat.append((time.perf_counter() - t0) * 1e3)
    fwd.close(); adj.close()
    del fwd, adj

    # ---- e2e through the public API with host buffers (pinned) ----
    log("e2e")
    e2e = None
    if True:
        from sparc_gb300 import sources
        from sparc_gb300.solver import Solver
        pa = p32.replace(compute_forward=False, compute_adjoint=True)
        series = sources.ricker_series(p32, 20000)

        def pinned(shape):
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

        plane_h = [pinned((p32.ny, p32.nx)) for _ in range(S)]
        adj_h = [pinned((args.nplanes, p32.ny, p32.nx)) for _ in range(S)]
        for s, gi in enumerate(mine):
            plane_h[s][...], adj_h[s][...] = source_inputs(p32, args.nplanes, gi, seed=3)
        fwd, adj = Solver(p32, tab), Solver(pa, tab)
        ksum = torch.empty((3, p32.nz, p32.ny, p32.nx), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        Ke = max(K, cad)                      # at least one kernel accumulation (every cad steps)
        nrec = Ke // cad + 2
        rec_h = pinned((nrec, p32.ny, p32.nx))
        k_h = [pinned((p32.nz, p32.ny, p32.nx)) for _ in range(3)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in range(S):
            fwd.set_source_series(plane_h[s], series, slot=s)
            adj.set_source_lagrange(adj_h[s], slot=s)
        fwd.record_surface(nrec)
        run_steps(fwd, adj, Ke, cad)
        d2h = 0
        for s in range(S):
            r = fwd.records(slot=s)
            rec_h[: r.shape[0]] = r
            d2h += r.nbytes
        # kernels summed over this rank's sources into device memory, then
        # over all ranks by one FP64 all-reduce (grad.py:158-165), then one
        # device-to-host copy
        adj.kernels_into(ksum.data_ptr(), sum_slots=True)
        adj.sync()
        sd.reduce_kernels(ksum)
        kd = ksum.cpu().numpy()
        for i in range(3):
            k_h[i][...] = kd[i]
        d2h += kd.nbytes
        dt = time.perf_counter() - t0
        h2d = S * (plane_h[0].nbytes + series.nbytes + adj_h[0].nbytes)
        e2e = {"value": 2 * N * S * Ke * ws / dt / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d // Ke), "d2h_bytes_per_step": int(d2h // Ke),
               "wall_s": dt, "steps": Ke}
        fwd.close(); adj.close()

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 set-up and kernel accumulation)", "data": "synthetic",
        "config": arm_config(p0, cad, S, args.nplanes, ws),
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "kernel": "fused_step_kernel (FP32, one launch per time step of all sources)",
                     "avg_launch_ms": st_ms, "alg_bytes_per_launch": own,
                     "alg_bytes_per_point_step": own / (N * S),
                     "alg_what": "compulsory bytes of the fused step: read and write a (12 spectral field "
                                 "accesses), the two PML auxiliaries on their planes (read and write), one "
                                 "source plane, per source",
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of a "
                                       "single-source launch at this grid, times nsrc (a scaled constant, not "
                                       "measured in this run)" if traffic else None,
                     "issue": issue_roofline(winst, st_ms, clocks, sm_count),
                     "schedule_credit": {
                         "bytes_per_point_step": bpps, "bytes_per_launch": bpps * N * S,
                         "achieved_gbs": bpps * N * S / (st_ms * 1e-3) / 1e9,
                         "frac": bpps * N * S / (st_ms * 1e-3) / 1e9 / hbm_peak,
                         "what": "the compulsory bytes of the minimal per-stage schedule of the reference's "
                                 "physical-space formulation (163.3 field accesses per point-step), credited "
                                 "to each point-step whatever the kernel moves; above 1 it says the fused "
                                 "step does a step's work faster than that schedule could move its bytes"},
                     "peak_source": f"{peak_src} hbm_gbs"},
        "step_latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                            "what": "one batched forward+adjoint step, host-synchronised"},
        "e2e": e2e,
    }
    line["tuning"] = tuning
    if ws == 1:
        log("small-grid step latency")
        line["small_grid_step"] = small_step_latency()
        if not args.skip_fp64:
            log("1-h configuration, full length")
            try:
                line["config1_full"] = config1_full()
            except Exception as e:   # reported, not fatal
                line["config1_full"] = {"error": str(e)}
    if ws == 1 and not args.skip_fp64:
        log("FP32 against FP64")
        try:
            line["accuracy"] = accuracy_section()
        except Exception as e:   # reported, not fatal
            line["accuracy"] = {"error": str(e)}
    if ws == 1 and not args.skip_mhd:
        log("MHD flux tube")
        try:
            line["mhd"] = mhd_section(grid=(p0.nx, p0.ny, p0.nz) if args.small else None)
        except Exception as e:   # reported, not fatal
            line["mhd"] = {"error": str(e)}
    if args.serve_requests > 0 and ws == 1:
        line["serving"] = {}
        for prec in ("f32", "f64"):
            log(f"serving stream {prec}")
            try:
                line["serving"][prec] = serving_section(prec, args.serve_requests, args.serve_compress)
            except Exception as e:   # reported, not fatal: the timed headline above is complete
                line["serving"][prec] = {"error": str(e)}
        line["serving"]["what"] = ("Poisson stream, 4 requests/s, 60/30/10 % of 128^2x150/256^2x300/512^2x300, "
                                   "half forward+adjoint, 1-4 h of solar time compressed by serve-compress; "
                                   "continuous batching with per-slot clocks")
    if "fp64_plain" in out:
        line["fp64_plain"] = out["fp64_plain"]
        line["ratio_fp32_batched_over_fp64_plain"] = value / out["fp64_plain"]["value"]
    if rank == 0 and ws == 1 and not args.skip_cpu:
        log("cpu baseline")
        try:
            line["cpu_baseline"] = cpu_baseline(p0, tab)
        except Exception as e:  # the oracle is only the reported baseline
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"failed: {e}"}
        try:
            line["cpu_baseline"]["production"] = cpu_production()
        except Exception as e:
            line["cpu_baseline"]["production"] = {"value": None, "sample": f"failed: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
